"""CPU oracle for the kvtomo engine -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and reference
legs may import this package.  The engine (kevernals_gb300) never does.
"""
