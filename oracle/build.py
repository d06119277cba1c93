"""Builds the CPU oracle (TEST INFRASTRUCTURE).

liboracle.so   kvtomo_oracle.c, gcc -O2 -fopenmp -ffp-contract=off (no fused
               multiply-add, so the RC restatement is bit-identical to the
               reference kernels compiled for the host).
_ref/libkvref.so  the reference's own kernels, compiled from the reference
               tree by build_ref.sh when that tree is present (with the
               GPU cubins _ref/ref_kernels*.cubin, see ref_gpu.py).
_ref/ref_geometry  the reference's XML geometry reader (its geometry module
               and tinyxml2) behind ref_geometry_driver.cpp, the same way.
_ref/ref_histogram  the reference's histogram tools behind
               ref_histogram_driver.cpp, against ref_vtk_stub/.
_ref/ref_drivers  the reference's ART / MLEM drivers (Reconstructors.h) on
               the host build of its kernels, behind ref_drivers_main.cpp.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libkvref.so")
REF_GEOMETRY = os.path.join(HERE, "_ref", "ref_geometry")
REF_HISTOGRAM = os.path.join(HERE, "_ref", "ref_histogram")
REF_DRIVERS = os.path.join(HERE, "_ref", "ref_drivers")
# The reference tree: $KVTOMO_REFERENCE_ROOT, else a directory named
# "reference" beside the one that holds this repository.
REFERENCE_ROOT = (os.environ.get("KVTOMO_REFERENCE_ROOT")
                  or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build_oracle(force=False):
    src = os.path.join(HERE, "kvtomo_oracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           src, "-o", ORACLE_SO, "-lm"]
    subprocess.run(cmd, check=True)
    return ORACLE_SO


def build_ref(force=False):
    """Compiles the reference kernels when the reference tree is present."""
    if not os.path.isdir(REFERENCE_ROOT):
        return None
    cubins = [os.path.join(HERE, "_ref", f) for f in ("ref_kernels.cubin", "ref_kernels_nofma.cubin")]
    if (not force and all(os.path.exists(f) for f in (REF_SO, REF_GEOMETRY, REF_HISTOGRAM, REF_DRIVERS, *cubins))):
        return REF_SO
    subprocess.run([os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT], check=True)
    return REF_SO if os.path.exists(REF_SO) else None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
