/*
 * ref_gpu_wrap.cu -- compiles the reference's own projector kernels for the
 * GB300 (TEST INFRASTRUCTURE: a checker and the "reference GPU" timing line;
 * never part of the product path).
 *
 * build_ref.sh extracts lines 22-785 of the reference's
 * source/modules/reconstruction/Projector.cu (floatEq / floatSupEq /
 * floatInfEq, FindProjectionAlphas_d, CudaPerformProjection at :227 and
 * CudaPerformBackProjection at :376; no host code) into
 * oracle/_ref/ref_kernels_gpu.inc, compiles this file to a cubin with nvcc
 * and deletes the extracted lines again.  The kernels get C linkage here so
 * the loader (oracle/ref_gpu.py) finds them by their plain names; their
 * parameter lists are the reference's.
 */
#define __forceinline __forceinline__

extern "C" {
#include "ref_kernels_gpu.inc"
}
