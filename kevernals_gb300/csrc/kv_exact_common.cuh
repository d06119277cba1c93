// kv_exact_common.cuh -- the arithmetic shared by every EXACT-family kernel:
// sizes, the slice-local plane-crossing parameter and the per-ray slice
// length.  Every kernel that evaluates a Siddon weight uses these same
// expressions, which is what keeps the backprojector the exact transpose of
// the forward projector.
#pragma once

#include <cuda_runtime.h>

namespace {

struct ExGeom {
    int nx, ny, nz, nu, nv, n_views;
};

// Slice-local parameter t at which a ray whose position (relative to its
// table base, in voxels) is `ft` on the slice's top plane reaches the plane
// `rel_plane`; `ix` = -1 / (slope * dh).
__device__ __forceinline__ float cross_t(int rel_plane, float ft, float ix) {
    return __fmul_rn(__fsub_rn((float)rel_plane, ft), ix);
}

// The same with the plane given as an exactly representable float.
__device__ __forceinline__ float cross_tf(float rel_plane, float ft, float ix) {
    return __fmul_rn(__fsub_rn(rel_plane, ft), ix);
}

// Ls = sqrt(ax^2 + ay^2 + H^2) * dz / H : length of the ray inside one slice.
__device__ __forceinline__ float ray_factor(float ax, float ay, float4 vi) {
    return __fmul_rn(__fsqrt_rn(__fadd_rn(__fmaf_rn(ax, ax, __fmul_rn(ay, ay)), vi.x)), vi.y);
}

}  // namespace
