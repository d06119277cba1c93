// kv_unet_kernels.cuh -- kernels of the 3D U-Net warm start (BF16 storage,
// FP32 accumulation), channels-last layout [D][H][W][C].
//
// The 3x3x3 convolutions are implicit GEMMs on the tensor cores
// (mma.sync m16n8k16, BF16 x BF16 -> FP32):
//   forward / backward-data: M = voxels, N = output channels, K = 27 x input
//     channels; a warp owns 16 consecutive voxels of one row and all of its
//     output channels (up to 64), the A fragments come straight from the
//     channels-last activations (32-bit loads of channel pairs), the B
//     fragments from the [Cout][27][Cin] weights.  Backward-data is the
//     forward convolution of the output gradient with the flipped, transposed
//     weights.
//   backward-weight: per tap, M = Cout, N = Cin, K = voxels; a warp stages 16
//     voxels of the output gradient and of the shifted input in shared memory
//     and forms both (transposed) operands with ldmatrix.trans; each CTA adds
//     its partial sums for one voxel chunk into the FP32 gradient.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace unet {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t ld32(const bf16 *p) {
    return __ldg(reinterpret_cast<const unsigned int *>(p));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3,
                                                  const void *smem_row) {
    const unsigned addr = static_cast<unsigned>(__cvta_generic_to_shared(smem_row));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

// 3x3x3 convolution, zero padding, optional concatenated second input
// (channels [0,c1) from in1, [c1,c1+c2) from in2), output channels
// [n_off, n_off + 8*NT) of a tensor with c_out_total channels.
// Requires W % 16 == 0, c1 % 16 == 0, c2 % 16 == 0.
template <int NT, bool RELU>
__global__ void __launch_bounds__(128) conv3_fwd(const bf16 *__restrict__ in1, int c1,
                                                 const bf16 *__restrict__ in2, int c2,
                                                 const bf16 *__restrict__ w, const float *__restrict__ bias,
                                                 bf16 *__restrict__ out, int c_out_total, int n_off, int D,
                                                 int H, int W) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long m0 = ((long long)blockIdx.x * 4 + warp) * 16;
    const long long nvox = (long long)D * H * W;
    if (m0 >= nvox) return;
    const int x0 = (int)(m0 % W);
    const long long zy = m0 / W;
    const int y = (int)(zy % H), z = (int)(zy / H);
    const int g = lane >> 2, t = lane & 3;
    const int cin = c1 + c2;
    float acc[NT][4];
#pragma unroll
    for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
    for (int tap = 0; tap < 27; ++tap) {
        const int zz = z + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const bool zy_in = (unsigned)zz < (unsigned)D && (unsigned)yy < (unsigned)H;
        const int xa = x0 + g + dx, xb = xa + 8;
        const bool ina = zy_in && (unsigned)xa < (unsigned)W;
        const bool inb = zy_in && (unsigned)xb < (unsigned)W;
        const long long va = ((long long)zz * H + yy) * W + xa;
        for (int cc = 0; cc < cin; cc += 16) {
            const bf16 *src = cc < c1 ? in1 : in2;
            const int cs = cc < c1 ? c1 : c2;
            const int co = (cc < c1 ? cc : cc - c1) + 2 * t;
            const uint32_t a0 = ina ? ld32(src + va * cs + co) : 0u;
            const uint32_t a1 = inb ? ld32(src + (va + 8) * cs + co) : 0u;
            const uint32_t a2 = ina ? ld32(src + va * cs + co + 8) : 0u;
            const uint32_t a3 = inb ? ld32(src + (va + 8) * cs + co + 8) : 0u;
            const bf16 *wk = w + (size_t)tap * cin + cc + 2 * t;
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const bf16 *wr = wk + (size_t)(n_off + n * 8 + g) * 27 * cin;
                mma_bf16(acc[n], a0, a1, a2, a3, ld32(wr), ld32(wr + 8));
            }
        }
    }
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const int oc = n_off + n * 8 + 2 * t;
        const float b0 = bias ? bias[oc] : 0.f, b1 = bias ? bias[oc + 1] : 0.f;
        float v0 = acc[n][0] + b0, v1 = acc[n][1] + b1, v2 = acc[n][2] + b0, v3 = acc[n][3] + b1;
        if (RELU) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
            v2 = fmaxf(v2, 0.f);
            v3 = fmaxf(v3, 0.f);
        }
        *reinterpret_cast<__nv_bfloat162 *>(out + (m0 + g) * c_out_total + oc) = __floats2bfloat162_rn(v0, v1);
        *reinterpret_cast<__nv_bfloat162 *>(out + (m0 + g + 8) * c_out_total + oc) = __floats2bfloat162_rn(v2, v3);
    }
}

// Weight gradient of a 3x3x3 convolution for one tap (blockIdx.y), one tile
// of 16 output channels (blockIdx.z / ci groups) and one chunk of voxels
// (blockIdx.x): dW[co][tap][ci] += sum_v dY[v][co] * X[v + tap][ci].
// 4 warps split the chunk; partial sums meet in shared memory and one atomic
// add per weight per CTA goes to global memory.  NTW n-tiles of 8 input
// channels per warp (ci group = 8*NTW channels).
template <int NTW>
__global__ void __launch_bounds__(128) conv3_wgrad(const bf16 *__restrict__ dy, int cout,
                                                   const bf16 *__restrict__ in1, int c1,
                                                   const bf16 *__restrict__ in2, int c2,
                                                   float *__restrict__ dw, int D, int H, int W, int chunk) {
    __shared__ __align__(16) bf16 sA[4][16][16];          // [warp][voxel][co]
    __shared__ __align__(16) bf16 sB[4][16][8 * NTW];     // [warp][voxel][ci]
    __shared__ float red[4][16][8 * NTW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tap = blockIdx.y;
    const int n_ci_groups = (c1 + c2) / (8 * NTW);
    const int co0 = (blockIdx.z / n_ci_groups) * 16;
    const int ci0 = (blockIdx.z % n_ci_groups) * 8 * NTW;
    const int cin = c1 + c2;
    const int dz = tap / 9 - 1, dy_ = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const long long nvox = (long long)D * H * W;
    const long long v_begin = (long long)blockIdx.x * chunk;
    const long long v_end = v_begin + chunk < nvox ? v_begin + chunk : nvox;
    float acc[NTW][4];
#pragma unroll
    for (int n = 0; n < NTW; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
    // each warp takes every 4th group of 16 voxels of the chunk
    for (long long v0 = v_begin + warp * 16; v0 < v_end; v0 += 64) {
        // stage dY[v0..v0+15][co0..co0+15]: lane -> voxel lane/2, 8 channels
        {
            const int vv = lane >> 1, half = lane & 1;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (v0 + vv < v_end) val = __ldg(reinterpret_cast<const uint4 *>(dy + (v0 + vv) * cout + co0 + half * 8));
            *reinterpret_cast<uint4 *>(&sA[warp][vv][half * 8]) = val;
        }
        // stage X[v0+tap..][ci0..ci0+8*NTW) (zero outside the volume)
        {
            const int x0 = (int)(v0 % W);
            const long long zy = v0 / W;
            const int y = (int)(zy % H), z = (int)(zy / H);
            const int zz = z + dz, yy = y + dy_;
            const bool zy_in = (unsigned)zz < (unsigned)D && (unsigned)yy < (unsigned)H;
            constexpr int VEC = NTW;   // 16-byte vectors per voxel row of the group
            for (int e = lane; e < 16 * VEC; e += 32) {
                const int vv = e / VEC, q = e % VEC;
                const int xx = x0 + vv + dx;
                uint4 val = make_uint4(0, 0, 0, 0);
                if (zy_in && (unsigned)xx < (unsigned)W && v0 + vv < v_end) {
                    const long long src_v = ((long long)zz * H + yy) * W + xx;
                    const int ci = ci0 + q * 8;
                    const bf16 *p = ci < c1 ? in1 + src_v * c1 + ci : in2 + src_v * c2 + (ci - c1);
                    val = __ldg(reinterpret_cast<const uint4 *>(p));
                }
                *reinterpret_cast<uint4 *>(&sB[warp][vv][q * 8]) = val;
            }
        }
        __syncwarp();
        // A (16 co x 16 voxels) = dY^T, B (16 voxels x 8 ci) = X: both transposed loads
        uint32_t a0, a1, a2, a3;
        {
            const int r = lane & 7, m = lane >> 3;   // matrix m: (voxel half, co half)
            const int vrow = r + ((m >> 1) << 3), col = (m & 1) << 3;
            ldmatrix_x4_trans(a0, a1, a2, a3, &sA[warp][vrow][col]);
        }
#pragma unroll
        for (int n = 0; n < NTW; n += 2) {
            uint32_t b0, b1, b2, b3;
            const int r = lane & 7, m = lane >> 3;   // (voxel half, ci tile)
            const int vrow = r + ((m & 1) << 3), col = (n + (m >> 1)) * 8;
            ldmatrix_x4_trans(b0, b1, b2, b3, &sB[warp][vrow][col]);
            mma_bf16(acc[n], a0, a1, a2, a3, b0, b1);
            if (n + 1 < NTW) mma_bf16(acc[n + 1], a0, a1, a2, a3, b2, b3);
        }
        __syncwarp();
    }
    // reduce the 4 warps and add to the gradient
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int n = 0; n < NTW; ++n) {
        red[warp][g][n * 8 + 2 * t] = acc[n][0];
        red[warp][g][n * 8 + 2 * t + 1] = acc[n][1];
        red[warp][g + 8][n * 8 + 2 * t] = acc[n][2];
        red[warp][g + 8][n * 8 + 2 * t + 1] = acc[n][3];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 16 * 8 * NTW; e += blockDim.x) {
        const int r = e / (8 * NTW), c = e % (8 * NTW);
        const float s = red[0][r][c] + red[1][r][c] + red[2][r][c] + red[3][r][c];
        atomicAdd(dw + ((size_t)(co0 + r) * 27 + tap) * cin + ci0 + c, s);
    }
}

}  // namespace unet
