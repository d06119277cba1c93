// kv_conv_tc.cuh -- 3x3x3 convolution as an implicit GEMM on the Blackwell
// tensor cores: TMA tile loads into swizzled shared memory, tcgen05.mma with
// the accumulator in tensor memory (TMEM), tcgen05.ld epilogue.
//
// GEMM view (channels-last activations [D][H][W][C], BF16):
//   D[m][n] = sum over taps t and input channels k of A_t[m][k] * B_t[n][k]
//   m: a CTA tile of 128*T voxels (T = 1, 2 or 4 sub-tiles of 128, one MMA
//      each, all sharing the stage's weight slice), BW x BH x BD (x, y, z)
//      with BW = min(W, 128), BH = min(H, 128*T / BW), BD = the rest;
//      n: output channels (N = 16..256),
//   k: input channels of the (possibly concatenated) input, in segments of
//      16 / 32 / 64 channels (one TMA box each; 128-channel inputs are two
//      segments).
// A_t is the input shifted by tap t = (dz,dy,dx): the TMA box starts at
// (x0+dx, y0+dy, z0+dz); coordinates outside the volume read zeros, which is
// the convolution's zero padding.  B_t is the weight slice w[n][t][k]
// ([Cout][27][Cin] layout, K contiguous), also one TMA box per segment.
// Both operands are K-major with the swizzle matching the segment's row
// width (32 / 64 / 128 bytes); one tcgen05.mma (M=128, N, K=16, BF16 in,
// FP32 accumulate) per 16 channels.
//
// Warp roles (192 threads): warp 0 issues the TMA loads into a ring of
// stages (one tap of every segment per stage), warp 1 owns the TMEM
// allocation and issues the MMAs (one elected thread), warps 2-5 drain the
// accumulator (each warp reads its 32 TMEM lanes = 32 voxels), add the bias,
// apply ReLU, convert to BF16 and store.  The CTA is persistent over tiles.
// Every wait on an mbarrier is bounded: on timeout the thread records an
// error code, raises the CTA's abort flag and every role winds down, so a
// fault in the pipeline ends the kernel with a status instead of a hang.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <cstdio>

#include "kv_tma.cuh"

namespace convtc {

constexpr int kThreads = 192;
constexpr int kMaxSeg = 4;        // input channel segments (e.g. 64 + 64 + 64 for 192 channels)
constexpr int kTileM = 128;
constexpr uint32_t kWaitLimit = 1u << 22;   // try_wait rounds before a wait is declared failed

struct SegInfo {
    int n;                        // number of segments
    int kseg[kMaxSeg];            // channels in each segment (16, 32 or 64)
    int src[kMaxSeg];             // which activation map (0 or 1)
    int c0[kMaxSeg];              // first channel of the segment within its activation tensor
    int kglob[kMaxSeg];           // first channel of the segment within the concatenated input
    uint32_t a_off[kMaxSeg];      // byte offset of the segment's A tile within a stage
    uint32_t b_off[kMaxSeg];      // byte offset of the segment's B tile within a stage
};

struct Params {
    SegInfo seg;
    int N;                        // output channels
    int D, H, W;                  // this level's volume
    int BW, BH, BD;               // tile extent in x, y and z (BW * BH * BD = 128 * T)
    int T;                        // 128-voxel sub-tiles (MMAs) per tile
    long long tiles;
    uint32_t stage_bytes, stages, tmem_cols;
    uint32_t tx_bytes;            // bytes the TMA loads of one stage deliver
    uint32_t idesc;               // tcgen05 instruction descriptor
    const float *bias;            // nullptr: none
    int relu;
    __nv_bfloat16 *out;           // [voxels][N]
    int *status;                  // 0 ok; set on a failed wait
};

using kvtma::mbar_arrive;
using kvtma::mbar_arrive_expect_tx;
using kvtma::mbar_init;
using kvtma::mbar_try_wait;
using kvtma::smem_u32;
using kvtma::tma_load_3d;
using kvtma::tma_load_4d;

// Bounded wait for the phase of `bar` with parity `parity` to complete.
// Returns false (after recording `code`) on timeout or when another role
// has already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort, int *status,
                                          int code) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
        if (i >= 16) __nanosleep(128);
    }
    atomicCAS(status, 0, code);
    *abort = 1;
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand tile whose rows are
// `row_bytes` (32 / 64 / 128) long, stored with the matching swizzle by TMA:
// start address >> 4 (bits 0-13), leading byte offset (unused for swizzled
// K-major tiles, 16 bytes) >> 4 (16-29), stride byte offset = 8 rows >> 4
// (32-45), descriptor version 1 (46-47), swizzle mode (61-63:
// 6 = 32 B, 4 = 64 B, 2 = 128 B).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t row_bytes) {
    const uint64_t layout = row_bytes == 128 ? 2ull : (row_bytes == 64 ? 4ull : 6ull);
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(((8u * row_bytes) >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    d |= layout << 61;
    return d;
}

__global__ void __launch_bounds__(kThreads, 1)
    conv3_tc_kernel(const __grid_constant__ CUtensorMap map_a0, const __grid_constant__ CUtensorMap map_a1,
                    const __grid_constant__ CUtensorMap map_b, const __grid_constant__ Params P) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[8], empty_bar[8], acc_full, acc_empty, drain_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_flag;
    __shared__ unsigned long long issued_sh, consumed_sh;   // stages loaded by TMA / consumed by MMA
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // stage ring, 1024-byte aligned (the 128-byte swizzle repeats every 8 rows)
    const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (uint32_t s = 0; s < P.stages; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_full, 1);
        mbar_init(&acc_empty, 4);
        mbar_init(&drain_bar, 1);
        issued_sh = 0;
        consumed_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base_sh)),
                     "r"(P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const int tiles_x = P.W / P.BW, tiles_y = P.H / P.BH;   // tiles_z = D / BD

    if (warp == 0) {
        // ---------------------------------------------------------- TMA producer
        if (lane == 0) {
            uint32_t stage = 0, phase = 0;
            for (long long tile = blockIdx.x; tile < P.tiles && !abort_flag; tile += gridDim.x) {
                const int tx = (int)(tile % tiles_x);
                const long long r = tile / tiles_x;
                const int ty = (int)(r % tiles_y), tz = (int)(r / tiles_y);
                const int x0 = tx * P.BW, y0 = ty * P.BH, z0 = tz * P.BD;
                for (int tap = 0; tap < 27; ++tap) {
                    if (!mbar_wait(&empty_bar[stage], phase ^ 1u, &abort_flag, P.status, 1)) break;
                    mbar_arrive_expect_tx(&full_bar[stage], P.tx_bytes);
                    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
                    const uint32_t sb = base + stage * P.stage_bytes;
                    for (int s = 0; s < P.seg.n; ++s) {
                        const CUtensorMap *ma = P.seg.src[s] == 0 ? &map_a0 : &map_a1;
                        tma_load_4d(sb + P.seg.a_off[s], ma, &full_bar[stage], P.seg.c0[s], x0 + dx, y0 + dy,
                                    z0 + dz);
                        tma_load_3d(sb + P.seg.b_off[s], &map_b, &full_bar[stage], P.seg.kglob[s], tap, 0);
                    }
                    ++issued_sh;
                    if (++stage == P.stages) { stage = 0; phase ^= 1u; }
                }
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            // descriptors of stage 0; a later stage, K step or sub-tile only adds
            // its byte offset >> 4 to the start-address field (shared-memory
            // addresses stay below 2^18, so the 14-bit field never carries)
            uint64_t desc_a[kMaxSeg], desc_b[kMaxSeg];
#pragma unroll
            for (int s = 0; s < kMaxSeg; ++s) {
                desc_a[s] = smem_desc(base + P.seg.a_off[s], (uint32_t)P.seg.kseg[s] * 2u);
                desc_b[s] = smem_desc(base + P.seg.b_off[s], (uint32_t)P.seg.kseg[s] * 2u);
            }
            uint32_t stage = 0, phase = 0, acc_phase = 0;
            for (long long tile = blockIdx.x; tile < P.tiles && !abort_flag; tile += gridDim.x) {
                if (!mbar_wait(&acc_empty, acc_phase ^ 1u, &abort_flag, P.status, 2)) break;
                acc_phase ^= 1u;
                tc_fence_after();
                bool ok = true;
                for (int tap = 0; tap < 27 && ok; ++tap) {
                    if (!mbar_wait(&full_bar[stage], phase, &abort_flag, P.status, 3)) { ok = false; break; }
                    tc_fence_after();
                    const uint64_t so = (uint64_t)((stage * P.stage_bytes) >> 4);
#pragma unroll
                    for (int s = 0; s < kMaxSeg; ++s) {
                        if (s >= P.seg.n) break;
                        const uint64_t sub = (uint64_t)((kTileM * P.seg.kseg[s] * 2) >> 4);   // one sub-tile
                        for (int k = 0; k < P.seg.kseg[s]; k += 16) {
                            const uint64_t ko = (uint64_t)((k * 2) >> 4);                   // 32 B per K step
                            const uint64_t bd = desc_b[s] + so + ko;
                            for (int j = 0; j < P.T; ++j)   // sub-tile j: rows 128j.., TMEM columns jN..
                                tc_mma(tmem + (uint32_t)(j * P.N), desc_a[s] + so + ko + (uint64_t)j * sub, bd,
                                       P.idesc, (tap > 0 || s > 0 || k > 0) ? 1u : 0u);
                        }
                    }
                    tc_commit(&empty_bar[stage]);      // frees the stage when these MMAs are done
                    ++consumed_sh;
                    if (++stage == P.stages) { stage = 0; phase ^= 1u; }
                }
                if (!ok) break;
                tc_commit(&acc_full);                  // the tile's accumulator is complete
            }
        }
    } else {
        // ---------------------------------------------------------- epilogue (warps 2-5)
        const int quarter = warp & 3;                  // TMEM lanes 32*quarter .. +31
        uint32_t acc_phase = 0;
        for (long long tile = blockIdx.x; tile < P.tiles; tile += gridDim.x) {
            const bool got = mbar_wait(&acc_full, acc_phase, &abort_flag, P.status, 4);
            if (!__all_sync(0xffffffffu, got)) break;    // warp-uniform: tcgen05.ld below is .sync.aligned
            acc_phase ^= 1u;
            tc_fence_after();
            const int tx = (int)(tile % tiles_x);
            const long long r = tile / tiles_x;
            const int ty = (int)(r % tiles_y), tz = (int)(r / tiles_y);
          for (int j = 0; j < P.T; ++j) {
            const int m = j * kTileM + quarter * 32 + lane;   // voxel row of the tile
            const int x = tx * P.BW + (m % P.BW), y = ty * P.BH + (m / P.BW) % P.BH;
            const int z = tz * P.BD + m / (P.BW * P.BH);
            const long long vox = ((long long)z * P.H + y) * P.W + x;
            __nv_bfloat16 *dst = P.out + vox * P.N;
            for (int c = 0; c < P.N; c += 16) {
                uint32_t v[16];
                tc_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(j * P.N + c), v);
                tc_wait_ld();
                __align__(16) __nv_bfloat162 o[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    float a = __uint_as_float(v[2 * j]), b = __uint_as_float(v[2 * j + 1]);
                    if (P.bias != nullptr) {
                        a += P.bias[c + 2 * j];
                        b += P.bias[c + 2 * j + 1];
                    }
                    if (P.relu) {
                        a = fmaxf(a, 0.f);
                        b = fmaxf(b, 0.f);
                    }
                    o[j] = __floats2bfloat162_rn(a, b);
                }
                const uint4 *src = reinterpret_cast<const uint4 *>(o);
                uint4 *d4 = reinterpret_cast<uint4 *>(dst + c);
                d4[0] = src[0];
                d4[1] = src[1];
            }
          }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty);
        }
    }

    // wind down: every role has left its loop (all waits are bounded)
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && abort_flag) {
        // after an abort, wait (bounded) for the TMA loads still in flight
        volatile int never = 0;
        for (unsigned long long q = consumed_sh; q < issued_sh; ++q)
            mbar_wait(&full_bar[q % P.stages], (uint32_t)((q / P.stages) & 1u), &never, P.status, 5);
    }
    if (threadIdx.x == 32) {
        // every MMA this thread issued has completed before TMEM is released
        volatile int never = 0;
        tc_commit(&drain_bar);
        mbar_wait(&drain_bar, 0, &never, P.status, 6);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P.tmem_cols)
                     : "memory");
    }
}

// ------------------------------------------------------------------ host side

using kvtma::encoder;

inline CUtensorMapSwizzle swizzle_for(int row_bytes) {
    return row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                            : (row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

// Activation map: [D][H][W][C] BF16, box {kseg, BW, BH, BD}.
inline bool encode_act(CUtensorMap *m, const void *ptr, int C, int D, int H, int W, int kseg, int BW, int BH,
                       int BD) {
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {(cuuint32_t)kseg, (cuuint32_t)BW, (cuuint32_t)BH, (cuuint32_t)BD};
    cuuint32_t es[4] = {1, 1, 1, 1};
    return encoder()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kseg * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Weight map: [N][27][K] BF16, box {kseg, 1, N}.
inline bool encode_w(CUtensorMap *m, const void *ptr, int N, int K, int kseg) {
    cuuint64_t dims[3] = {(cuuint64_t)K, 27, (cuuint64_t)N};
    cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)27 * K * 2};
    cuuint32_t box[3] = {(cuuint32_t)kseg, 1, (cuuint32_t)N};
    cuuint32_t es[3] = {1, 1, 1};
    return encoder()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kseg * 2), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline uint32_t align1k(uint32_t x) { return (x + 1023u) & ~1023u; }

// The tile of M = 128*T voxels of a D x H x W volume: BW = min(W, 128),
// BH = min(H, M / BW), BD = the rest (at most 256, the TMA box limit); false
// when the volume is not a whole number of such tiles (the dimensions must
// be powers of two below the tile extents or multiples of them).
inline bool tile_shape(int D, int H, int W, int &BW, int &BH, int &BD, int T = 1) {
    const int M = kTileM * T;
    BW = W < kTileM ? W : kTileM;
    if (BW <= 0 || M % BW != 0 || W % BW != 0) return false;
    BH = H < M / BW ? H : M / BW;
    if (BH <= 0 || (M / BW) % BH != 0 || H % BH != 0 || BH > 256) return false;
    BD = M / (BW * BH);
    return BD <= 256 && D % BD == 0;
}

// out[v][N] = conv3(in1 (c1 channels) ++ in2 (c2 channels), w [N][27][c1+c2]) + bias, ReLU optional.
// Returns a message on a configuration this kernel does not cover (nullptr: launched).
inline const char *launch(const __nv_bfloat16 *in1, int c1, const __nv_bfloat16 *in2, int c2,
                          const __nv_bfloat16 *w, const float *bias, bool relu, __nv_bfloat16 *out, int N, int D,
                          int H, int W, int *status, int sm_count, cudaStream_t stream) {
    if (encoder() == nullptr) return "cuTensorMapEncodeTiled is not available";
    const int K = c1 + c2;
    auto ok_c = [](int c) { return c == 16 || c == 32 || c == 64 || c == 128; };
    if (!ok_c(c1) || (c2 != 0 && !ok_c(c2))) return "input channels must be 16, 32, 64 or 128";
    if (N % 16 != 0 || N < 16 || N > 256) return "output channels must be a multiple of 16 up to 256";
    int kseg = c1 < 64 ? c1 : 64;
    if (c2 != 0 && c2 < kseg) kseg = c2;
    // sub-tiles per tile: as many as keep T*N <= 128 TMEM columns and a stage
    // within 64 KB (narrow layers need several MMAs per stage to keep the
    // tensor pipe busy between TMA round trips)
    int T = 1;
    for (int t = 4; t > 1; t /= 2) {
        int bw, bh, bd;
        if (t * N <= 128 && (kTileM * t + N) * K * 2 <= 64 * 1024 && tile_shape(D, H, W, bw, bh, bd, t)) {
            T = t;
            break;
        }
    }
    int BW, BH, BD;
    if (!tile_shape(D, H, W, BW, BH, BD, T)) return "volume is not a whole number of 128-voxel tiles";
    Params P{};
    P.seg.n = 0;
    for (int src = 0; src < 2; ++src) {
        const int C = src == 0 ? c1 : c2;
        for (int c0 = 0; c0 < C; c0 += kseg) {
            if (P.seg.n == kMaxSeg) return "too many input channel segments";
            const int s = P.seg.n++;
            P.seg.kseg[s] = kseg;
            P.seg.src[s] = src;
            P.seg.c0[s] = c0;
            P.seg.kglob[s] = (src == 0 ? 0 : c1) + c0;
        }
    }
    uint32_t off = 0;
    for (int s = 0; s < P.seg.n; ++s) {
        P.seg.a_off[s] = off;
        off = align1k(off + (uint32_t)kTileM * T * kseg * 2);
    }
    for (int s = 0; s < P.seg.n; ++s) {
        P.seg.b_off[s] = off;
        off = align1k(off + (uint32_t)N * kseg * 2);
    }
    P.stage_bytes = off;
    P.tx_bytes = (uint32_t)(kTileM * T + N) * K * 2;
    const uint32_t budget = 200u * 1024u;
    P.stages = budget / P.stage_bytes;
    if (P.stages > 8) P.stages = 8;
    if (P.stages < 2) return "stage does not fit in shared memory";
    P.tmem_cols = 32;
    while (P.tmem_cols < (uint32_t)(N * T)) P.tmem_cols <<= 1;
    P.T = T;
    P.N = N;
    P.D = D;
    P.H = H;
    P.W = W;
    P.BW = BW;
    P.BH = BH;
    P.BD = BD;
    P.tiles = (long long)(D / BD) * (H / BH) * (W / BW);
    // kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), BF16 A
    // and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28
    P.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
    P.bias = bias;
    P.relu = relu ? 1 : 0;
    P.out = out;
    P.status = status;
    CUtensorMap ma0, ma1, mb;
    if (!encode_act(&ma0, in1, c1, D, H, W, kseg, BW, BH, BD)) return "activation tensor map rejected";
    if (!encode_act(&ma1, c2 ? in2 : in1, c2 ? c2 : c1, D, H, W, kseg, BW, BH, BD))
        return "activation tensor map rejected";
    if (!encode_w(&mb, w, N, K, kseg)) return "weight tensor map rejected";
    const size_t smem = (size_t)P.stages * P.stage_bytes + 1024;
    if (cudaFuncSetAttribute(conv3_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return "shared memory request rejected";
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv3_tc_kernel, kThreads, smem) != cudaSuccess ||
        per_sm < 1)
        return "occupancy query failed";
    if ((uint32_t)per_sm * P.tmem_cols > 512u) per_sm = (int)(512u / P.tmem_cols);
    long long grid = (long long)sm_count * per_sm;
    if (grid > P.tiles) grid = P.tiles;
    conv3_tc_kernel<<<(unsigned)grid, kThreads, smem, stream>>>(ma0, ma1, mb, P);
    return nullptr;
}

}  // namespace convtc
