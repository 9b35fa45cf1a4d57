// Kernels of the learned surrogate: a BF16 multilayer perceptron with a
// count-aware head (or a mixture-density head) over the dimer's protein and
// dimer counts, trained on ensembles the SSA engine generates.
//
//   * gemm_bf16: C[M][N] (+)= op(A) op(B) with BF16 operands and FP32
//     accumulation on mma.sync m16n8k16 (the legacy-path comparison).
//   * gemm_tc05: the same product on tcgen05 with the accumulator in tensor
//     memory, operands staged by vector loads, every orientation, split K for
//     the weight gradients (split_reduce sums the splits in a fixed order).
//   * gemm_tma: C = A B^T on tcgen05 with the operands loaded by
//     cp.async.bulk.tensor through a four-stage mbarrier ring (the forward
//     pass).
//   * mlp_infer: the whole forward pass for 128-query tiles in one persistent
//     kernel -- activations in shared memory, weights by TMA, each layer's
//     accumulator in tensor memory, bias and SiLU in the drain.
//   * bias_silu: Z += b; H = bf16(silu(Z)) (or identity for the head).
//   * silu_backward / head_backward: dZ = dH * silu'(Z) and the bias
//     gradients (column sums in a fixed order).
//   * count_loss: negative log-likelihood of the count-aware head (per
//     species a categorical over the counts 0 .. 30 and a tail class, the
//     tail a Gaussian mixture over the log-count residual) and its gradient
//     with respect to the head's raw outputs.
//   * mdn_loss: the same for a K-component diagonal Gaussian mixture in two
//     dimensions.
//   * adam: FP32 master weights, BF16 copies refreshed in place.
//   * rre: the reaction rate equations (RK4) at each query; an unrolled
//     variant for networks of 4 species and 5 reactions.
//   * mdn_sample / count_prep + count_draw: draws from each query's
//     distribution.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

namespace rbg {

namespace {

constexpr int kTileM = 64, kTileN = 64, kTileK = 32;

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// C = alpha * op(A) op(B) + beta * C, row-major everything.  op(A) is M x K:
// A[m][k] at A[m*lda + k], or A[k][m] at A[k*lda + m] when TA.  op(B) is
// K x N: B[k][n] at B[k*ldb + n], or B[n][k] at B[n*ldb + k] when TB.
// Block 64 x 64 of C, four warps of 32 x 32, K in steps of 32.
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const __nv_bfloat16 *__restrict__ A, int lda,
                                                        const __nv_bfloat16 *__restrict__ B, int ldb,
                                                        float *__restrict__ C, int ldc, int M, int N, int K,
                                                        float beta) {
    __shared__ __nv_bfloat16 As[kTileM][kTileK + 8];  // [m][k]
    __shared__ __nv_bfloat16 Bs[kTileN][kTileK + 8];  // [n][k]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.y * kTileM, n0 = blockIdx.x * kTileN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int g = lane >> 2, tg = lane & 3;
    float acc[2][4][4] = {};
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    for (int k0 = 0; k0 < K; k0 += kTileK) {
        for (int e = tid; e < kTileM * kTileK; e += 128) {
            const int mm = e / kTileK, kk = e % kTileK;
            const int m = m0 + mm, k = k0 + kk;
            As[mm][kk] = (m < M && k < K) ? (TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : zero;
        }
        for (int e = tid; e < kTileN * kTileK; e += 128) {
            const int nn = e / kTileK, kk = e % kTileK;
            const int n = n0 + nn, k = k0 + kk;
            Bs[nn][kk] = (n < N && k < K) ? (TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]) : zero;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kTileK; ks += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + g, c = ks + tg * 2;
                af[i][0] = pack_bf16(As[r][c], As[r][c + 1]);
                af[i][1] = pack_bf16(As[r + 8][c], As[r + 8][c + 1]);
                af[i][2] = pack_bf16(As[r][c + 8], As[r][c + 9]);
                af[i][3] = pack_bf16(As[r + 8][c + 8], As[r + 8][c + 9]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int n = wn + j * 8 + g, c = ks + tg * 2;
                bfr[j][0] = pack_bf16(Bs[n][c], Bs[n][c + 1]);
                bfr[j][1] = pack_bf16(Bs[n][c + 8], Bs[n][c + 9]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                        "{%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
                        : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]),
                          "r"(bfr[j][1]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int m = m0 + wm + i * 16 + g + h * 8;
                const int n = n0 + wn + j * 8 + tg * 2;
                if (m >= M) continue;
                for (int q = 0; q < 2; ++q) {
                    if (n + q >= N) continue;
                    float *c = C + (size_t)m * ldc + n + q;
                    const float v = acc[i][j][h * 2 + q];
                    *c = beta == 0.0f ? v : __fmaf_rn(beta, *c, v);
                }
            }
}

// ---------------------------------------------------------------- tcgen05
// The same product on the 5th-generation tensor cores: one CTA of four warps
// owns a 128 x 32 tile of C in tensor memory (32 columns of 32-bit
// accumulators).  K advances in rounds of up to kTcSlabs slabs of 64: every
// slab of a round is staged in shared memory at once (dynamic shared memory,
// the canonical K-major layout without swizzle: 8 x 16-byte core matrices,
// adjacent along K at 128 B, along M/N at 1 KiB).  Both orientations of an
// operand load 16-byte vectors, eight in flight per thread, coalesced along
// the dimension that is contiguous in memory; a K-contiguous operand stores
// each vector as one core-matrix row, an M/N-contiguous one scatters its
// eight elements over eight rows (lane groups rotate the order so the
// scattered stores of a warp fall in distinct banks).  One thread then issues
// four tcgen05.mma (K = 16 each) per slab and commits them to an mbarrier that
// every thread waits on, with an iteration limit, before the next round
// overwrites the operands.  For K <= 256 -- every product of the surrogate's
// forward pass -- that is one round: one latency of loads, 16 MMAs, one wait.
// Each warp then reads its 32 rows from its own tensor-memory lane quadrant,
// transposes them through shared memory and writes C one 128-byte row segment
// per store.  Products with few tiles and a long K (the weight gradients,
// K = the batch) split K over gridDim.z; each split writes its partial tile to
// a workspace and split_reduce_kernel adds the splits in a fixed order, so
// the result does not depend on scheduling.  A wait that runs out sets *err
// and the tile is left unwritten; tensor memory is always freed.
constexpr int kTcM = 128, kTcN = 32, kTcK = 64, kTcSlabs = 4;
constexpr size_t kTcSmem = (size_t)kTcSlabs * (kTcM + kTcN) * kTcK * 2;  // 80 KB

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start >> 4, leading (K) byte offset >> 4,
// stride (M/N) byte offset >> 4, descriptor version 1 (bits 46-48), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Element index of (row r, k) of slab s in the canonical layout.
template <int ROWS>
__device__ __forceinline__ int tc_index(int s, int r, int k) {
    return s * ROWS * kTcK + ((r >> 3) * (kTcK / 8) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

// Stage rows [r0, r0 + ROWS) x K range [k0, k0 + 64 * slabs) of op(X) into the
// canonical layout of `dst` ([slab][ROWS * kTcK] elements).  T = false: X is
// [rows][K] (K contiguous); T = true: X is [K][rows].  vec: ld a multiple of 8
// and X 16-byte aligned, so every 16-byte piece is one aligned vector load;
// pieces that cross the edge of X load element by element.  Out-of-range
// elements are zero.
template <int ROWS, bool T>
__device__ __forceinline__ void tc_stage(__nv_bfloat16 *dst, const __nv_bfloat16 *__restrict__ X, int ld, int r0,
                                         int R, int k0, int K, int slabs, bool vec) {
    const int tid = threadIdx.x;
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    if (!vec) {
        const int kw = slabs * kTcK;
        for (int e = tid; e < ROWS * kw; e += 128) {
            // T: consecutive threads take consecutive rows (contiguous in X)
            const int r = T ? e % ROWS : e / kw, kg = T ? e / ROWS : e % kw, m = r0 + r, kk = k0 + kg;
            const __nv_bfloat16 v = (m < R && kk < K) ? (T ? X[(size_t)kk * ld + m] : X[(size_t)m * ld + kk]) : zero;
            dst[tc_index<ROWS>(kg / kTcK, r, kg % kTcK)] = v;
        }
        return;
    }
    const int total = ROWS * slabs * (kTcK / 8);  // 16-byte pieces
    for (int e0 = 0; e0 < total; e0 += 128 * 8) {
        uint4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = e0 + u * 128 + tid;
            v[u] = make_uint4(0, 0, 0, 0);
            if (e >= total) continue;
            __nv_bfloat16 *w = reinterpret_cast<__nv_bfloat16 *>(&v[u]);
            if (!T) {
                // piece = 8 consecutive k of one row
                const int n8 = slabs * (kTcK / 8), m = r0 + e / n8, kk = k0 + (e % n8) * 8;
                if (m >= R) continue;
                if (kk + 8 <= K) {
                    v[u] = *reinterpret_cast<const uint4 *>(X + (size_t)m * ld + kk);
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j) w[j] = kk + j < K ? X[(size_t)m * ld + kk + j] : zero;
                }
            } else {
                // piece = 8 consecutive rows at one k; eight neighbouring
                // threads take eight consecutive k
                const int kl = e & 7, rest = e >> 3, r8 = rest % (ROWS / 8), kk = k0 + (rest / (ROWS / 8)) * 8 + kl;
                const int m = r0 + r8 * 8;
                if (kk >= K) continue;
                if (m + 8 <= R) {
                    v[u] = *reinterpret_cast<const uint4 *>(X + (size_t)kk * ld + m);
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j) w[j] = m + j < R ? X[(size_t)kk * ld + m + j] : zero;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = e0 + u * 128 + tid;
            if (e >= total) continue;
            if (!T) {
                const int n8 = slabs * (kTcK / 8), r = e / n8, g = e % n8;
                *reinterpret_cast<uint4 *>(&dst[tc_index<ROWS>(g >> 3, r, (g & 7) * 8)]) = v[u];
            } else {
                const int kl = e & 7, rest = e >> 3, r8 = rest % (ROWS / 8), kg = (rest / (ROWS / 8)) * 8 + kl;
                // rotate the four words by the lane group so that the four
                // groups of a warp write rows 2 apart: distinct banks
                const int g = (tid >> 3) & 3;
                const uint32_t w0 = v[u].x, w1 = v[u].y, w2 = v[u].z, w3 = v[u].w;
                const uint32_t a0 = (g & 1) ? w1 : w0, a1 = (g & 1) ? w2 : w1, a2 = (g & 1) ? w3 : w2,
                               a3 = (g & 1) ? w0 : w3;
                const uint32_t q[4] = {(g & 2) ? a2 : a0, (g & 2) ? a3 : a1, (g & 2) ? a0 : a2, (g & 2) ? a1 : a3};
                const int base = tc_index<ROWS>(kg / kTcK, r8 * 8, kg % kTcK);
                uint16_t *d16 = reinterpret_cast<uint16_t *>(dst);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int j = (2 * (i + g)) & 7;  // q[i] holds elements j, j + 1
                    d16[base + j * 8] = (uint16_t)(q[i] & 0xFFFFu);
                    d16[base + (j + 1) * 8] = (uint16_t)(q[i] >> 16);
                }
            }
        }
    }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_tc05_kernel(const __nv_bfloat16 *__restrict__ A, int lda,
                                                        const __nv_bfloat16 *__restrict__ B, int ldb,
                                                        float *__restrict__ C, int ldc, int M, int N, int K,
                                                        int k_split, float beta, int *err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(tc_smem);            // [slab][kTcM * kTcK]
    __nv_bfloat16 *Bs = As + (size_t)kTcSlabs * kTcM * kTcK;                    // [slab][kTcN * kTcK]
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
    // this CTA's K range; with splits, C is the split's own partial tile
    const int kb = blockIdx.z * k_split, ke = min(K, kb + k_split);
    if (gridDim.z > 1) C += (size_t)blockIdx.z * M * ldc;
    const uint32_t mb = smem_u32(&mbar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTcN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb));
        failed = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    // idesc: F32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                           ((uint32_t)(kTcM >> 4) << 24);
    const bool a_vec = (lda % 8) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
    const bool b_vec = (ldb % 8) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
    uint32_t parity = 0;
    bool any = false;
    for (int k0 = kb; k0 < ke; k0 += kTcSlabs * kTcK) {
        const int slabs = min(kTcSlabs, (ke - k0 + kTcK - 1) / kTcK);
        tc_stage<kTcM, TA>(As, A, lda, m0, M, k0, ke, slabs, a_vec);
        tc_stage<kTcN, !TB>(Bs, B, ldb, n0, N, k0, ke, slabs, b_vec);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0 && !failed) {
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            for (int sl = 0; sl < slabs; ++sl)
                for (int s = 0; s < kTcK / 16; ++s) {
                    const uint64_t ad =
                        smem_desc(smem_u32(As + (size_t)sl * kTcM * kTcK) + s * 256, 128, (kTcK / 8) * 128);
                    const uint64_t bd =
                        smem_desc(smem_u32(Bs + (size_t)sl * kTcN * kTcK) + s * 256, 128, (kTcK / 8) * 128);
                    const uint32_t acc = (any || sl > 0 || s > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                         : "memory");
        }
        any = true;
        __syncthreads();
        if (!failed) {
            if (!mbar_wait(mb, parity)) failed = 1;
        }
        parity ^= 1u;
        __syncthreads();
        if (failed) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (!failed) {
        // warp w reads tensor-memory lanes 32w .. 32w+31 = rows of its quadrant
        // (an empty K range leaves the accumulator unwritten: the tile is 0)
        uint32_t v[kTcN];
#pragma unroll
        for (int c0 = 0; c0 < kTcN; c0 += 16) {
            const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(v[c0 + 0]), "=r"(v[c0 + 1]), "=r"(v[c0 + 2]), "=r"(v[c0 + 3]), "=r"(v[c0 + 4]),
                  "=r"(v[c0 + 5]), "=r"(v[c0 + 6]), "=r"(v[c0 + 7]), "=r"(v[c0 + 8]), "=r"(v[c0 + 9]),
                  "=r"(v[c0 + 10]), "=r"(v[c0 + 11]), "=r"(v[c0 + 12]), "=r"(v[c0 + 13]), "=r"(v[c0 + 14]),
                  "=r"(v[c0 + 15])
                : "r"(addr));
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        // transpose through the (now idle) operand buffer: tile[row][col], row
        // pitch 33 words, so both the row writes and the column reads are
        // free of bank conflicts
        float *tile = reinterpret_cast<float *>(tc_smem) + warp * 32 * 33;
#pragma unroll
        for (int j = 0; j < kTcN; ++j) tile[lane * 33 + j] = any ? __uint_as_float(v[j]) : 0.0f;
        __syncwarp();
        const int n = n0 + lane;
        for (int rr = 0; rr < 32; ++rr) {
            const int row = m0 + warp * 32 + rr;
            if (row < M && n < N) {
                float *c = C + (size_t)row * ldc + n;
                const float x = tile[rr * 33 + lane];
                *c = beta == 0.0f ? x : __fmaf_rn(beta, *c, x);
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcN));
}

// C[m][n] = beta * C[m][n] + sum over splits s (in order) of P[s][m][n].
__global__ void split_reduce_kernel(const float *__restrict__ P, int splits, float *__restrict__ C, int ldc, int M,
                                    int N, float beta) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M * N) return;
    const int m = (int)(i / N), n = (int)(i % N);
    float acc = 0.0f;
    for (int s = 0; s < splits; ++s) acc += P[((size_t)s * M + m) * N + n];
    float *c = C + (size_t)m * ldc + n;
    *c = beta == 0.0f ? acc : __fmaf_rn(beta, *c, acc);
}

// ---------------------------------------------------------------- TMA-fed tcgen05
// C = A B^T for K-contiguous A [M][K] and B [N][K] (the forward pass: inputs
// times weights) with operands that TMA can address (row pitch a multiple of
// 16 bytes, 16-byte aligned base).  One CTA of four warps owns a 128 x 64
// tile of C in tensor memory.  A ring of four stages holds 64-wide K slices
// of A (128 rows) and B (64 rows) in the 128-byte-swizzle layout that the
// tensor map writes and the MMA descriptors read (8-row atoms of 1 KiB).
// Thread 0 of warp 0 issues the cp.async.bulk.tensor loads (the box's bytes
// counted on the stage's full barrier), thread 0 of warp 1 the MMAs (K = 16
// each, the descriptor start advanced 32 bytes per step inside the atom) and
// a commit to the stage's empty barrier; the producer waits on that before
// reloading the stage.  A last commit releases the four warps to drain tensor
// memory and write C through a shared-memory transpose.  Every wait has an
// iteration limit: one that runs out sets *err, no further copy or MMA is
// issued, copies already issued are waited for (again with a limit), and
// tensor memory is freed.
constexpr int kTmM = 128, kTmN = 64, kTmK = 64, kTmStages = 4;
constexpr int kTmABytes = kTmM * kTmK * 2, kTmBBytes = kTmN * kTmK * 2, kTmStage = kTmABytes + kTmBBytes;
constexpr size_t kTmSmem = (size_t)kTmStages * kTmStage + 1024;  // + alignment slack to 1 KiB

// Shared-memory descriptor of a K-major operand in the 128-byte swizzle:
// stride between 8-row atoms 1024 B, leading offset unused (1), version 1,
// layout type 2 (128-byte swizzle) in bits 61-63.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
            "r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__global__ void __launch_bounds__(128) gemm_tma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                       const __grid_constant__ CUtensorMap tmB, float *__restrict__ C,
                                                       int ldc, int M, int N, int K, float beta, int *err) {
    extern __shared__ unsigned char tm_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tm_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[kTmStages], empty[kTmStages], done;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    __shared__ int issued;  // k slices whose loads were issued
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kTmM, n0 = blockIdx.x * kTmN;
    const int nk = (K + kTmK - 1) / kTmK;
    const uint32_t sbase = smem_u32(sm);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int s = 0; s < kTmStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        failed = 0;
        issued = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    // idesc: F32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTmN >> 3) << 17) |
                           ((uint32_t)(kTmM >> 4) << 24);
    if (tid == 0) {
        // producer
        for (int kb = 0; kb < nk && !failed; ++kb) {
            const int s = kb % kTmStages;
            if (kb >= kTmStages && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((kb / kTmStages - 1) & 1))) {
                failed = 1;
                break;
            }
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(kTmStage)
                         : "memory");
            const uint32_t a_dst = sbase + s * kTmStage;
            tma_load_2d(a_dst, &tmA, kb * kTmK, m0, fb);
            tma_load_2d(a_dst + kTmABytes, &tmB, kb * kTmK, n0, fb);
            issued = kb + 1;
        }
    } else if (tid == 32) {
        // MMA issuer
        int kb = 0;
        for (; kb < nk; ++kb) {
            const int s = kb % kTmStages;
            if (failed || !mbar_wait(smem_u32(&full[s]), (uint32_t)((kb / kTmStages) & 1))) {
                failed = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            const uint32_t a_addr = sbase + s * kTmStage, b_addr = a_addr + kTmABytes;
            for (int k = 0; k < kTmK / 16; ++k) {
                const uint64_t ad = smem_desc_sw128(a_addr + k * 32), bd = smem_desc_sw128(b_addr + k * 32);
                const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&empty[s]))
                         : "memory");
        }
        // the last commit: every MMA issued so far has completed when it fires
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         smem_u32(&done))
                     : "memory");
    }
    __syncwarp();
    if (!mbar_wait(smem_u32(&done), 0u)) failed = 1;
    __syncthreads();
    if (failed) {
        // let every copy already issued land before the CTA's shared memory goes
        if (tid == 0)
            for (int kb = max(0, issued - kTmStages); kb < issued; ++kb)
                mbar_wait(smem_u32(&full[kb % kTmStages]), (uint32_t)((kb / kTmStages) & 1));
        if (tid == 0) atomicExch(err, 1);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;\n");
        // warp w drains tensor-memory lanes 32w .. 32w+31 (rows of its quadrant),
        // 32 columns at a time, through a [32][33] transpose in shared memory
        float *tile = reinterpret_cast<float *>(sm) + warp * 32 * 33;
        for (int c0 = 0; c0 < kTmN; c0 += 32) {
            uint32_t v[32];
#pragma unroll
            for (int h = 0; h < 32; h += 16) {
                const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c0 + h);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];\n"
                    : "=r"(v[h + 0]), "=r"(v[h + 1]), "=r"(v[h + 2]), "=r"(v[h + 3]), "=r"(v[h + 4]), "=r"(v[h + 5]),
                      "=r"(v[h + 6]), "=r"(v[h + 7]), "=r"(v[h + 8]), "=r"(v[h + 9]), "=r"(v[h + 10]),
                      "=r"(v[h + 11]), "=r"(v[h + 12]), "=r"(v[h + 13]), "=r"(v[h + 14]), "=r"(v[h + 15])
                    : "r"(addr));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = __uint_as_float(v[j]);
            __syncwarp();
            const int n = n0 + c0 + lane;
            for (int rr = 0; rr < 32; ++rr) {
                const int row = m0 + warp * 32 + rr;
                if (row < M && n < N) {
                    float *c = C + (size_t)row * ldc + n;
                    const float x = tile[rr * 33 + lane];
                    *c = beta == 0.0f ? x : __fmaf_rn(beta, *c, x);
                }
            }
            __syncwarp();
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmN));
}

__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + __expf(-x)); }

// ---------------------------------------------------------------- fused inference
// The whole forward pass of the surrogate for 128 queries per tile, in one
// kernel: features -> 4 x (256, SiLU) -> head.  The activations of a tile
// stay in shared memory as the next layer's A operand (128 x 256 BF16, the
// 128-byte-swizzle K-major layout: four 64-wide K slices of 16 KB); the
// weights stream through a three-stage ring by cp.async.bulk.tensor (one
// 64-wide K slice of a layer's [N][K] matrix per stage, issued by a producer
// warp that runs ahead across layers and tiles); the accumulator is a
// 128 x 256 FP32 tile in tensor memory.  Per layer thread 0 issues the MMAs
// (K = 16 each) and commits; eight warps then drain the accumulator (two per
// lane quadrant), add the bias and apply SiLU and write BF16
// back into the activation buffer, or the head's FP32 outputs to global
// memory.  Waits are bounded; one that runs out sets *err, the tile loop ends
// at the next layer boundary, issued copies are waited for, tensor memory is
// freed.
constexpr int kInfHid = 256, kInfLayers = 5, kInfStages = 3, kInfWarps = 9;  // 8 compute + 1 producer
constexpr int kInfHBytes = 128 * kInfHid * 2;              // activations, 64 KB
constexpr int kInfStageBytes = kInfHid * 128;              // one weight K slice of up to 256 rows
constexpr size_t kInfSmem = (size_t)kInfHBytes + (size_t)kInfStages * kInfStageBytes + 1024;

struct InferMaps {
    CUtensorMap w[kInfLayers];
};

// OR of v over the 256 threads of warps 0-7 at named barrier 1: every one of
// them gets the same answer, so a loop they leave on it is left by all.
__device__ __forceinline__ bool bar_or_256(bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, 256, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

__global__ void __launch_bounds__(32 * kInfWarps, 1) mlp_infer_kernel(const __grid_constant__ InferMaps maps,
                                                                      const float *__restrict__ F, int Q, int n_in,
                                                                      const float *__restrict__ x_mean,
                                                                      const float *__restrict__ x_std,
                                                                      const float *__restrict__ b0,
                                                                      const float *__restrict__ b1,
                                                                      const float *__restrict__ b2,
                                                                      const float *__restrict__ b3,
                                                                      const float *__restrict__ b4, int n_out,
                                                                      float *__restrict__ O, int *err) {
    extern __shared__ unsigned char inf_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(inf_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char *H = sm;                     // [4 slices][128 rows][128 B], swizzled
    unsigned char *ring = sm + kInfHBytes;     // [stage][up to 256 rows][128 B]
    __shared__ float bias[kInfLayers - 1][kInfHid];
    __shared__ float bias_out[kInfHid];
    __shared__ __align__(8) uint64_t full[kInfStages], empty[kInfStages], layer_done;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    __shared__ int issued;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_tiles = (Q + 127) / 128;
    const int n_mma = (n_out + 15) & ~15;  // head MMA width (the tensor map zero-fills rows >= n_out)
    // K slices and weight rows per layer
    auto slices = [&](int l) { return l == 0 ? 1 : kInfHid / 64; };
    auto rows = [&](int l) { return l == kInfLayers - 1 ? n_mma : kInfHid; };
    for (int k = tid; k < kInfHid; k += blockDim.x) {
        bias[0][k] = b0[k];
        bias[1][k] = b1[k];
        bias[2][k] = b2[k];
        bias[3][k] = b3[k];
        bias_out[k] = k < n_out ? b4[k] : 0.0f;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(kInfHid));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int s = 0; s < kInfStages; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&layer_done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        failed = 0;
        issued = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_base;
    const uint32_t h_addr = smem_u32(H), ring_addr = smem_u32(ring);

    if (warp == kInfWarps - 1) {
        // ---- producer: every weight slice of every layer of every tile, in order
        if (lane == 0) {
            int seq = 0;
            for (int tile = blockIdx.x; tile < n_tiles && !failed; tile += gridDim.x)
                for (int l = 0; l < kInfLayers && !failed; ++l)
                    for (int ks = 0; ks < slices(l); ++ks, ++seq) {
                        const int st = seq % kInfStages;
                        if (seq >= kInfStages &&
                            !mbar_wait(smem_u32(&empty[st]), (uint32_t)((seq / kInfStages - 1) & 1))) {
                            failed = 1;
                            break;
                        }
                        const uint32_t fb = smem_u32(&full[st]);
                        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb),
                                     "r"(rows(l) * 128)
                                     : "memory");
                        tma_load_2d(ring_addr + st * kInfStageBytes, &maps.w[l], ks * 64, 0, fb);
                        issued = seq + 1;
                    }
        }
    } else {
        // ---- eight warps: stage inputs, issue MMAs (thread 0), drain and
        // activate.  Warp w reads tensor-memory lanes 32 (w % 4) .. + 31 (rows
        // of its quadrant); warps w and w + 4 split the columns in 32-wide
        // chunks.
        const int r = (warp & 3) * 32 + lane;  // this thread's row of the tile (tensor-memory lane)
        const int half = warp >> 2;
        const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
        int seq = 0, layers_run = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
            const int q = tile * 128 + r;
            if (half == 0) {
                // features of row r, normalised, as BF16 in K slice 0 (zeros beyond n_in)
                uint32_t w4[4] = {0u, 0u, 0u, 0u};
                if (q < Q)
                    for (int j = 0; j < 8 && j < n_in; j += 2) {
                        const float v0 = (F[(size_t)q * n_in + j] - x_mean[j]) / x_std[j];
                        const float v1 =
                            j + 1 < n_in ? (F[(size_t)q * n_in + j + 1] - x_mean[j + 1]) / x_std[j + 1] : 0.0f;
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v0, v1);
                        w4[j >> 1] = *reinterpret_cast<const uint32_t *>(&h2);
                    }
                for (int c = 0; c < 8; ++c) {
                    const uint4 v = c == 0 ? make_uint4(w4[0], w4[1], w4[2], w4[3]) : make_uint4(0u, 0u, 0u, 0u);
                    *reinterpret_cast<uint4 *>(H + r * 128 + ((c ^ (r & 7)) << 4)) = v;
                }
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("bar.sync 1, 256;\n" ::: "memory");
            for (int l = 0; l < kInfLayers; ++l) {
                if (tid == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;\n");
                    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) |
                                           ((uint32_t)(rows(l) >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
                    const int ksteps = l == 0 ? (n_in + 15) / 16 : 4;  // 16-wide K steps per slice
                    for (int ks = 0; ks < slices(l); ++ks, ++seq) {
                        const int st = seq % kInfStages;
                        if (failed || !mbar_wait(smem_u32(&full[st]), (uint32_t)((seq / kInfStages) & 1))) {
                            failed = 1;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;\n");
                        for (int k = 0; k < ksteps; ++k) {
                            const uint64_t ad = smem_desc_sw128(h_addr + ks * 16384 + k * 32);
                            const uint64_t bd = smem_desc_sw128(ring_addr + st * kInfStageBytes + k * 32);
                            const uint32_t acc = (ks > 0 || k > 0) ? 1u : 0u;
                            asm volatile(
                                "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                        }
                        asm volatile(
                            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                smem_u32(&empty[st]))
                            : "memory");
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     smem_u32(&layer_done))
                                 : "memory");
                }
                __syncwarp();
                bool bad = !mbar_wait(smem_u32(&layer_done), (uint32_t)(layers_run & 1));
                ++layers_run;
                // one decision for all eight warps (the producer may set failed
                // at any moment; the epilogue's tensor-memory loads are
                // warp-collective and its barriers count all 256 threads)
                stop = bar_or_256(bad || failed != 0);
                if (stop) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                const bool last = l == kInfLayers - 1;
                const int ncol = last ? n_mma : kInfHid;
                for (int c0 = half * 32; c0 < ncol; c0 += 64) {
                    uint32_t v[32];
#pragma unroll
                    for (int h = 0; h < 32; h += 16)
                        asm volatile(
                            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                            "%15}, [%16];\n"
                            : "=r"(v[h + 0]), "=r"(v[h + 1]), "=r"(v[h + 2]), "=r"(v[h + 3]), "=r"(v[h + 4]),
                              "=r"(v[h + 5]), "=r"(v[h + 6]), "=r"(v[h + 7]), "=r"(v[h + 8]), "=r"(v[h + 9]),
                              "=r"(v[h + 10]), "=r"(v[h + 11]), "=r"(v[h + 12]), "=r"(v[h + 13]), "=r"(v[h + 14]),
                              "=r"(v[h + 15])
                            : "r"(lane_base + (uint32_t)(c0 + h)));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                    if (last) {
                        if (q < Q)
#pragma unroll
                            for (int j = 0; j < 32; j += 4) {
                                const int n = c0 + j;
                                if (n + 4 <= n_out) {
                                    *reinterpret_cast<float4 *>(O + (size_t)q * n_out + n) = make_float4(
                                        __uint_as_float(v[j]) + bias_out[n], __uint_as_float(v[j + 1]) + bias_out[n + 1],
                                        __uint_as_float(v[j + 2]) + bias_out[n + 2],
                                        __uint_as_float(v[j + 3]) + bias_out[n + 3]);
                                } else {
                                    for (int u = 0; u < 4 && n + u < n_out; ++u)
                                        O[(size_t)q * n_out + n + u] = __uint_as_float(v[j + u]) + bias_out[n + u];
                                }
                            }
                    } else {
                        // bias, SiLU (z / (1 + e^-z) with the fast reciprocal), BF16
                        uint32_t pk[16];
#pragma unroll
                        for (int j = 0; j < 32; j += 2) {
                            const float z0 = __uint_as_float(v[j]) + bias[l][c0 + j];
                            const float z1 = __uint_as_float(v[j + 1]) + bias[l][c0 + j + 1];
                            const __nv_bfloat162 h2 = __floats2bfloat162_rn(__fdividef(z0, 1.0f + __expf(-z0)),
                                                                            __fdividef(z1, 1.0f + __expf(-z1)));
                            pk[j >> 1] = *reinterpret_cast<const uint32_t *>(&h2);
                        }
                        // columns c0 .. c0+31: K slice c0 / 64, 16-byte chunks (c0 % 64) / 8 .. + 3
                        unsigned char *row = H + (c0 >> 6) * 16384 + r * 128;
                        const int ch = (c0 & 63) >> 3;
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            *reinterpret_cast<uint4 *>(row + (((ch + i) ^ (r & 7)) << 4)) =
                                make_uint4(pk[4 * i], pk[4 * i + 1], pk[4 * i + 2], pk[4 * i + 3]);
                    }
                }
                // the accumulator is read and the activations written before the
                // next layer's MMAs start
                asm volatile("tcgen05.fence::before_thread_sync;\n");
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                asm volatile("bar.sync 1, 256;\n" ::: "memory");
            }
            if (stop) break;
        }
        if (stop && tid == 0) failed = 1;
    }
    __syncthreads();
    if (failed) {
        if (tid == 0) {
            // copies already issued land before the shared memory is released
            const int n = issued;
            for (int sq = max(0, n - kInfStages); sq < n; ++sq)
                mbar_wait(smem_u32(&full[sq % kInfStages]), (uint32_t)((sq / kInfStages) & 1));
            atomicExch(err, 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kInfHid));
}

// Z[m][n] += b[n]; H = bf16(silu(Z)) (act = 1) or bf16(Z) (act = 0).
__global__ void bias_act_kernel(float *Z, const float *b, __nv_bfloat16 *H, int M, int N, int act) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M * N) return;
    const float z = Z[i] + b[i % N];
    Z[i] = z;
    if (H) H[i] = __float2bfloat16(act ? z * sigmoidf_(z) : z);
}

// Column sums of the backward pass: a block of 32 x 32 threads owns 32
// columns; thread (x, y) walks rows y, y + 32, ... of column x (a warp reads
// 128 contiguous bytes per row), then the 32 partial sums of a column are
// added in a fixed order, so db does not depend on scheduling.
constexpr int kColX = 32, kColY = 32;

// dZ = dH * silu'(Z) as BF16 for the next GEMMs; db[n] = sum_m dZ[m][n].
__global__ void __launch_bounds__(kColX *kColY) silu_backward_kernel(const float *Z, const float *dH,
                                                                     __nv_bfloat16 *dZ, float *db, int M, int N) {
    __shared__ float part[kColY][kColX + 1];
    const int n = blockIdx.x * kColX + threadIdx.x;
    float s = 0.0f;
    if (n < N)
        for (int m = threadIdx.y; m < M; m += kColY) {
            const size_t i = (size_t)m * N + n;
            const float z = Z[i], sg = sigmoidf_(z);
            const float d = dH[i] * sg * (1.0f + z * (1.0f - sg));
            dZ[i] = __float2bfloat16(d);
            s += d;
        }
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && n < N) {
        float t = 0.0f;
        for (int j = 0; j < kColY; ++j) t += part[j][threadIdx.x];
        db[n] = t;
    }
}

// Bias gradient of the head and its BF16 copy: db[n] = sum_m G[m][n].
__global__ void __launch_bounds__(kColX *kColY) head_backward_kernel(const float *G, __nv_bfloat16 *Gb, float *db,
                                                                     int M, int N) {
    __shared__ float part[kColY][kColX + 1];
    const int n = blockIdx.x * kColX + threadIdx.x;
    float s = 0.0f;
    if (n < N)
        for (int m = threadIdx.y; m < M; m += kColY) {
            const float v = G[(size_t)m * N + n];
            Gb[(size_t)m * N + n] = __float2bfloat16(v);
            s += v;
        }
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && n < N) {
        float t = 0.0f;
        for (int j = 0; j < kColY; ++j) t += part[j][threadIdx.x];
        db[n] = t;
    }
}

__device__ __forceinline__ float softplusf_(float x) { return x > 20.0f ? x : log1pf(__expf(x)); }

// Head layout per row (K components): logits[K] | mu1[K] | mu2[K] | s1[K] | s2[K],
// sigma = softplus(s) + 1e-3.  loss[row] = -log sum_k pi_k N(y1; mu1, s1) N(y2; mu2, s2);
// G = d(mean loss)/d(raw head outputs).
__global__ void mdn_loss_kernel(const float *O, const float *Y, int B, int K, float *loss, float *G) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= B) return;
    const float *o = O + (size_t)row * 5 * K;
    float *gr = G + (size_t)row * 5 * K;
    const float y1 = Y[2 * row], y2 = Y[2 * row + 1];
    float lmax = -1e30f, mx = -1e30f;
    for (int k = 0; k < K; ++k) lmax = fmaxf(lmax, o[k]);
    float zs = 0.0f;
    for (int k = 0; k < K; ++k) zs += __expf(o[k] - lmax);
    const float logz = lmax + logf(zs);
    float lp[16];
    for (int k = 0; k < K; ++k) {
        const float s1 = softplusf_(o[3 * K + k]) + 1e-3f, s2 = softplusf_(o[4 * K + k]) + 1e-3f;
        const float e1 = (y1 - o[K + k]) / s1, e2 = (y2 - o[2 * K + k]) / s2;
        lp[k] = (o[k] - logz) - 0.5f * (e1 * e1 + e2 * e2) - logf(s1) - logf(s2) - 1.8378770664f;
        mx = fmaxf(mx, lp[k]);
    }
    float tot = 0.0f;
    for (int k = 0; k < K; ++k) tot += __expf(lp[k] - mx);
    const float ll = mx + logf(tot);
    loss[row] = -ll;
    const float inv_b = 1.0f / (float)B;
    for (int k = 0; k < K; ++k) {
        const float r = __expf(lp[k] - ll);              // responsibility
        const float pi = __expf(o[k] - logz);
        const float s1 = softplusf_(o[3 * K + k]) + 1e-3f, s2 = softplusf_(o[4 * K + k]) + 1e-3f;
        const float e1 = (y1 - o[K + k]) / s1, e2 = (y2 - o[2 * K + k]) / s2;
        gr[k] = (pi - r) * inv_b;
        gr[K + k] = -r * e1 / s1 * inv_b;
        gr[2 * K + k] = -r * e2 / s2 * inv_b;
        // d/ds of -log N: (1 - e^2)/sigma * dsigma/ds, dsigma/ds = sigmoid(s)
        gr[3 * K + k] = r * (1.0f - e1 * e1) / s1 * sigmoidf_(o[3 * K + k]) * inv_b;
        gr[4 * K + k] = r * (1.0f - e2 * e2) / s2 * sigmoidf_(o[4 * K + k]) * inv_b;
    }
}

// Count-aware head, per species s a block of HS = kNC + 3 KT outputs at s * HS:
// logits[kNC] (class c < kNC - 1: the count c; class kNC - 1: a count of at
// least kNC - 1), then the tail's KT (at most kKTMax) weight logits, means and raw scales
// (sigma = softplus(raw) + 1e-3) over the residual y = log(n + v) - b_s of a
// tail count n (v ~ U[0, 1), b_s the rate-equation log mean).  Y rows are
// (n_protein, n_dimer, y_protein, y_dimer).  loss[row] = sum_s -log P_s with
// P_s = pi_c for a small count c, pi_tail * sum_k w_k N(y; mu_k, sigma_k) for
// a tail count; G = d(mean loss)/d(raw head outputs).
constexpr int kNC = 32, kKTMax = 16;

__global__ void count_loss_kernel(const float *O, const float *Y, int B, int kKT, float *loss, float *G) {
    const int kHS = kNC + 3 * kKT;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= B) return;
    const float inv_b = 1.0f / (float)B;
    float total = 0.0f;
    for (int sp = 0; sp < 2; ++sp) {
        const float *o = O + (size_t)row * 2 * kHS + sp * kHS;
        float *gr = G + (size_t)row * 2 * kHS + sp * kHS;
        const float n = Y[4 * row + sp], y = Y[4 * row + 2 + sp];
        const int c = n < (float)(kNC - 1) ? (int)n : kNC - 1;
        float lmax = -1e30f;
        for (int k = 0; k < kNC; ++k) lmax = fmaxf(lmax, o[k]);
        float zs = 0.0f;
        for (int k = 0; k < kNC; ++k) zs += __expf(o[k] - lmax);
        const float logz = lmax + logf(zs);
        total += logz - o[c];
        for (int k = 0; k < kNC; ++k) gr[k] = (__expf(o[k] - logz) - (k == c ? 1.0f : 0.0f)) * inv_b;
        const float *tw = o + kNC, *tm = tw + kKT, *ts = tm + kKT;
        float *gw = gr + kNC, *gm = gw + kKT, *gs = gm + kKT;
        if (c < kNC - 1) {
            for (int k = 0; k < kKT; ++k) gw[k] = gm[k] = gs[k] = 0.0f;
            continue;
        }
        float wmax = -1e30f;
        for (int k = 0; k < kKT; ++k) wmax = fmaxf(wmax, tw[k]);
        float ws = 0.0f;
        for (int k = 0; k < kKT; ++k) ws += __expf(tw[k] - wmax);
        const float logw = wmax + logf(ws);
        float lp[kKTMax], mx = -1e30f;
        for (int k = 0; k < kKT; ++k) {
            const float sg = softplusf_(ts[k]) + 1e-3f, e = (y - tm[k]) / sg;
            lp[k] = (tw[k] - logw) - 0.5f * e * e - logf(sg) - 0.9189385332f;
            mx = fmaxf(mx, lp[k]);
        }
        float tot = 0.0f;
        for (int k = 0; k < kKT; ++k) tot += __expf(lp[k] - mx);
        const float ll = mx + logf(tot);
        total -= ll;
        for (int k = 0; k < kKT; ++k) {
            const float r = __expf(lp[k] - ll), w = __expf(tw[k] - logw);
            const float sg = softplusf_(ts[k]) + 1e-3f, e = (y - tm[k]) / sg;
            gw[k] = (w - r) * inv_b;
            gm[k] = -r * e / sg * inv_b;
            gs[k] = r * (1.0f - e * e) / sg * sigmoidf_(ts[k]) * inv_b;
        }
    }
    loss[row] = total;
}

__global__ void adam_kernel(float *w, __nv_bfloat16 *wb, const float *g, float *m, float *v, int n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Draws: row r of out takes query r / per_query's mixture; component by its
// weight, then two Gaussians (Box-Muller).  With `base` ([queries][2]) the
// draw z is a residual in log space and the row receives the count
// floor(exp(z + base)), at least 0.
__global__ void mdn_sample_kernel(const float *O, int B, int K, uint64_t seed, float *out, int per_query,
                                  const float *base) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= B) return;
    const float *o = O + (size_t)(row / per_query) * 5 * K;
    const uint64_t h = mix64(seed ^ mix64((uint64_t)row + 0x9E3779B97F4A7C15ull));
    const float u0 = (float)(h >> 40) * 0x1p-24f, u1 = ((float)((h >> 16) & 0xFFFFFF) + 0.5f) * 0x1p-24f;
    const uint64_t h2 = mix64(h);
    const float u2 = (float)(h2 >> 40) * 0x1p-24f;
    float lmax = -1e30f;
    for (int k = 0; k < K; ++k) lmax = fmaxf(lmax, o[k]);
    float zs = 0.0f;
    for (int k = 0; k < K; ++k) zs += __expf(o[k] - lmax);
    float acc = 0.0f;
    int c = K - 1;
    for (int k = 0; k < K; ++k) {
        acc += __expf(o[k] - lmax) / zs;
        if (u0 < acc) {
            c = k;
            break;
        }
    }
    const float rad = sqrtf(-2.0f * logf(u1)), ang = 6.2831853f * u2;
    const float s1 = softplusf_(o[3 * K + c]) + 1e-3f, s2 = softplusf_(o[4 * K + c]) + 1e-3f;
    const float z1 = o[K + c] + s1 * rad * cosf(ang), z2 = o[2 * K + c] + s2 * rad * sinf(ang);
    if (base) {
        const float *bq = base + (size_t)(row / per_query) * 2;
        out[2 * row] = fmaxf(floorf(expf(z1 + bq[0])), 0.0f);
        out[2 * row + 1] = fmaxf(floorf(expf(z2 + bq[1])), 0.0f);
    } else {
        out[2 * row] = z1;
        out[2 * row + 1] = z2;
    }
}

// Reaction rate equations of a mass-action network -- the deterministic
// limit of the SSA, dx/dt = sum_r nu_r k_r prod_s ff(x_s, e_rs) with ff the
// falling factorial x (x - 1) ... (x - e + 1), clamped at 0 where it would turn
// negative -- integrated in float32 from x0 to each query's t by classic
// fourth-order Runge-Kutta with n_steps equal steps.  E[R][S] holds the
// reactant orders, N[R][S] the net changes; rates is [Q][R].  out[q][j] is
// the solution's species out_idx[j] at t_q.  The surrogate predicts the SSA's
// count distribution relative to this solution.
constexpr int kRreMaxS = 16, kRreMaxR = 32;

__device__ void rre_rhs(const int *E, const float *N, const float *k, int S, int R, const float *x, float *dx) {
    for (int s = 0; s < S; ++s) dx[s] = 0.0f;
    for (int r = 0; r < R; ++r) {
        float a = k[r];
        for (int s = 0; s < S; ++s) {
            const int e = E[r * S + s];
            for (int j = 0; j < e; ++j) a *= fmaxf(x[s] - (float)j, 0.0f);
        }
        for (int s = 0; s < S; ++s) dx[s] += N[r * S + s] * a;
    }
}

__global__ void rre_kernel(const float *rates, const float *tq, int Q, int S, int R, const int *E, const float *N,
                           const float *x0, int n_steps, const int *out_idx, int n_out, float *out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Q) return;
    float k[kRreMaxR], x[kRreMaxS], xt[kRreMaxS], k1[kRreMaxS], k2[kRreMaxS], k3[kRreMaxS], k4[kRreMaxS];
    for (int r = 0; r < R; ++r) k[r] = rates[(size_t)q * R + r];
    for (int s = 0; s < S; ++s) x[s] = x0[s];
    const float h = tq[q] / (float)n_steps;
    for (int n = 0; n < n_steps; ++n) {
        rre_rhs(E, N, k, S, R, x, k1);
        for (int s = 0; s < S; ++s) xt[s] = x[s] + 0.5f * h * k1[s];
        rre_rhs(E, N, k, S, R, xt, k2);
        for (int s = 0; s < S; ++s) xt[s] = x[s] + 0.5f * h * k2[s];
        rre_rhs(E, N, k, S, R, xt, k3);
        for (int s = 0; s < S; ++s) xt[s] = x[s] + h * k3[s];
        rre_rhs(E, N, k, S, R, xt, k4);
        for (int s = 0; s < S; ++s) x[s] = fmaxf(x[s] + h / 6.0f * (k1[s] + 2.0f * k2[s] + 2.0f * k3[s] + k4[s]), 0.0f);
    }
    for (int j = 0; j < n_out; ++j) out[(size_t)q * n_out + j] = x[out_idx[j]];
}

// The same integration for a network of exactly S_ species and R_ reactions
// whose propensities have at most two factors each (mass action of order
// <= 2): reaction r's factors are the slots (species, offset) in the generic
// loop's order -- species ascending, offsets 0 then 1 -- so a = k * f1 * f2
// with f = max(x[species] - offset, 0) (an unused slot multiplies by 1) is
// the generic product, factor for factor; the changes are applied to every
// species as there.  Same operations in the same order, same results.  A
// network outside that form takes the generic loops.
template <int S_>
__device__ __forceinline__ float rre_pick(const float (&x)[S_], int s) {
    float v = 1.0f;  // s == S_: the constant factor of an unused slot
#pragma unroll
    for (int i = 0; i < S_; ++i) v = s == i ? x[i] : v;
    return v;
}

template <int S_, int R_>
__device__ __forceinline__ void rre_rhs_fixed(const int (&s1)[R_], const float (&o1)[R_], const int (&s2)[R_],
                                              const float (&o2)[R_], const float (&nn)[R_][S_], const float (&k)[R_],
                                              const float (&x)[S_], float (&dx)[S_]) {
#pragma unroll
    for (int s = 0; s < S_; ++s) dx[s] = 0.0f;
#pragma unroll
    for (int r = 0; r < R_; ++r) {
        float a = k[r];
        if (s1[r] < S_) a *= fmaxf(rre_pick<S_>(x, s1[r]) - o1[r], 0.0f);
        if (s2[r] < S_) a *= fmaxf(rre_pick<S_>(x, s2[r]) - o2[r], 0.0f);
#pragma unroll
        for (int s = 0; s < S_; ++s) dx[s] += nn[r][s] * a;
    }
}

template <int S_, int R_>
__global__ void rre_fixed_kernel(const float *rates, const float *tq, int Q, const int *E, const float *N,
                                 const float *x0, int n_steps, const int *out_idx, int n_out, float *out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Q) return;
    int s1[R_], s2[R_];
    float o1[R_], o2[R_], nn[R_][S_], k[R_], x[S_], xt[S_], k1[S_], k2[S_], k3[S_], k4[S_];
    bool two = true;  // every reaction of order <= 2
#pragma unroll
    for (int r = 0; r < R_; ++r) {
        k[r] = rates[(size_t)q * R_ + r];
        s1[r] = s2[r] = S_;
        o1[r] = o2[r] = 0.0f;
        int n_f = 0;
#pragma unroll
        for (int s = 0; s < S_; ++s) {
            nn[r][s] = N[r * S_ + s];
            const int e = E[r * S_ + s];
            for (int j = 0; j < e; ++j, ++n_f) {
                if (n_f == 0) {
                    s1[r] = s;
                    o1[r] = (float)j;
                } else if (n_f == 1) {
                    s2[r] = s;
                    o2[r] = (float)j;
                }
            }
        }
        two = two && n_f <= 2;
    }
    if (!two) {  // higher orders: the generic loops
        float kk[kRreMaxR], xg[kRreMaxS], xtg[kRreMaxS], g1[kRreMaxS], g2[kRreMaxS], g3[kRreMaxS], g4[kRreMaxS];
        for (int r = 0; r < R_; ++r) kk[r] = k[r];
        for (int s = 0; s < S_; ++s) xg[s] = x0[s];
        const float h = tq[q] / (float)n_steps;
        for (int n = 0; n < n_steps; ++n) {
            rre_rhs(E, N, kk, S_, R_, xg, g1);
            for (int s = 0; s < S_; ++s) xtg[s] = xg[s] + 0.5f * h * g1[s];
            rre_rhs(E, N, kk, S_, R_, xtg, g2);
            for (int s = 0; s < S_; ++s) xtg[s] = xg[s] + 0.5f * h * g2[s];
            rre_rhs(E, N, kk, S_, R_, xtg, g3);
            for (int s = 0; s < S_; ++s) xtg[s] = xg[s] + h * g3[s];
            rre_rhs(E, N, kk, S_, R_, xtg, g4);
            for (int s = 0; s < S_; ++s)
                xg[s] = fmaxf(xg[s] + h / 6.0f * (g1[s] + 2.0f * g2[s] + 2.0f * g3[s] + g4[s]), 0.0f);
        }
        for (int j = 0; j < n_out; ++j) out[(size_t)q * n_out + j] = xg[out_idx[j]];
        return;
    }
#pragma unroll
    for (int s = 0; s < S_; ++s) x[s] = x0[s];
    const float h = tq[q] / (float)n_steps;
    const float h2 = 0.5f * h, h6 = h / 6.0f;  // the generic kernel's (0.5f * h) and (h / 6.0f)
    for (int n = 0; n < n_steps; ++n) {
        rre_rhs_fixed<S_, R_>(s1, o1, s2, o2, nn, k, x, k1);
#pragma unroll
        for (int s = 0; s < S_; ++s) xt[s] = x[s] + h2 * k1[s];
        rre_rhs_fixed<S_, R_>(s1, o1, s2, o2, nn, k, xt, k2);
#pragma unroll
        for (int s = 0; s < S_; ++s) xt[s] = x[s] + h2 * k2[s];
        rre_rhs_fixed<S_, R_>(s1, o1, s2, o2, nn, k, xt, k3);
#pragma unroll
        for (int s = 0; s < S_; ++s) xt[s] = x[s] + h * k3[s];
        rre_rhs_fixed<S_, R_>(s1, o1, s2, o2, nn, k, xt, k4);
#pragma unroll
        for (int s = 0; s < S_; ++s)
            x[s] = fmaxf(x[s] + h6 * (k1[s] + 2.0f * k2[s] + 2.0f * k3[s] + k4[s]), 0.0f);
    }
    for (int j = 0; j < n_out; ++j) {
        float v = 0.0f;
#pragma unroll
        for (int s = 0; s < S_; ++s)
            if (s == out_idx[j]) v = x[s];
        out[(size_t)q * n_out + j] = v;
    }
}

// Draws from the count-aware head, in two passes.  count_prep_kernel turns
// each (query, species) head block into what the draws need: the running sums
// of the class probabilities (softmax in the block's order, as the loss
// computes it), the running sums of the tail weights, the tail means and the
// tail scales softplus(s) + 1e-3.  count_draw_kernel then takes one draw per
// thread: class c = the first class whose running sum exceeds u0 (a binary
// search over the non-decreasing sums: #{k : cum_k <= u0}), a count below 31
// returned as is; the tail class picks a component by the same rule on u1
// and draws z = mu + sigma * N(0, 1) (Box-Muller on u2, u3), returning
// max(floor(exp(z + b)), 31).  The uniforms come from a SplitMix64-style
// hash of (seed, draw, species).  P has O's layout: per species 32 + 3 KT
// floats.
__global__ void count_prep_kernel(const float *O, int Q, int kKT, float *P) {
    const int kHS = kNC + 3 * kKT;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * Q) return;
    const float *o = O + (size_t)i * kHS;
    float *p = P + (size_t)i * kHS;
    float lmax = -1e30f;
    for (int k = 0; k < kNC; ++k) lmax = fmaxf(lmax, o[k]);
    float zs = 0.0f;
    for (int k = 0; k < kNC; ++k) zs += __expf(o[k] - lmax);
    float acc = 0.0f;
    for (int k = 0; k < kNC; ++k) {
        acc += __expf(o[k] - lmax) / zs;
        p[k] = acc;
    }
    const float *tw = o + kNC, *tm = tw + kKT, *ts = tm + kKT;
    float wmax = -1e30f;
    for (int k = 0; k < kKT; ++k) wmax = fmaxf(wmax, tw[k]);
    float ws = 0.0f;
    for (int k = 0; k < kKT; ++k) ws += __expf(tw[k] - wmax);
    acc = 0.0f;
    for (int k = 0; k < kKT; ++k) {
        acc += __expf(tw[k] - wmax) / ws;
        p[kNC + k] = acc;
        p[kNC + kKT + k] = tm[k];
        p[kNC + 2 * kKT + k] = softplusf_(ts[k]) + 1e-3f;
    }
}

// #{k < N : cum[k] <= u} for non-decreasing cum (binary search, N a power of 2)
template <int N>
__device__ __forceinline__ int count_le(const float *cum, float u) {
    int c = 0;
#pragma unroll
    for (int step = N / 2; step > 0; step >>= 1)
        if (cum[c + step - 1] <= u) c += step;
    return c + (cum[c] <= u ? 1 : 0);
}

// #{k < n : cum[k] <= u} for any n (binary search)
__device__ __forceinline__ int count_le_n(const float *cum, int n, float u) {
    int c = 0;
    int step = 1;
    while (step * 2 <= n) step *= 2;
    for (; step > 0; step >>= 1)
        if (c + step <= n && cum[c + step - 1] <= u) c += step;
    return c;
}

// Persistent grid: a block takes query after query, copies its prepared
// distributions (both species) to shared memory and its threads take the
// query's draws; KT_ is the tail size when a power of two (the search
// unrolled), else 0 (kt at run time).
template <int KT_>
__global__ void __launch_bounds__(256) count_draw_kernel(const float *P, int Q, int kt, uint64_t seed, float *out,
                                                         int per_query, const float *base) {
    __shared__ float tab[2 * (kNC + 3 * kKTMax)];
    const int KT = KT_ > 0 ? KT_ : kt;
    const int kHS = kNC + 3 * KT;
    for (int q = blockIdx.x; q < Q; q += gridDim.x) {
        __syncthreads();  // every thread is done with the previous query's table
        for (int i = threadIdx.x; i < 2 * kHS; i += blockDim.x) tab[i] = P[(size_t)q * 2 * kHS + i];
        __syncthreads();
        const float b0 = base[2 * q], b1 = base[2 * q + 1];
        for (int d = threadIdx.x; d < per_query; d += blockDim.x) {
            const long long row = (long long)q * per_query + d;
            float v[2];
#pragma unroll
            for (int sp = 0; sp < 2; ++sp) {
                const float *p = tab + sp * kHS;
                uint64_t h = mix64(seed ^ mix64(((uint64_t)row << 1 | (uint64_t)sp) + 0x9E3779B97F4A7C15ull));
                const float u0 = (float)(h >> 40) * 0x1p-24f;
                const int c = min(count_le<kNC>(p, u0), kNC - 1);
                if (c < kNC - 1) {
                    v[sp] = (float)c;
                    continue;
                }
                h = mix64(h);
                const float u1 = (float)(h >> 40) * 0x1p-24f, u2 = ((float)((h >> 16) & 0xFFFFFF) + 0.5f) * 0x1p-24f;
                h = mix64(h);
                const float u3 = (float)(h >> 40) * 0x1p-24f;
                const int t =
                    min(KT_ > 0 ? count_le<(KT_ > 0 ? KT_ : 1)>(p + kNC, u1) : count_le_n(p + kNC, KT, u1), KT - 1);
                const float z = p[kNC + KT + t] + p[kNC + 2 * KT + t] * sqrtf(-2.0f * logf(u2)) * cosf(6.2831853f * u3);
                v[sp] = fmaxf(floorf(expf(z + (sp ? b1 : b0))), (float)(kNC - 1));
            }
            *reinterpret_cast<float2 *>(out + 2 * row) = make_float2(v[0], v[1]);
        }
    }
}

}  // namespace

}  // namespace rbg

extern "C" {

// Count-aware head: loss and gradient, and draws (see count_loss_kernel,
// count_prep_kernel, count_draw_kernel); device pointers; `work` holds the
// prepared distributions, as many floats as O has for the queries drawn from.
int rbg_mdn_count_loss(const float *O, const float *Y, int B, int KT, float *loss, float *G, void *stream) {
    if (KT < 1 || KT > rbg::kKTMax) return (int)cudaErrorInvalidValue;
    rbg::count_loss_kernel<<<(B + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(O, Y, B, KT, loss, G);
    return (int)cudaGetLastError();
}

int rbg_mdn_count_sample(const float *O, int B, int KT, uint64_t seed, float *out, int per_query, const float *base,
                         float *work, void *stream) {
    if (per_query < 1 || !base || !work || KT < 1 || KT > rbg::kKTMax || B < 0) return (int)cudaErrorInvalidValue;
    if (B == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int Q = B / per_query;
    if (B % per_query != 0 || (reinterpret_cast<uintptr_t>(out) & 7) != 0) return (int)cudaErrorInvalidValue;
    rbg::count_prep_kernel<<<(2 * Q + 127) / 128, 128, 0, st>>>(O, Q, KT, work);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::max(1, std::min(Q, 8 * std::max(sms, 1)));
    switch (KT) {
    case 4: rbg::count_draw_kernel<4><<<grid, 256, 0, st>>>(work, Q, KT, seed, out, per_query, base); break;
    case 8: rbg::count_draw_kernel<8><<<grid, 256, 0, st>>>(work, Q, KT, seed, out, per_query, base); break;
    case 16: rbg::count_draw_kernel<16><<<grid, 256, 0, st>>>(work, Q, KT, seed, out, per_query, base); break;
    default: rbg::count_draw_kernel<0><<<grid, 256, 0, st>>>(work, Q, KT, seed, out, per_query, base);
    }
    return (int)cudaGetLastError();
}

// Rate-equation solution at each query (see rre_kernel); device pointers.
int rbg_mdn_rre(const float *rates, const float *tq, int Q, int S, int R, const int *E, const float *N,
                const float *x0, int n_steps, const int *out_idx, int n_out, float *out, void *stream) {
    if (S < 1 || S > rbg::kRreMaxS || R < 1 || R > rbg::kRreMaxR || n_steps < 1) return (int)cudaErrorInvalidValue;
    if (Q == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (S == 4 && R == 5)  // the surrogate's dimer network
        rbg::rre_fixed_kernel<4, 5><<<(Q + 127) / 128, 128, 0, st>>>(rates, tq, Q, E, N, x0, n_steps, out_idx,
                                                                     n_out, out);
    else
        rbg::rre_kernel<<<(Q + 127) / 128, 128, 0, st>>>(rates, tq, Q, S, R, E, N, x0, n_steps, out_idx, n_out, out);
    return (int)cudaGetLastError();
}

// Surrogate kernels (device pointers, the caller's stream).  Internal to the
// Python surrogate module; no counterpart in the reference.
int rbg_mdn_gemm(const void *A, int lda, int ta, const void *B, int ldb, int tb, float *C, int ldc, int M, int N,
                 int K, float beta, void *stream) {
    using namespace rbg;
    const dim3 grid((N + kTileN - 1) / kTileN, (M + kTileM - 1) / kTileM);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto a = static_cast<const __nv_bfloat16 *>(A);
    auto b = static_cast<const __nv_bfloat16 *>(B);
    if (ta && tb) gemm_bf16_kernel<true, true><<<grid, 128, 0, st>>>(a, lda, b, ldb, C, ldc, M, N, K, beta);
    else if (ta) gemm_bf16_kernel<true, false><<<grid, 128, 0, st>>>(a, lda, b, ldb, C, ldc, M, N, K, beta);
    else if (tb) gemm_bf16_kernel<false, true><<<grid, 128, 0, st>>>(a, lda, b, ldb, C, ldc, M, N, K, beta);
    else gemm_bf16_kernel<false, false><<<grid, 128, 0, st>>>(a, lda, b, ldb, C, ldc, M, N, K, beta);
    return (int)cudaGetLastError();
}

namespace {

constexpr int kMaxDevices = 64;

// Dynamic shared memory above 48 KB for `kern`, asked once per (kernel, device):
// the attribute belongs to the current device's context.
cudaError_t opt_in_smem(const void *kern, size_t bytes) {
    static std::mutex mu;
    static std::vector<std::pair<const void *, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    for (const auto &d : done)
        if (d.first == kern && d.second == dev) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done.emplace_back(kern, dev);
    return e;
}

// The TMA-fed kernel takes C = A B^T with both operands K-contiguous, rows
// 16-byte multiples apart from a 16-byte aligned base (what a tensor map can
// address) and K >= 8; RB_GEMM_TMA=0 sends every product to the staged kernel.
bool tma_gemm_ok(const void *A, int lda, int ta, const void *B, int ldb, int tb, int K) {
    const char *e = std::getenv("RB_GEMM_TMA");
    const bool off = e && std::strcmp(e, "0") == 0;
    return !off && !ta && tb && K >= 8 && lda % 8 == 0 && ldb % 8 == 0 &&
           (reinterpret_cast<uintptr_t>(A) & 15) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
}

// 2-D tensor map of a row-major BF16 matrix [rows][K] (row pitch ld elements)
// read in boxes of 64 (K) x box_rows with the 128-byte swizzle; false if the
// driver has no encoder or refuses the operands.
bool encode_rows(CUtensorMap &map, const void *base, int rows, int K, int ld, int box_rows) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }();
    if (!encode) return false;
    const cuuint64_t dim[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t stride[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)rbg::kTmK, (cuuint32_t)box_rows};
    const cuuint32_t elem[2] = {1, 1};
    return encode(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dim, stride, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launch gemm_tma_kernel; returns a CUDA error code, or -1 when no tensor map
// could be made (nothing launched).
int gemm_tma(const void *A, int lda, const void *B, int ldb, float *C, int ldc, int M, int N, int K, float beta,
             int *err, cudaStream_t st) {
    using namespace rbg;
    CUtensorMap ma, mb;
    if (!encode_rows(ma, A, M, K, lda, kTmM) || !encode_rows(mb, B, N, K, ldb, kTmN)) return -1;
    const cudaError_t attr = opt_in_smem(reinterpret_cast<const void *>(gemm_tma_kernel), kTmSmem);
    if (attr != cudaSuccess) return (int)attr;
    const dim3 grid((N + kTmN - 1) / kTmN, (M + kTmM - 1) / kTmM);
    gemm_tma_kernel<<<grid, 128, kTmSmem, st>>>(ma, mb, C, ldc, M, N, K, beta, err);
    return (int)cudaGetLastError();
}

}  // namespace

// The same product on tcgen05 (see gemm_tc05_kernel); *err (device int) is set
// if a completion wait ran out.  K is split over gridDim.z when the product
// has fewer than 64 tiles and K >= 1024; the splits' partial tiles go to a
// workspace this function keeps per device (grown on demand, released at
// exit), so split products on different streams of one device must not
// overlap.
int rbg_mdn_gemm_tc05(const void *A, int lda, int ta, const void *B, int ldb, int tb, float *C, int ldc, int M,
                      int N, int K, float beta, int *err, void *stream) {
    using namespace rbg;
    if (M <= 0 || N <= 0 || K < 0) return (int)cudaErrorInvalidValue;
    const int gx = (N + kTcN - 1) / kTcN, gy = (M + kTcM - 1) / kTcM, round = kTcSlabs * kTcK;
    const int rounds = (K + round - 1) / round;
    int splits = 1;
    if (gx * gy < 64 && K >= 1024) splits = std::max(1, std::min(rounds, 256 / (gx * gy)));
    const int k_split = splits > 1 ? ((rounds + splits - 1) / splits) * round : std::max(K, 1);
    if (splits > 1) splits = (K + k_split - 1) / k_split;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto a = static_cast<const __nv_bfloat16 *>(A);
    auto b = static_cast<const __nv_bfloat16 *>(B);
    if (splits == 1 && tma_gemm_ok(A, lda, ta, B, ldb, tb, K)) {
        const int e = gemm_tma(A, lda, B, ldb, C, ldc, M, N, K, beta, err, st);
        if (e >= 0) return e;  // < 0: no tensor map for these operands; the staged kernel runs
    }
    auto kern = ta && tb ? gemm_tc05_kernel<true, true>
                : ta     ? gemm_tc05_kernel<true, false>
                : tb     ? gemm_tc05_kernel<false, true>
                         : gemm_tc05_kernel<false, false>;
    {
        const cudaError_t e = opt_in_smem(reinterpret_cast<const void *>(kern), kTcSmem);
        if (e != cudaSuccess) return (int)e;
    }
    if (splits == 1) {
        kern<<<dim3(gx, gy, 1), 128, kTcSmem, st>>>(a, lda, b, ldb, C, ldc, M, N, K, k_split, beta, err);
        return (int)cudaGetLastError();
    }
    // the split workspace of the current device (grown on demand)
    static std::mutex mu;
    static float *work[kMaxDevices] = {};
    static size_t work_n[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(mu);
    const size_t need = (size_t)splits * M * N;
    if (need > work_n[dev]) {
        if (work[dev]) cudaFree(work[dev]);  // synchronises the device: no launch still reads the old workspace
        work[dev] = nullptr;
        work_n[dev] = 0;
        cudaError_t e = cudaMalloc(&work[dev], need * sizeof(float));
        if (e != cudaSuccess) return (int)e;
        work_n[dev] = need;
    }
    float *const wk = work[dev];
    kern<<<dim3(gx, gy, splits), 128, kTcSmem, st>>>(a, lda, b, ldb, wk, N, M, N, K, k_split, 0.0f, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    const size_t n = (size_t)M * N;
    split_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(wk, splits, C, ldc, M, N, beta);
    return (int)cudaGetLastError();
}

// The surrogate's whole forward pass in one launch (mlp_infer_kernel): F
// [Q][n_in] raw features (n_in = 8), normalised by x_mean / x_std; W0 [256][8],
// W1..W3 [256][256], W4 [n_out][256] BF16 weights (row-major [out][in]); b0..b4
// FP32 biases; O [Q][n_out] FP32 head outputs.  n_out <= 256 and a multiple of
// 4.  Returns a CUDA error code (cudaErrorInvalidValue for shapes it does not
// cover, cudaErrorNotSupported without a tensor-map encoder).
int rbg_mdn_infer(const float *F, int Q, int n_in, const float *x_mean, const float *x_std, const void *W0,
                  const void *W1, const void *W2, const void *W3, const void *W4, const float *b0, const float *b1,
                  const float *b2, const float *b3, const float *b4, int n_out, float *O, int *err, void *stream) {
    using namespace rbg;
    if (Q < 0 || n_in != 8 || n_out <= 0 || n_out > kInfHid || n_out % 4 != 0) return (int)cudaErrorInvalidValue;
    if (Q == 0) return 0;
    for (const void *w : {W0, W1, W2, W3, W4})
        if (reinterpret_cast<uintptr_t>(w) & 15) return (int)cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(O) & 15) != 0) return (int)cudaErrorInvalidValue;
    const int n_mma = (n_out + 15) & ~15;
    InferMaps maps;
    if (!encode_rows(maps.w[0], W0, kInfHid, n_in, n_in, kInfHid) ||
        !encode_rows(maps.w[1], W1, kInfHid, kInfHid, kInfHid, kInfHid) ||
        !encode_rows(maps.w[2], W2, kInfHid, kInfHid, kInfHid, kInfHid) ||
        !encode_rows(maps.w[3], W3, kInfHid, kInfHid, kInfHid, kInfHid) ||
        !encode_rows(maps.w[4], W4, n_out, kInfHid, kInfHid, n_mma))
        return (int)cudaErrorNotSupported;
    const cudaError_t attr = opt_in_smem(reinterpret_cast<const void *>(mlp_infer_kernel), kInfSmem);
    if (attr != cudaSuccess) return (int)attr;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (Q + 127) / 128;
    const int grid = std::max(1, std::min(tiles, sms));
    mlp_infer_kernel<<<grid, 32 * kInfWarps, kInfSmem, static_cast<cudaStream_t>(stream)>>>(
        maps, F, Q, n_in, x_mean, x_std, b0, b1, b2, b3, b4, n_out, O, err);
    return (int)cudaGetLastError();
}

int rbg_mdn_bias_act(float *Z, const float *b, void *H, int M, int N, int act, void *stream) {
    const size_t n = (size_t)M * N;
    rbg::bias_act_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        Z, b, static_cast<__nv_bfloat16 *>(H), M, N, act);
    return (int)cudaGetLastError();
}

int rbg_mdn_silu_backward(const float *Z, const float *dH, void *dZ, float *db, int M, int N, void *stream) {
    rbg::silu_backward_kernel<<<(N + rbg::kColX - 1) / rbg::kColX, dim3(rbg::kColX, rbg::kColY), 0,
                                static_cast<cudaStream_t>(stream)>>>(
        Z, dH, static_cast<__nv_bfloat16 *>(dZ), db, M, N);
    return (int)cudaGetLastError();
}

int rbg_mdn_head_backward(const float *G, void *Gb, float *db, int M, int N, void *stream) {
    rbg::head_backward_kernel<<<(N + rbg::kColX - 1) / rbg::kColX, dim3(rbg::kColX, rbg::kColY), 0,
                                static_cast<cudaStream_t>(stream)>>>(
        G, static_cast<__nv_bfloat16 *>(Gb), db, M, N);
    return (int)cudaGetLastError();
}

int rbg_mdn_loss(const float *O, const float *Y, int B, int K, float *loss, float *G, void *stream) {
    if (K > 16) return (int)cudaErrorInvalidValue;
    rbg::mdn_loss_kernel<<<(B + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(O, Y, B, K, loss, G);
    return (int)cudaGetLastError();
}

int rbg_mdn_adam(float *w, void *wb, const float *g, float *m, float *v, int n, float lr, float b1, float b2,
                 float eps, int step, void *stream) {
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    rbg::adam_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        w, static_cast<__nv_bfloat16 *>(wb), g, m, v, n, lr, b1, b2, eps, c1, c2);
    return (int)cudaGetLastError();
}

int rbg_mdn_sample(const float *O, int B, int K, uint64_t seed, float *out, int per_query, const float *base,
                   void *stream) {
    if (per_query < 1) return (int)cudaErrorInvalidValue;
    rbg::mdn_sample_kernel<<<(B + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(O, B, K, seed, out,
                                                                                          per_query, base);
    return (int)cudaGetLastError();
}

}  // extern "C"
