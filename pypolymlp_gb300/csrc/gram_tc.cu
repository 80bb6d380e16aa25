// Mixed-precision X^T X on the fifth-generation tensor cores, accurate to the
// Gram of the FP32 rows: fixed-point BF16 slices, tcgen05.mma (kind::f16,
// BF16 x BF16 -> FP32) with exactly representable partial sums in tensor
// memory, and float-float accumulation of the 1,024-row segments.
//
// Why not a plain BF16 split.  The ridge systems of a polynomial MLP are very
// ill-conditioned: after column scaling the Gram of the reference's MgO pair
// fit has lambda_max ~ 1.2e8 while the smallest ridge parameter is 1e-3, so an
// error of order 1e-11 of |X|^T |X| spread over the Gram already makes the
// shifted matrix indefinite (or decides the fit where it does not).  A
// BF16 x 3 split with FP32 accumulation errs by ~1e-5, and even an elementwise
// 6e-8 (FP32 accumulation of exact products) moves the fitted errors far
// beyond 0.05 meV/atom.  What does hold is the Gram of a slightly perturbed X:
// the FP32 rows themselves fit like the FP64 rows.
//
// Scheme (an Ozaki-style splitting).  Rows are taken in segments of 1,024.
// Per (segment, column) e = the exponent with max |x| < 2^e, and
//   x = 2^e (n1 2^-7 + n2 2^-14 + n3 2^-21 + n4 2^-28) + O(2^(e-29)),
// |n1| <= 128, |n2..n4| <= 64 integers; slice k is stored as the BF16 value
// s_k = n_k 2^-7k (exact: at most 8 significant bits) and e beside it, so the
// tensor cores see values of order one whatever the column's magnitude.  The
// Gram of the sliced X is a sum of slice products (i, j) of "level" i + j - 1,
// times 2^(e_a + e_b); per segment
//   A1 = s1^T s1                         (level 1)
//   A2 = s1^T s2 + s2^T s1               (level 2)
//   A3 = s1^T s3 + s3^T s1 + s2^T s2     (level 3)
//   A4 = levels 4 and 5 (7 products)
// accumulate in four FP32 tensor-memory accumulators.  A1 and A2 are exact:
// every product is an integer multiple of 2^-14 (resp. 2^-21) below 2^14
// (resp. 2^14 for the pair) of those units, so 1,024 rows sum to below 2^24
// units, which FP32 holds exactly.  A3 (~2^-15 of A1) and A4
// (~2^-22) round at 2^-24 of themselves per MMA; the dropped levels 6, 7 are
// below 2^-37 of |x_a x_b|.  The segment value (A1 + A2 + (A3 + A4))
// 2^(e_a + e_b) is added to a float-float (~48-bit) running sum per Gram
// element; the row splits are reduced in FP64.  The result is the Gram of X
// quantised to 28 bits of its segment's column maximum, to ~1e-12 of
// |X|^T |X|.  The running sums are FP32 pairs: Gram elements beyond FP32's
// range (|x_a x_b| summed below ~1e-38 or above ~3e38) are not represented;
// columns below ~1e-10 are dropped by the fit's column-scale threshold anyway.
//
// Work unit: (upper 128 x 128 tile, row split).  Block of 320 threads:
//   warp 0      one thread issues the TMA loads of a stage (32 rows of the
//               four slices of tile rows I and of tile columns J, 64-byte
//               swizzle) into a 3-stage ring,
//   warp 1      allocates 512 TMEM columns (four 128-column accumulators)
//               and one thread issues the 26 MMAs of a stage,
//   warps 2-9   drain the accumulators after each segment (tcgen05.ld, two
//               groups of 32 columns per thread), scale the segment by
//               2^(e_a + e_b) and add it to the unit's float-float partial
//               tile; the accumulators are freed for the next segment once
//               the second group is in registers.  (Ten warps leave each
//               of the four SM sub-partitions at most three warps, so at most
//               168 registers a thread: the drain keeps 32 columns at a time.)
// Every wait is bounded (clock64 deadline); a timeout sets an error flag, the
// block stops issuing work, waits (bounded) for what it issued and frees TMEM.
// Partial tiles of the row splits are summed in split order (deterministic).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "async.cuh"
#include "kernels.h"

namespace pg {

constexpr int kTcTile = 128;                          // M = N
constexpr int kTcK = 32;                              // X rows per stage (one 64-byte swizzle row of bf16)
constexpr int kTcStages = 3;
constexpr int kTcSegRows = 1024;                      // rows per exact FP32 segment
constexpr int kTcSegStages = kTcSegRows / kTcK;       // 32
constexpr int kTcSlices = 4;
constexpr int kTcThreads = 320;
constexpr int kTcEpiThreads = 256;
constexpr uint32_t kTcOpBytes = kTcTile * kTcK * 2;   // 8 KB per operand (slice x 128 features x 32 rows)
constexpr uint32_t kTcStageBytes = 2 * kTcSlices * kTcOpBytes;  // 64 KB per stage
constexpr size_t kTcSmem = (size_t)kTcStages * kTcStageBytes + 1024;
constexpr int kTcSplitThreads = 256;                  // pg_split_fx4: 4 rows per thread

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 64-byte swizzle, 8-row
// groups 512 bytes apart (start address and offsets in 16-byte units;
// descriptor version 1 at bit 46; layout type 4 = 64-byte swizzle at bit 61).
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}
// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kIdescBf16M128N128 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcTile >> 3) << 17) | ((uint32_t)(kTcTile >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kIdescBf16M128N128), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 2^k for k in [-126, 127], exactly.
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// a + b = s + e exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// ---------------------------------------------------------------- kernels
// Fixed-point slices of X (FP32, column-major, leading dimension ld) per
// (1,024-row segment, column): S[k] (k = 0..3, each column-major with leading
// dimension ldh, slice k at S + k F ldh) = n_{k+1} 2^(-7 (k+1)) and
// E[segment F + column] = e.  All-zero segments store zeros (e = 0); a
// non-finite value passes into the first slice (e = 0), so that the Gram shows
// it.  Grid: (segments, F); 256 threads x 4 rows.
__global__ void __launch_bounds__(kTcSplitThreads) pg_split_fx4(const float* X, long long ld, long long rows, int F,
                                                                __nv_bfloat16* S, long long ldh, int* E) {
    __shared__ float red[kTcSplitThreads / 32];
    const int c = blockIdx.y;
    const long long r0 = (long long)blockIdx.x * kTcSegRows;
    float x[4];
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long r = r0 + threadIdx.x + q * kTcSplitThreads;
        x[q] = r < rows ? X[(size_t)c * ld + r] : 0.f;
        m = fmaxf(m, fabsf(x[q]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = red[0];
#pragma unroll
    for (int w = 1; w < kTcSplitThreads / 32; ++w) m = fmaxf(m, red[w]);
    int e = 0;
    frexpf(m, &e);  // m = f 2^e, f in [0.5, 1): max |x| < 2^e
    const bool finite = isfinite(m);
    const bool zero = !(m > 0.f) || !finite;
    if (zero) e = 0;
    if (threadIdx.x == 0) E[(size_t)blockIdx.x * F + c] = e;
    const size_t plane = (size_t)F * ldh;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long r = r0 + threadIdx.x + q * kTcSplitThreads;
        if (r >= rows) break;
        // x 2^(7 - e) in [-128, 128], exactly (a power-of-two scaling)
        float u = zero ? 0.f : ldexpf(x[q], 7 - e);
        __nv_bfloat16* o = S + (size_t)c * ldh + r;
#pragma unroll
        for (int k = 0; k < kTcSlices; ++k) {
            const float n = rintf(u);
            u = __fmul_rn(__fsub_rn(u, n), 128.f);
            const float v = zero ? (!finite && k == 0 ? x[q] : 0.f) : __fmul_rn(n, pow2f(-7 * (k + 1)));
            o[k * plane] = __float2bfloat16_rn(v);
        }
    }
}

// Slice products of a K16 step: (I-side slice, J-side slice) of product p;
// p = 0 accumulates into A1, p = 1, 2 into A2, p = 3..5 into A3 and
// p = 6..12 (levels 4, 5) into A4.
constexpr int kTcProducts = 13;
__device__ __forceinline__ constexpr int prod_a(int p) {
    return p == 0 ? 0 : p == 1 ? 0 : p == 2 ? 1 : p == 3 ? 0 : p == 4 ? 2 : p == 5 ? 1 : p == 6 ? 0
         : p == 7 ? 3 : p == 8 ? 1 : p == 9 ? 2 : p == 10 ? 1 : p == 11 ? 3 : 2;
}
__device__ __forceinline__ constexpr int prod_b(int p) {
    return p == 0 ? 0 : p == 1 ? 1 : p == 2 ? 0 : p == 3 ? 2 : p == 4 ? 0 : p == 5 ? 1 : p == 6 ? 3
         : p == 7 ? 0 : p == 8 ? 2 : p == 9 ? 1 : p == 10 ? 3 : p == 11 ? 1 : 2;
}

// units[b] = (tile row block I, tile column block J, row split, 0), I <= J.
// Ph, Pl: per split the float-float partial Gram (F x F, upper tiles).
__global__ void __launch_bounds__(kTcThreads, 1)
    pg_gram_tc(const __grid_constant__ CUtensorMap mapS, const int* E, long long n_rows, int F, const int4* units,
               int n_splits, float* Ph, float* Pl, int* err) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kTcStages], empty_bar[kTcStages], accf_bar, acce_bar, done_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~static_cast<uintptr_t>(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int4 u = units[blockIdx.x];
    const int ti = u.x, tj = u.y, sp = u.z;
    const long long n_seg_all = (n_rows + kTcSegRows - 1) / kTcSegRows;
    const long long per = (n_seg_all + n_splits - 1) / n_splits;
    const long long sb = min(n_seg_all, per * sp), se = min(n_seg_all, sb + per);
    const int nseg = (int)(se - sb);
    // stages of this unit: full segments, the last one possibly shorter
    const long long row_b = sb * kTcSegRows, row_e = min(n_rows, se * kTcSegRows);
    const int nst = nseg > 0 ? (int)((row_e - row_b + kTcK - 1) / kTcK) : 0;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        mbar_init(smem_u32(&accf_bar), 1);
        mbar_init(smem_u32(&acce_bar), kTcEpiThreads);
        mbar_init(smem_u32(&done_bar), 1);
        mbar_init_fence();
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_base;

    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int c = 0; c < nst; ++c) {
                const int s = c % kTcStages;
                const uint32_t k = (uint32_t)(c / kTcStages);
                if (c >= kTcStages && !mbar_wait(smem_u32(&empty_bar[s]), (k - 1) & 1, &abort_flag)) break;
                unsigned char* st = base + (size_t)s * kTcStageBytes;
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, kTcStageBytes);
                const int x = (int)(row_b + (long long)c * kTcK);
#pragma unroll
                for (int q = 0; q < kTcSlices; ++q) {
                    tma_load_3d(smem_u32(st + q * kTcOpBytes), &mapS, x, ti * kTcTile, q, fb);
                    tma_load_3d(smem_u32(st + (kTcSlices + q) * kTcOpBytes), &mapS, x, tj * kTcTile, q, fb);
                }
                issued = c + 1;
            }
            // on an abort, let the loads already issued land before the block exits
            if (abort_flag) {
                volatile int never = 0;
                for (int c = max(0, issued - kTcStages); c < issued; ++c)
                    mbar_wait(smem_u32(&full_bar[c % kTcStages]), (uint32_t)(c / kTcStages) & 1, &never);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            for (int c = 0; c < nst; ++c) {
                const int s = c % kTcStages;
                const uint32_t k = (uint32_t)(c / kTcStages);
                const int seg = c / kTcSegStages;
                const bool first = (c % kTcSegStages) == 0;
                const bool last = (c % kTcSegStages) == kTcSegStages - 1 || c == nst - 1;
                // the epilogue must have read the previous segment's accumulators
                if (first && seg >= 1 && !mbar_wait(smem_u32(&acce_bar), (uint32_t)(seg - 1) & 1, &abort_flag)) break;
                if (!mbar_wait(smem_u32(&full_bar[s]), k & 1, &abort_flag)) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(base + (size_t)s * kTcStageBytes);
                const uint32_t sbj = sa + kTcSlices * kTcOpBytes;
#pragma unroll
                for (int kk = 0; kk < kTcK / 16; ++kk) {
#pragma unroll
                    for (int p = 0; p < kTcProducts; ++p) {
                        const int acc = p == 0 ? 0 : (p < 3 ? 1 : (p < 6 ? 2 : 3));
                        const uint64_t da = sw64_desc(sa + prod_a(p) * kTcOpBytes + kk * 32);
                        const uint64_t db = sw64_desc(sbj + prod_b(p) * kTcOpBytes + kk * 32);
                        const bool init = first && kk == 0 && (p == 0 || p == 1 || p == 3 || p == 6);
                        umma_bf16(tbase + (uint32_t)acc * kTcTile, da, db, init ? 0u : 1u);
                    }
                }
                umma_commit(smem_u32(&empty_bar[s]));
                if (last) umma_commit(smem_u32(&accf_bar));
            }
            // every MMA issued has completed once this barrier flips
            umma_commit(smem_u32(&done_bar));
            volatile int never = 0;
            mbar_wait(smem_u32(&done_bar), 0, &never);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (accumulator rows);
        // warps 2-5 take columns 0-63 of the tile, warps 6-9 columns 64-127
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int m = 32 * q + lane;
        const int gi = ti * kTcTile + m;
        const size_t off = (size_t)sp * F * F;
        float* ph = Ph + off;
        float* pl = Pl + off;
        const uint32_t lane_addr = (uint32_t)(32 * q) << 16;
        for (int seg = 0; seg < nseg; ++seg) {
            // the warp leaves together, so tcgen05.ld below always runs on a full warp
            const bool ok = mbar_wait(smem_u32(&accf_bar), (uint32_t)seg & 1, &abort_flag);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
            const int* Es = E + (size_t)(sb + seg) * F;
            const int ea = gi < F ? Es[gi] : 0;
            // two groups of 32 columns; the accumulators are released once the
            // second group is in registers, before its partial-tile update
#pragma unroll 1
            for (int cc = 0; cc < 2; ++cc) {
                const uint32_t col = (uint32_t)(half * 64 + cc * 32);
                float sv[32], tv[32];
                {
                    uint32_t r1[32], r2[32];
                    tmem_ld_32x32b_x32(tbase + col + lane_addr, r1);
                    tmem_ld_32x32b_x32(tbase + kTcTile + col + lane_addr, r2);
#pragma unroll
                    for (int k2 = 0; k2 < 32; ++k2) two_sum(__uint_as_float(r1[k2]), __uint_as_float(r2[k2]), sv[k2], tv[k2]);
                    tmem_ld_32x32b_x32(tbase + 2 * kTcTile + col + lane_addr, r1);
                    tmem_ld_32x32b_x32(tbase + 3 * kTcTile + col + lane_addr, r2);
#pragma unroll
                    for (int k2 = 0; k2 < 32; ++k2)
                        tv[k2] = __fadd_rn(tv[k2], __fadd_rn(__uint_as_float(r1[k2]), __uint_as_float(r2[k2])));
                }
                if (cc == 1) {
                    // accumulators read: the next segment's MMAs may start
                    tc_fence_before();
                    mbar_arrive(smem_u32(&acce_bar));
                }
                if (gi < F) {
                    // eight columns at a time: their partial sums are loaded
                    // together (one L2 round trip), then updated and stored
#pragma unroll
                    for (int k0 = 0; k0 < 32; k0 += 8) {
                        float oh[8], ol[8];
                        int ex[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int gj = tj * kTcTile + (int)col + k0 + u;
                            const bool in = gj < F && gi <= gj;
                            const size_t idx = (size_t)gj * F + gi;
                            ex[u] = in ? __ldg(Es + gj) : 0;
                            oh[u] = (in && seg > 0) ? __ldcg(ph + idx) : 0.f;
                            ol[u] = (in && seg > 0) ? __ldcg(pl + idx) : 0.f;
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int gj = tj * kTcTile + (int)col + k0 + u;
                            if (gj < F && gi <= gj) {
                                const size_t idx = (size_t)gj * F + gi;
                                const int k = ea + ex[u];
                                const float sa = ldexpf(sv[k0 + u], k), ta = ldexpf(tv[k0 + u], k);
                                float x, y;
                                two_sum(oh[u], sa, x, y);
                                y = __fadd_rn(y, __fadd_rn(ol[u], ta));
                                const float h = __fadd_rn(x, y);
                                __stcg(ph + idx, h);
                                __stcg(pl + idx, __fsub_rn(y, __fsub_rn(h, x)));
                            }
                        }
                    }
                }
            }
        }
        if (nseg == 0 && gi < F)
            for (int k2 = 0; k2 < 64; ++k2) {
                const int gj = tj * kTcTile + half * 64 + k2;
                if (gj < F && gi <= gj) {
                    ph[(size_t)gj * F + gi] = 0.f;
                    pl[(size_t)gj * F + gi] = 0.f;
                }
            }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(512) : "memory");
    }
    if (threadIdx.x == 0 && abort_flag) atomicExch(err, 1);
}

// G[j F + i] += sum over splits of (Ph_s + Pl_s)[j F + i], i <= j, in split order.
__global__ void pg_gram_tc_reduce(const float* Ph, const float* Pl, int n_splits, int F, double* G) {
    const int j = blockIdx.y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= j && i < F; i += gridDim.x * blockDim.x) {
        const size_t idx = (size_t)j * F + i;
        double s = 0.0;
        for (int p = 0; p < n_splits; ++p) {
            const size_t q = (size_t)p * F * F + idx;
            s += (double)Ph[q] + (double)Pl[q];
        }
        G[idx] += s;
    }
}

// ---------------------------------------------------------------- host
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

// The four slice planes as one 3-D tensor (rows, F, slice), boxes of 32 rows x 128 features.
CUtensorMap make_map(const __nv_bfloat16* base, long long rows, int F, long long ldh) {
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)rows, (cuuint64_t)F, (cuuint64_t)kTcSlices};
    const cuuint64_t strides[2] = {(cuuint64_t)ldh * 2, (cuuint64_t)ldh * F * 2};
    const cuuint32_t box[3] = {(cuuint32_t)kTcK, (cuuint32_t)kTcTile, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(base), dims,
                                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed");
    return m;
}

}  // namespace

// G (F x F FP64, upper triangle column-major) += X^T X for X FP32 column-major
// (rows x F, leading dimension ld), on the tensor cores.
void gram_tc_accumulate(const float* X, long long ld, long long rows, int F, double* G, GramTcScratch& S,
                        cudaStream_t st) {
    if (rows <= 0) return;
    if (F > 65535) throw std::runtime_error("too many features for the tensor-core Gram");
    if (rows > (1LL << 31) - kTcSegRows) throw std::runtime_error("too many rows for one tensor-core Gram call");
    const long long ldh = (rows + 7) / 8 * 8;  // TMA strides are multiples of 16 bytes
    const long long n_seg = (rows + kTcSegRows - 1) / kTcSegRows;
    S.H.reserve((size_t)ldh * F * kTcSlices * 2);
    S.E.reserve((size_t)n_seg * F * sizeof(int));
    if (S.err.bytes() == 0) {  // cumulative until gram_tc_check reads it
        S.err.alloc(sizeof(int));
        zero_async(S.err.as<void>(), sizeof(int));
    }
    // work units: upper tiles x row splits, split-major (tiles of one split share rows in L2)
    if (S.F != F || S.rows != rows) {
        int dev = 0, sms = 148;
        PG_CUDA(cudaGetDevice(&dev));
        PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int nt = (F + kTcTile - 1) / kTcTile;
        const int n_tiles = nt * (nt + 1) / 2;
        const long long segs = (rows + kTcSegRows - 1) / kTcSegRows;
        int best = 1;
        double best_eff = 0.0;
        for (int s = 1; s <= 8; ++s) {
            if (s > 1 && segs / s < 2) break;
            const long long n = (long long)n_tiles * s;
            const double eff = (double)n / (double)(((n + sms - 1) / sms) * sms);
            if (eff > best_eff + 0.02) {
                best_eff = eff;
                best = s;
            }
        }
        std::vector<int4> u;
        for (int s = 0; s < best; ++s)
            for (int j = 0; j < nt; ++j)
                for (int i = 0; i <= j; ++i) u.push_back(make_int4(i, j, s, 0));
        upload(S.units, u);
        S.n_units = (int)u.size();
        S.n_splits = best;
        S.F = F;
        S.rows = rows;
        S.P.reserve((size_t)best * F * F * 2 * sizeof(float));
    }
    auto* Sl = S.H.as<__nv_bfloat16>();
    {
        dim3 grid((unsigned)((rows + kTcSegRows - 1) / kTcSegRows), (unsigned)F);
        pg_split_fx4<<<grid, kTcSplitThreads, 0, st>>>(X, ld, rows, F, Sl, ldh, S.E.as<int>());
    }
    const CUtensorMap ms = make_map(Sl, rows, F, ldh);
    float* Ph = S.P.as<float>();
    float* Pl = Ph + (size_t)S.n_splits * F * F;
    PG_CUDA(cudaFuncSetAttribute(pg_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    pg_gram_tc<<<S.n_units, kTcThreads, kTcSmem, st>>>(ms, S.E.as<int>(), rows, F, S.units.as<int4>(), S.n_splits,
                                                       Ph, Pl, S.err.as<int>());
    dim3 rg((unsigned)((F + 255) / 256), (unsigned)F);
    pg_gram_tc_reduce<<<rg, 256, 0, st>>>(Ph, Pl, S.n_splits, F, G);
    PG_CUDA(cudaGetLastError());
}

// Status of the last tensor-core Gram launches (after the stream has synchronised).
void gram_tc_check(GramTcScratch& S) {
    if (S.err.bytes() == 0) return;
    int e = 0;
    copy_d2h(&e, S.err.as<int>(), sizeof(int));
    if (e) {
        zero_async(S.err.as<void>(), sizeof(int));
        throw std::runtime_error("tensor-core Gram timed out waiting on its pipeline");
    }
}

}  // namespace pg
