// Mixed-precision X^T X on the fifth-generation tensor cores: TMA loads into
// 128-byte-swizzled shared memory, tcgen05.mma (kind::f16, BF16 x BF16 -> FP32)
// accumulating in tensor memory, FP32 segments flushed into FP64.
//
// X (FP32, column-major, one column per feature) is split into BF16 hi and lo
// parts (x = hi + lo + O(2^-16 x)); each upper 128 x 128 tile (I, J) of the Gram
// accumulates hi_I^T hi_J + hi_I^T lo_J + lo_I^T hi_J over the rows, so the
// products carry ~16 significant bits per operand, as the reference's
// X^T X (data_sequential.py:145-152) in FP64 is approximated in the mixed path.
//
// Work unit: (tile, row split).  Block of 192 threads:
//   warp 0      one thread issues the TMA loads of a 4-operand stage
//               (A_hi, A_lo of tile rows I, B_hi, B_lo of tile columns J;
//               64 X rows x 128 features each) into a 3-stage ring,
//   warp 1      allocates 256 TMEM columns (two 128 x 128 FP32 accumulators)
//               and one thread issues the 12 MMAs of a stage,
//   warps 2-5   drain an accumulator every 4,096 rows (tcgen05.ld) into the
//               unit's FP64 partial tile while the MMAs fill the other one.
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

#include "kernels.h"

namespace pg {

constexpr int kTcTile = 128;                          // M = N
constexpr int kTcK = 64;                              // X rows per stage (one 128-byte swizzle atom of bf16)
constexpr int kTcStages = 3;
constexpr int kTcSegChunks = 64;                      // stages per FP32 segment (4,096 rows)
constexpr int kTcThreads = 192;
constexpr uint32_t kTcOpBytes = kTcTile * kTcK * 2;   // 16 KB per operand
constexpr uint32_t kTcStageBytes = 4 * kTcOpBytes;    // 64 KB per stage
constexpr long long kTcWaitCycles = 4000000000LL;     // about 2 s at 2 GHz
constexpr size_t kTcSmem = (size_t)kTcStages * kTcStageBytes + 1024;

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase of the given parity; false on abort or after the deadline.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile int* abort_flag) {
    const long long t0 = clock64();
    while (!mbar_try(a, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kTcWaitCycles) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1,024 bytes apart (start address and offsets in 16-byte units;
// descriptor version 1 at bit 46; layout type 2 = 128-byte swizzle at bit 61).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
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

// ---------------------------------------------------------------- kernels
// hi = bf16(x), lo = bf16(x - hi); H, L column-major with leading dimension ldh.
__global__ void pg_split_bf16(const float* X, long long ld, long long rows, __nv_bfloat16* H, __nv_bfloat16* L,
                              long long ldh) {
    const long long c = blockIdx.y;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
         r += (long long)gridDim.x * blockDim.x) {
        const float x = X[c * ld + r];
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        H[c * ldh + r] = h;
        L[c * ldh + r] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
}

// units[b] = (tile row block I, tile column block J, row split, 0), I <= J.
__global__ void __launch_bounds__(kTcThreads, 1)
    pg_gram_tc(const __grid_constant__ CUtensorMap mapH, const __grid_constant__ CUtensorMap mapL, long long n_rows,
               int F, const int4* units, int n_splits, double* P, int* err) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[kTcStages], empty_bar[kTcStages], accf_bar[2], acce_bar[2], done_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~static_cast<uintptr_t>(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int4 u = units[blockIdx.x];
    const int ti = u.x, tj = u.y, sp = u.z;
    const long long n_chunks_all = (n_rows + kTcK - 1) / kTcK;
    const long long per = (n_chunks_all + n_splits - 1) / n_splits;
    const long long cb = min(n_chunks_all, per * sp), ce = min(n_chunks_all, cb + per);
    const int nch = (int)(ce - cb);
    const int nseg = (nch + kTcSegChunks - 1) / kTcSegChunks;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&accf_bar[b]), 1);
            mbar_init(smem_u32(&acce_bar[b]), 128);
        }
        mbar_init(smem_u32(&done_bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(256)
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
            for (int c = 0; c < nch; ++c) {
                const int s = c % kTcStages;
                const uint32_t k = (uint32_t)(c / kTcStages);
                if (c >= kTcStages && !mbar_wait(smem_u32(&empty_bar[s]), (k - 1) & 1, &abort_flag)) break;
                unsigned char* st = base + (size_t)s * kTcStageBytes;
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, kTcStageBytes);
                const int x = (int)((cb + c) * kTcK);
                tma_load_2d(smem_u32(st), &mapH, x, ti * kTcTile, fb);
                tma_load_2d(smem_u32(st + kTcOpBytes), &mapL, x, ti * kTcTile, fb);
                tma_load_2d(smem_u32(st + 2 * kTcOpBytes), &mapH, x, tj * kTcTile, fb);
                tma_load_2d(smem_u32(st + 3 * kTcOpBytes), &mapL, x, tj * kTcTile, fb);
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
            for (int c = 0; c < nch; ++c) {
                const int s = c % kTcStages;
                const uint32_t k = (uint32_t)(c / kTcStages);
                const int seg = c / kTcSegChunks, b = seg & 1;
                const bool first = (c % kTcSegChunks) == 0;
                if (first && seg >= 2 && !mbar_wait(smem_u32(&acce_bar[b]), (uint32_t)((seg >> 1) - 1) & 1, &abort_flag))
                    break;
                if (!mbar_wait(smem_u32(&full_bar[s]), k & 1, &abort_flag)) break;
                tc_fence_after();
                const uint32_t d = tbase + (uint32_t)b * kTcTile;
                const uint32_t st = smem_u32(base + (size_t)s * kTcStageBytes);
#pragma unroll
                for (int kk = 0; kk < kTcK / 16; ++kk) {
                    const uint64_t ah = sw128_desc(st + kk * 32);
                    const uint64_t al = sw128_desc(st + kTcOpBytes + kk * 32);
                    const uint64_t bh = sw128_desc(st + 2 * kTcOpBytes + kk * 32);
                    const uint64_t bl = sw128_desc(st + 3 * kTcOpBytes + kk * 32);
                    umma_bf16(d, ah, bh, (first && kk == 0) ? 0u : 1u);
                    umma_bf16(d, ah, bl, 1u);
                    umma_bf16(d, al, bh, 1u);
                }
                umma_commit(smem_u32(&empty_bar[s]));
                if ((c % kTcSegChunks) == kTcSegChunks - 1 || c == nch - 1) umma_commit(smem_u32(&accf_bar[b]));
            }
            // every MMA issued has completed once this barrier flips
            umma_commit(smem_u32(&done_bar));
            volatile int never = 0;
            mbar_wait(smem_u32(&done_bar), 0, &never);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 = accumulator rows
        const int q = warp & 3;
        const int m = 32 * q + lane;
        const int gi = ti * kTcTile + m;
        double* Ps = P + (size_t)sp * F * F;
        for (int seg = 0; seg < nseg; ++seg) {
            const int b = seg & 1;
            // the warp leaves together, so tcgen05.ld below always runs on a full warp
            const bool ok = mbar_wait(smem_u32(&accf_bar[b]), (uint32_t)(seg >> 1) & 1, &abort_flag);
            if (!__all_sync(0xffffffffu, ok)) break;
            tc_fence_after();
#pragma unroll 1
            for (int cc = 0; cc < kTcTile / 32; ++cc) {
                uint32_t r[32];
                tmem_ld_32x32b_x32(tbase + (uint32_t)b * kTcTile + (uint32_t)cc * 32 + ((uint32_t)(32 * q) << 16), r);
#pragma unroll
                for (int k2 = 0; k2 < 32; ++k2) {
                    const int gj = tj * kTcTile + cc * 32 + k2;
                    if (gi < F && gj < F && gi <= gj) {
                        double* o = Ps + (size_t)gj * F + gi;
                        const double v = (double)__uint_as_float(r[k2]);
                        *o = seg == 0 ? v : *o + v;
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(smem_u32(&acce_bar[b]));
        }
        if (nseg == 0 && gi < F)
            for (int k2 = 0; k2 < kTcTile; ++k2) {
                const int gj = tj * kTcTile + k2;
                if (gj < F && gi <= gj) Ps[(size_t)gj * F + gi] = 0.0;
            }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        __syncwarp();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(256) : "memory");
    }
    if (threadIdx.x == 0 && abort_flag) atomicExch(err, 1);
}

// G[j F + i] += sum over splits of P_s[j F + i], i <= j, in split order.
__global__ void pg_gram_tc_reduce(const double* P, int n_splits, int F, double* G) {
    const int j = blockIdx.y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= j && i < F; i += gridDim.x * blockDim.x) {
        const size_t idx = (size_t)j * F + i;
        double s = 0.0;
        for (int p = 0; p < n_splits; ++p) s += P[(size_t)p * F * F + idx];
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

CUtensorMap make_map(const __nv_bfloat16* base, long long rows, int F, long long ldh) {
    CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)F};
    const cuuint64_t strides[1] = {(cuuint64_t)ldh * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)kTcTile};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims,
                                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
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
    const long long ldh = (rows + 7) / 8 * 8;  // TMA strides are multiples of 16 bytes
    S.H.reserve((size_t)ldh * F * 2);
    S.L.reserve((size_t)ldh * F * 2);
    if (S.err.bytes() == 0) {  // cumulative until gram_tc_check reads it
        S.err.alloc(sizeof(int));
        PG_CUDA(cudaMemset(S.err.as<void>(), 0, sizeof(int)));
    }
    // work units: upper tiles x row splits, split-major (tiles of one split share rows in L2)
    if (S.F != F || S.rows != rows) {
        int dev = 0, sms = 148;
        PG_CUDA(cudaGetDevice(&dev));
        PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int nt = (F + kTcTile - 1) / kTcTile;
        const int n_tiles = nt * (nt + 1) / 2;
        const long long chunks = (rows + kTcK - 1) / kTcK;
        int best = 1;
        double best_eff = 0.0;
        for (int s = 1; s <= 8; ++s) {
            if (s > 1 && chunks / s < 2 * kTcSegChunks) break;
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
        S.P.reserve((size_t)best * F * F * sizeof(double));
    }
    auto* H = S.H.as<__nv_bfloat16>();
    auto* L = S.L.as<__nv_bfloat16>();
    {
        dim3 grid((unsigned)std::min<long long>((rows + 255) / 256, 64), (unsigned)F);
        pg_split_bf16<<<grid, 256, 0, st>>>(X, ld, rows, H, L, ldh);
    }
    const CUtensorMap mh = make_map(H, rows, F, ldh), ml = make_map(L, rows, F, ldh);
    PG_CUDA(cudaFuncSetAttribute(pg_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    pg_gram_tc<<<S.n_units, kTcThreads, kTcSmem, st>>>(mh, ml, rows, F, S.units.as<int4>(), S.n_splits,
                                                       S.P.as<double>(), S.err.as<int>());
    dim3 rg((unsigned)((F + 255) / 256), (unsigned)F);
    pg_gram_tc_reduce<<<rg, 256, 0, st>>>(S.P.as<double>(), S.n_splits, F, G);
    PG_CUDA(cudaGetLastError());
}

// Status of the last tensor-core Gram launches (after the stream has synchronised).
void gram_tc_check(GramTcScratch& S) {
    if (S.err.bytes() == 0) return;
    int e = 0;
    PG_CUDA(cudaMemcpy(&e, S.err.as<int>(), sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        PG_CUDA(cudaMemset(S.err.as<void>(), 0, sizeof(int)));
        throw std::runtime_error("tensor-core Gram timed out waiting on its pipeline");
    }
}

}  // namespace pg
