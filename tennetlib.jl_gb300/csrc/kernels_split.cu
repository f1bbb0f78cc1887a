// Split-precision grouped GEMM on the 5th-generation tensor cores (tcgen05, sm_103a):
// FP64 operands are cut into bf16 slices (Ozaki scheme I: Ozaki, Ogita, Oishi & Rump,
// Numer. Algorithms 59, 2012) whose pairwise products are exact in the FP32 tensor-core
// accumulator; the partial sums are combined in double-float registers and rescaled to
// FP64, so the result carries ~8*s+1 significant bits per operand element.
//
//  * pack kernel: for every row of op(A) (every column of op(B)) a power-of-two exponent
//    E with max|x| < 2^E; x * 2^(8s-E) rounded to an integer X (|X| <= 2^(8s)) is written
//    as balanced base-256 digits d_1..d_s (|d_1| <= 256, |d_i| <= 128), stored as the
//    bf16 values d_i * 2^(-8(i-1)) in the canonical UMMA K-major SWIZZLE_128B tile layout
//    (8-row x 128-byte atoms, 16-byte chunks XOR-ed with the row index), one contiguous
//    tile per (row tile, k tile, slice), so that a 1D bulk copy moves it to shared memory;
//  * MMA kernel: persistent, one CTA per SM, warp-specialised (warp 0 producer, warp 1
//    MMA issuer + TMEM owner, warps 2-9 epilogue: lane quadrant warp % 4, column half
//    (warp - 2) / 4).  For each 128 x 64 output tile and each
//    k tile the slice pairs (i, j) with i + j <= s + 1 are multiplied into four TMEM
//    accumulators: level 2, 3, 4 (exact: integer multiples of 2^-8(l-2) below 2^24 for a
//    chunk of 128 k) and levels >= 5 (scaled, rounded far below the result's precision).
//    Every chunk of two k tiles the epilogue drains the accumulators (double-buffered in
//    TMEM) into (hi, lo) FP32 pairs with error-free additions; at the end of the tile the
//    pair is rescaled by 2^(E_row + E_col - 16) in FP64 and stored.
// Every mbarrier wait is bounded (about one second); a wait that gives up sets the error
// word, and all roles then drain with bounded waits, free TMEM and return.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "tn_internal.h"

namespace tn {
namespace {

constexpr int BM = 128;            // rows of an output tile (UMMA M)
constexpr int BN = 64;             // columns of an output tile (UMMA N)
constexpr int BKT = 64;            // k elements per tile (one 128-byte swizzle row of bf16)
constexpr int A_TILE = BM * BKT * 2;   // 16 KB
constexpr int B_TILE = BN * BKT * 2;   // 8 KB
constexpr int STAGE = A_TILE + B_TILE; // 24 KB
constexpr int NST = 8;             // ring stages (192 KB)
constexpr int KC = 2;              // k tiles per exact accumulation chunk
constexpr int NACC = 4;            // accumulators: level 2, 3, 4, >= 5
constexpr int TMEM_COLS = 512;     // 2 buffers x 4 accumulators x 64 columns
constexpr int THREADS = 320;       // 10 warps: producer, MMA, 8 epilogue
constexpr long long WAIT_LIMIT = 2000000000LL;  // clock cycles (about one second)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait.  Returns false (and sets *err) when the limit passes or an error is
// already flagged.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err,
                                          volatile int* shared_err) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try(bar, parity)) return true;
        if (*shared_err) return false;
        if (clock64() - t0 > WAIT_LIMIT) {
            *shared_err = 1;
            atomicExch(err, 1);
            return false;
        }
    }
}

// Bounded wait used only to drain before exit (no error bookkeeping).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > WAIT_LIMIT) return;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// K-major SWIZZLE_128B shared-memory matrix descriptor (start address, LBO = 16 B,
// SBO = 1024 B between 8-row groups, descriptor version 1, layout type 2 = 128B swizzle).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);
    d |= uint64_t(1) << 16;
    d |= uint64_t(1024 >> 4) << 32;
    d |= uint64_t(1) << 46;
    d |= uint64_t(2) << 61;
    return d;
}

// Instruction descriptor of kind::f16: D = F32, A = B = BF16, both K-major, N = 64, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// error-free addition of a into (hi, lo) (Knuth's TwoSum, lo collects the rounding errors)
__device__ __forceinline__ void df_add(float& hi, float& lo, float a) {
    const float s = hi + a;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (a - bp);
    hi = s;
    lo += e;
}

__device__ __forceinline__ double pow2(int e) {
    return __longlong_as_double(static_cast<long long>(1023 + e) << 52);
}

// ------------------------------------------------------------------------------------
// pack kernel: a row tile (128 rows for A, 64 for B) is shared by tile_rows / PACK_ROWS CTAs
// (gridDim.y), each packing all k tiles of its PACK_ROWS rows: the row maxima stay within a
// CTA, and small operands still spread over many SMs
// ------------------------------------------------------------------------------------
constexpr int PACK_THREADS = 256;
constexpr int PACK_ROWS = 32;

// Work item of the pack kernel: row r of the tile and one 8-wide chunk (16 bytes of bf16)
// of one k tile; consecutive threads take consecutive rows so that the loads of a column-
// major operand coalesce, and each thread keeps 8 independent loads in flight.
__global__ void __launch_bounds__(PACK_THREADS)
split_pack_kernel(const PackJob* __restrict__ jobs, const KTileSrc* __restrict__ ksrc, Bases b,
                  uint8_t* __restrict__ out, int* __restrict__ expo, int slices, int tile_rows) {
    __shared__ unsigned long long rowmax[PACK_ROWS];
    const PackJob jb = jobs[blockIdx.x];
    const int r0 = blockIdx.y * PACK_ROWS;
    const int nr = (tile_rows - r0) < PACK_ROWS ? (tile_rows - r0) : PACK_ROWS;
    if (nr <= 0) return;
    const int tile_bytes = tile_rows * BKT * 2;
    const int per_tile = nr * 8;                    // (row, chunk) items per k tile
    const int nitems = per_tile * jb.nkt;
    for (int r = threadIdx.x; r < nr; r += blockDim.x) rowmax[r] = 0ull;
    __syncthreads();
    // pass 1: row maxima of |x| as IEEE bit patterns (integer compare, no FP64 pipe)
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
        const int t = it / per_tile, rem = it % per_tile;
        const int rl = rem % nr, ch = rem / nr, r = r0 + rl;
        if (r >= jb.rows) continue;
        const KTileSrc ks = ksrc[jb.kt0 + t];
        const long long* x = reinterpret_cast<const long long*>(b.p[ks.buf] + ks.off) +
                             int64_t(jb.row0 + r) * ks.sr;
        unsigned long long mx = 0ull;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = ch * 8 + q;
            if (k < ks.kvalid) {
                const unsigned long long v = (unsigned long long)(x[int64_t(k) * ks.sk]) & 0x7fffffffffffffffull;
                mx = v > mx ? v : mx;
            }
        }
        if (mx) atomicMax(&rowmax[rl], mx);
    }
    __syncthreads();
    for (int rl = threadIdx.x; rl < nr && r0 + rl < jb.rows; rl += blockDim.x) {
        const unsigned long long m = rowmax[rl];
        expo[jb.eoff + r0 + rl] = m ? int((m >> 52) & 0x7ff) - 1022 : 0;
    }
    // pass 2: balanced base-256 digits.  x * 2^(8s - E) = sig * 2^(ex - 1075 + 8s - E), sig
    // the 53-bit significand: the rounded integer is sig shifted right by
    // sh = 1075 + E - 8s - ex (round half away from zero), integer pipe only.
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
        const int t = it / per_tile, rem = it % per_tile;
        const int rl = rem % nr, ch = rem / nr, r = r0 + rl;
        const KTileSrc ks = ksrc[jb.kt0 + t];
        const bool live = r < jb.rows && ks.kvalid > 0;
        const unsigned long long mxb = live ? rowmax[rl] : 0ull;
        const int E = mxb ? int((mxb >> 52) & 0x7ff) - 1022 : 0;
        const int base_sh = 1075 + E - 8 * slices;
        const long long* x = live ? reinterpret_cast<const long long*>(b.p[ks.buf] + ks.off) +
                                        int64_t(jb.row0 + r) * ks.sr
                                  : nullptr;
        __nv_bfloat16 dig[7][8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = ch * 8 + q;
            long long X = 0;
            if (mxb && k < ks.kvalid) {
                const long long v = x[int64_t(k) * ks.sk];
                const int ex = int((v >> 52) & 0x7ff);
                if (ex) {  // subnormals are far below the row scale: they round to 0
                    const long long m = (v & 0xfffffffffffffLL) | (1LL << 52);
                    const int sh = base_sh - ex;
                    long long a = 0;
                    if (sh <= 0) a = m << (-sh);
                    else if (sh < 63) a = (m + (1LL << (sh - 1))) >> sh;
                    X = v < 0 ? -a : a;
                }
            }
            // compile-time slice indices keep dig[][] in registers
#pragma unroll
            for (int i = 6; i >= 1; --i) {
                if (i >= slices) continue;
                int d = int(X & 255);
                if (d > 128) d -= 256;
                X = (X - d) >> 8;
                dig[i][q] = __float2bfloat16_rn(ldexpf(float(d), -8 * i));
            }
            dig[0][q] = __float2bfloat16_rn(float(X));
        }
        // swizzled position of (row r, chunk ch): 8-row atoms of 1024 bytes
        uint8_t* tile0 = out + jb.out_off + int64_t(t) * slices * tile_bytes;
        const int off = (r >> 3) * 1024 + (r & 7) * 128 + ((ch ^ (r & 7)) << 4);
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            if (i >= slices) continue;
            uint4 v;
            __builtin_memcpy(&v, dig[i], 16);
            *reinterpret_cast<uint4*>(tile0 + int64_t(i) * tile_bytes + off) = v;
        }
    }
}

// k-split pack for operands with long k: the k tiles of every job are divided among
// gridDim.y CTAs (kper tiles each).  Pass 1 (split_rowmax_kernel) folds each row's max |x|
// (IEEE bit pattern, an exact and order-independent maximum) into gmax with atomicMax;
// pass 2 (split_pack_part_kernel) writes the digits of its k tiles with the exponents taken
// from gmax.  Same digits as split_pack_kernel, many more CTAs.
__global__ void __launch_bounds__(PACK_THREADS)
split_rowmax_kernel(const PackJob* __restrict__ jobs, const KTileSrc* __restrict__ ksrc, Bases b,
                    unsigned long long* __restrict__ gmax, int tile_rows, int kper) {
    __shared__ unsigned long long rowmax[BM];
    const PackJob jb = jobs[blockIdx.x];
    const int t0 = blockIdx.y * kper;
    if (t0 >= jb.nkt) return;
    const int t1 = (t0 + kper) < jb.nkt ? (t0 + kper) : jb.nkt;
    const int per_tile = tile_rows * 8;
    const int nitems = per_tile * (t1 - t0);
    for (int r = threadIdx.x; r < tile_rows; r += blockDim.x) rowmax[r] = 0ull;
    __syncthreads();
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
        const int t = t0 + it / per_tile, rem = it % per_tile;
        const int r = rem % tile_rows, ch = rem / tile_rows;
        if (r >= jb.rows) continue;
        const KTileSrc ks = ksrc[jb.kt0 + t];
        const long long* x = reinterpret_cast<const long long*>(b.p[ks.buf] + ks.off) +
                             int64_t(jb.row0 + r) * ks.sr;
        unsigned long long mx = 0ull;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = ch * 8 + q;
            if (k < ks.kvalid) {
                const unsigned long long v = (unsigned long long)(x[int64_t(k) * ks.sk]) & 0x7fffffffffffffffull;
                mx = v > mx ? v : mx;
            }
        }
        if (mx) atomicMax(&rowmax[r], mx);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < jb.rows; r += blockDim.x)
        if (rowmax[r]) atomicMax(&gmax[jb.eoff + r], rowmax[r]);
}

__global__ void __launch_bounds__(PACK_THREADS)
split_pack_part_kernel(const PackJob* __restrict__ jobs, const KTileSrc* __restrict__ ksrc, Bases b,
                       uint8_t* __restrict__ out, int* __restrict__ expo,
                       const unsigned long long* __restrict__ gmax, int slices, int tile_rows,
                       int kper) {
    const PackJob jb = jobs[blockIdx.x];
    const int t0 = blockIdx.y * kper;
    if (t0 >= jb.nkt) return;
    const int t1 = (t0 + kper) < jb.nkt ? (t0 + kper) : jb.nkt;
    const int tile_bytes = tile_rows * BKT * 2;
    const int per_tile = tile_rows * 8;
    const int nitems = per_tile * (t1 - t0);
    if (blockIdx.y == 0)
        for (int r = threadIdx.x; r < jb.rows; r += blockDim.x) {
            const unsigned long long m = gmax[jb.eoff + r];
            expo[jb.eoff + r] = m ? int((m >> 52) & 0x7ff) - 1022 : 0;
        }
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
        const int t = t0 + it / per_tile, rem = it % per_tile;
        const int r = rem % tile_rows, ch = rem / tile_rows;
        const KTileSrc ks = ksrc[jb.kt0 + t];
        const bool live = r < jb.rows && ks.kvalid > 0;
        const unsigned long long mxb = live ? gmax[jb.eoff + r] : 0ull;
        const int E = mxb ? int((mxb >> 52) & 0x7ff) - 1022 : 0;
        const int base_sh = 1075 + E - 8 * slices;
        const long long* x = live ? reinterpret_cast<const long long*>(b.p[ks.buf] + ks.off) +
                                        int64_t(jb.row0 + r) * ks.sr
                                  : nullptr;
        __nv_bfloat16 dig[7][8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int k = ch * 8 + q;
            long long X = 0;
            if (mxb && k < ks.kvalid) {
                const long long v = x[int64_t(k) * ks.sk];
                const int ex = int((v >> 52) & 0x7ff);
                if (ex) {
                    const long long m = (v & 0xfffffffffffffLL) | (1LL << 52);
                    const int sh = base_sh - ex;
                    long long a = 0;
                    if (sh <= 0) a = m << (-sh);
                    else if (sh < 63) a = (m + (1LL << (sh - 1))) >> sh;
                    X = v < 0 ? -a : a;
                }
            }
            // compile-time slice indices keep dig[][] in registers
#pragma unroll
            for (int i = 6; i >= 1; --i) {
                if (i >= slices) continue;
                int d = int(X & 255);
                if (d > 128) d -= 256;
                X = (X - d) >> 8;
                dig[i][q] = __float2bfloat16_rn(ldexpf(float(d), -8 * i));
            }
            dig[0][q] = __float2bfloat16_rn(float(X));
        }
        uint8_t* tile0 = out + jb.out_off + int64_t(t) * slices * tile_bytes;
        const int off = (r >> 3) * 1024 + (r & 7) * 128 + ((ch ^ (r & 7)) << 4);
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            if (i >= slices) continue;
            uint4 v;
            __builtin_memcpy(&v, dig[i], 16);
            *reinterpret_cast<uint4*>(tile0 + int64_t(i) * tile_bytes + off) = v;
        }
    }
}

// ------------------------------------------------------------------------------------
// MMA kernel
// ------------------------------------------------------------------------------------
struct __align__(8) SplitShared {
    uint64_t full[NST];
    uint64_t empty[NST];
    uint64_t tfull[2];
    uint64_t tempty[2];
    uint64_t done;
    uint32_t tmem_base;
    int err;
};

__global__ void __launch_bounds__(THREADS, 1)
split_gemm_kernel(const SplitItem* __restrict__ items, int nitems,
                  const SplitTask* __restrict__ tasks, const uint8_t* __restrict__ apack,
                  const uint8_t* __restrict__ bpack, const int* __restrict__ ea,
                  const int* __restrict__ eb, Bases b, int slices, int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte aligned stage ring (the swizzle atom needs it)
    uint8_t* ring = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                               ~uintptr_t(1023));
    SplitShared* sh = reinterpret_cast<SplitShared*>(ring + NST * STAGE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int* serr = &sh->err;

    if (threadIdx.x == 0) {
        for (int i = 0; i < NST; ++i) {
            mbar_init(&sh->full[i], 1);
            mbar_init(&sh->empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&sh->tfull[i], 1);
            mbar_init(&sh->tempty[i], 8);  // one arrive per epilogue warp
        }
        mbar_init(&sh->done, 1);
        sh->err = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = sh->tmem_base;

    if (warp == 0) {
        // ---------------- producer ----------------
        if (lane == 0) {
            // test hook (tn_ctx_inject_wait_timeout, code 1): CTA 0 withholds the copies of its
            // first stage, so that the MMA warp's wait on it runs out and every role drains
            const bool withhold = blockIdx.x == 0 && atomicCAS(err + 1, 1, 0) == 1;
            uint32_t g = 0;  // global stage counter
            for (int it = blockIdx.x; it < nitems && !*serr; it += gridDim.x) {
                const SplitItem item = items[it];
                const SplitTask tk = tasks[item.task];
                for (int kt = 0; kt < tk.nkt && !*serr; ++kt)
                    for (int t = 0; t < slices; ++t, ++g) {
                        const int st = g % NST;
                        const uint32_t ph = (g / NST) & 1;
                        if (!mbar_wait(&sh->empty[st], ph ^ 1, err, serr)) break;
                        if (withhold && g == 0) continue;
                        uint8_t* dst = ring + st * STAGE;
                        mbar_expect_tx(&sh->full[st], STAGE);
                        const int64_t ao = tk.a_off + (int64_t(item.mt) * tk.nkt + kt) * slices * A_TILE +
                                           int64_t(t) * A_TILE;
                        const int64_t bo = tk.b_off + (int64_t(item.nt) * tk.nkt + kt) * slices * B_TILE +
                                           int64_t(t) * B_TILE;
                        bulk_g2s(dst, apack + ao, A_TILE, &sh->full[st]);
                        bulk_g2s(dst + A_TILE, bpack + bo, B_TILE, &sh->full[st]);
                    }
            }
            // before the CTA may exit, every copy this thread issued must have landed (in the
            // normal path the MMA warp has consumed them all; after an error this drains)
            for (uint32_t gg = (g > NST ? g - NST : 0); gg < g; ++gg)
                mbar_drain(&sh->full[gg % NST], (gg / NST) & 1);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(BM, BN);
            uint32_t g = 0;       // stage counter (matches the producer)
            uint32_t chunk = 0;   // accumulation chunk counter (TMEM double buffer)
            for (int it = blockIdx.x; it < nitems && !*serr; it += gridDim.x) {
                const SplitItem item = items[it];
                const SplitTask tk = tasks[item.task];
                for (int k0 = 0; k0 < tk.nkt && !*serr; k0 += KC, ++chunk) {
                    const int buf = chunk & 1;
                    if (!mbar_wait(&sh->tempty[buf], ((chunk >> 1) & 1) ^ 1, err, serr)) break;
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    bool first[NACC] = {true, true, true, true};
                    const int k1 = min(k0 + KC, tk.nkt);
                    bool ok = true;
                    for (int kt = k0; kt < k1 && ok; ++kt) {
                        const uint32_t g0 = g;
                        for (int t = 0; t < slices; ++t) {
                            const uint32_t gg = g0 + t;
                            if (!mbar_wait(&sh->full[gg % NST], (gg / NST) & 1, err, serr)) {
                                ok = false;
                                break;
                            }
                            asm volatile("tcgen05.fence::after_thread_sync;");
                            // pairs (i, j) with max(i, j) == t and i + j <= slices - 1
                            // (0-based slices: level = i + j + 2)
                            for (int i = 0; i <= t; ++i) {
                                for (int jj = 0; jj < 2; ++jj) {
                                    const int j = jj == 0 ? t : i;
                                    const int ii = jj == 0 ? i : t;
                                    if (jj == 1 && i == t) continue;  // (t, t) once
                                    if (ii + j > slices - 1) continue;
                                    const int lvl = min(ii + j, NACC - 1);
                                    const uint32_t sa = smem_u32(ring + ((g0 + ii) % NST) * STAGE);
                                    const uint32_t sb = smem_u32(ring + ((g0 + j) % NST) * STAGE + A_TILE);
                                    const uint32_t td = tmem + uint32_t(buf * NACC * BN + lvl * BN);
#pragma unroll
                                    for (int kk = 0; kk < BKT / 16; ++kk) {
                                        mma_bf16(td, sdesc(sa + kk * 32), sdesc(sb + kk * 32), idesc,
                                                 first[lvl] ? 0u : 1u);
                                        first[lvl] = false;
                                    }
                                }
                            }
                        }
                        if (!ok) break;
                        for (int t = 0; t < slices; ++t) mma_commit(&sh->empty[(g0 + t) % NST]);
                        g = g0 + slices;
                    }
                    if (!ok) break;
                    // with slices >= 4 every k tile writes all four levels, so every
                    // accumulator of this chunk has been (re)initialised
                    mma_commit(&sh->tfull[buf]);
                }
            }
            // every MMA this thread issued completes before TMEM is released
            mma_commit(&sh->done);
            mbar_drain(&sh->done, 0);
        }
    } else {
        // ---------------- epilogue (warps 2..9) ----------------
        constexpr int HC = BN / 2;       // columns per epilogue warp
        const int q = warp & 3;          // TMEM lane quadrant of this warp
        const int h = (warp - 2) >> 2;   // column half
        const int row = q * 32 + lane;   // row of the output tile
        uint32_t chunk = 0;
        for (int it = blockIdx.x; it < nitems && !*serr; it += gridDim.x) {
            const SplitItem item = items[it];
            const SplitTask tk = tasks[item.task];
            float hi[HC], lo[HC];
#pragma unroll
            for (int c = 0; c < HC; ++c) { hi[c] = 0.f; lo[c] = 0.f; }
            bool ok = true;
            for (int k0 = 0; k0 < tk.nkt; k0 += KC, ++chunk) {
                const int buf = chunk & 1;
                if (!mbar_wait(&sh->tfull[buf], (chunk >> 1) & 1, err, serr)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t tbase = tmem + (uint32_t(q * 32) << 16) + uint32_t(buf * NACC * BN + h * HC);
#pragma unroll
                for (int c0 = 0; c0 < HC; c0 += 16) {
#pragma unroll
                    for (int l = 0; l < NACC; ++l) {
                        float v[16];
                        tmem_ld16(tbase + l * BN + c0, v);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int c = 0; c < 16; ++c) df_add(hi[c0 + c], lo[c0 + c], v[c]);
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;");
                __syncwarp();
                if (lane == 0) mbar_arrive(&sh->tempty[buf]);
            }
            if (!ok) break;
            const int gr = item.mt * BM + row;
            if (gr < tk.m) {
                const int er = ea[tk.ea_off + gr];
                double* C = b.p[tk.cbuf] + tk.coff;
#pragma unroll
                for (int c = 0; c < HC; ++c) {
                    const int gc = item.nt * BN + h * HC + c;
                    if (gc < tk.n) {
                        const int ec = eb[tk.eb_off + gc];
                        const double v = (double(hi[c]) + double(lo[c])) * pow2(er + ec - 16);
                        double* c = C + gr + int64_t(gc) * tk.ldc;
                        *c = tk.accum ? *c + v : v;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
}

}  // namespace

int split_tile_bytes_a() { return A_TILE; }
int split_tile_bytes_b() { return B_TILE; }
int split_tile_rows_a() { return BM; }
int split_tile_rows_b() { return BN; }
int split_ktile() { return BKT; }

void launch_split_pack(const PackJob* jobs, int njobs, const KTileSrc* ksrc, const Bases& b,
                       uint8_t* out, int* expo, int slices, int tile_rows, cudaStream_t s,
                       int max_nkt, unsigned long long* gmax, int64_t nrows) {
    if (njobs <= 0) return;
    TN_REQUIRE(slices >= 4 && slices <= 7, "split precision needs 4..7 slices");
    TN_REQUIRE(tile_rows <= BM, "pack tile taller than the A tile");
    constexpr int KPER = 2;  // k tiles per CTA of the k-split pack
    if (max_nkt <= 2 * KPER || !gmax) {
        const dim3 g(njobs, (tile_rows + PACK_ROWS - 1) / PACK_ROWS);
        split_pack_kernel<<<g, PACK_THREADS, 0, s>>>(jobs, ksrc, b, out, expo, slices, tile_rows);
        TN_CUDA(cudaGetLastError());
        count_launch();
        return;
    }
    const dim3 g(njobs, (max_nkt + KPER - 1) / KPER);
    TN_CUDA(cudaMemsetAsync(gmax, 0, size_t(nrows) * sizeof(unsigned long long), s));
    split_rowmax_kernel<<<g, PACK_THREADS, 0, s>>>(jobs, ksrc, b, gmax, tile_rows, KPER);
    TN_CUDA(cudaGetLastError());
    split_pack_part_kernel<<<g, PACK_THREADS, 0, s>>>(jobs, ksrc, b, out, expo, gmax, slices,
                                                      tile_rows, KPER);
    TN_CUDA(cudaGetLastError());
    count_launch(2);
}

void launch_split_gemm(const SplitItem* items, int nitems, const SplitTask* tasks,
                       const uint8_t* apack, const uint8_t* bpack, const int* ea, const int* eb,
                       const Bases& b, int slices, int* err, int nsm, cudaStream_t s) {
    if (nitems <= 0) return;
    TN_REQUIRE(slices >= 4 && slices <= 7, "split precision needs 4..7 slices");
    const size_t shm = size_t(NST) * STAGE + sizeof(SplitShared) + 1024;
    static bool attr = false;
    if (!attr) {
        TN_CUDA(cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(shm)));
        attr = true;
    }
    const int grid = nitems < nsm ? nitems : nsm;
    split_gemm_kernel<<<grid, THREADS, shm, s>>>(items, nitems, tasks, apack, bpack, ea, eb, b,
                                                  slices, err);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tn
