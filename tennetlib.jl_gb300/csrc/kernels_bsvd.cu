// Multi-SM SVD of large charge blocks.
//
// A charge block of a two-site tensor at chi ~ 2048 has several hundred columns; one CTA per
// block (svd_qrj_kernel) then works out of L2 and uses a handful of SMs.  Here the O(n^3)
// work is spread over the whole GPU:
//  * the columns are ordered by decreasing norm before the QR: a static column pivoting that
//    leaves the rows of R graded as the pivoted QR of the Jacobi preconditioner does, so
//    that the sweeps on R^T converge several times faster on the graded blocks of DMRG;
//  * blocked Householder QR A = Q R: each 32-column panel is factored by one CTA in shared
//    memory (double-float), the trailing matrix is updated by grouped GEMMs with the compact
//    WY form Q_p = I - V T V^T (Schreiber & Van Loan 1989);
//  * one-sided Jacobi on R^T (Drmac & Veselic 2008: the triangular factor makes the cyclic
//    method converge in a few sweeps) by rounds of column-block pairs: in every round each CTA
//    of a matrix's group takes one pair of 16-column blocks (8 in double-float), stages the
//    columns of X and V in shared memory and rotates every column pair across the two blocks;
//    the pairs of one round are disjoint (round-robin tournament over the blocks), and the
//    group meets at a bounded barrier between rounds.  An FP32 presolve is followed, after a
//    Newton-Schulz re-orthonormalisation of V and Y = R^T V by GEMMs, by a double-float polish
//    (Higham, Tisseur, Webb & Zhou 2021);
//  * Q [V; 0] by grouped GEMMs, panel by panel in reverse.
// Every wait is bounded: a barrier that gives up sets the error word and the kernel returns.
#include <cuda_runtime.h>

#include "df_arith.cuh"
#include "tn_internal.h"

namespace tn {
namespace {
using namespace dfa;

constexpr int BT = 512;                       // threads per CTA
constexpr long long BJ_WAIT = 2000000000LL;   // barrier limit in clocks (about a second)
constexpr int SMEM_MAX = 227 * 1024 - 4096;   // dynamic shared memory budget (Jacobi)
constexpr int PANEL_SMEM = 227 * 1024 - 24 * 1024;  // panel kernel: 17 KB of static arrays

__device__ __forceinline__ df2 warp_sum_df(df2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = df_add(v, df_shfl_xor(v, o));
    return v;
}

// sum over the CTA, result in every thread (fixed order)
__device__ df2 block_sum_df(df2 v, df2* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum_df(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    df2 s{0.f, 0.f};
    for (int w = 0; w < BT / 32; ++w) s = df_add(s, red[w]);
    return s;
}

// largest |entry| of each block -> its scale exponent e (max |A| 2^-e in [1/2, 1))
__global__ void __launch_bounds__(BT) bsvd_scale_kernel(const BsvdBlk* __restrict__ descs,
                                                        const double* __restrict__ src,
                                                        double* __restrict__ ar) {
    const BsvdBlk d = descs[blockIdx.x];
    const int64_t tot = int64_t(d.rows) * d.cols;
    const double* M = src + d.src_off;
    __shared__ double red[BT / 32];
    double mx = 0.0;
    for (int64_t e = threadIdx.x; e < tot; e += BT) mx = fmax(mx, fabs(M[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 0; w < BT / 32; ++w) mx = fmax(mx, red[w]);
        int e = 0;
        if (mx > 0.0) frexp(mx, &e);
        ar[d.scl] = double(e);
    }
}

__global__ void bsvd_gather_kernel(const BsvdBlk* __restrict__ descs, const double* __restrict__ src,
                                   double* __restrict__ ar) {
    const BsvdBlk d = descs[blockIdx.y];
    const int64_t tot = int64_t(d.m) * d.n;
    const double* M = src + d.src_off;
    double* X = ar + d.xq;
    const int ex = int(ar[d.scl]);
    const int* pv = reinterpret_cast<const int*>(ar + d.piv);
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < tot;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int i = int(e % d.m), k = pv[int(e / d.m)];
        X[e] = ldexp(d.trans ? M[k + int64_t(i) * d.rows] : M[i + int64_t(k) * d.rows], -ex);
    }
}

// norms of the work matrix's columns (columns of the block, or its rows when it is worked on
// transposed): a warp per column, or a thread per row of the source when transposed, so the
// loads stay coalesced
__global__ void bsvd_colnorm_kernel(const BsvdBlk* __restrict__ descs,
                                    const double* __restrict__ src, double* __restrict__ ar) {
    const BsvdBlk d = descs[blockIdx.y];
    const double* M = src + d.src_off;
    double* cn = ar + d.cn;
    if (d.trans) {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.n; k += gridDim.x * blockDim.x) {
            double s = 0.0;
            for (int i = 0; i < d.m; ++i) {
                const double x = M[k + int64_t(i) * d.rows];
                s = fma(x, x, s);
            }
            cn[k] = sqrt(s);
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < d.n; k += nw) {
        const double* mk = M + int64_t(k) * d.rows;
        double s = 0.0;
        for (int i = lane; i < d.m; i += 32) s = fma(mk[i], mk[i], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) cn[k] = sqrt(s);
    }
}

// column order by decreasing norm, ties by index (bitonic sort of the padded key list in
// shared memory, one CTA per block): piv[k] = source column of work column k, piv[n + c] =
// work column of source column c
constexpr int SORT_MAX = 4096;  // >= bsvd_max_n()
__global__ void __launch_bounds__(BT) bsvd_presort_kernel(const BsvdBlk* __restrict__ descs,
                                                          double* __restrict__ ar) {
    __shared__ float key[SORT_MAX];
    __shared__ int idx[SORT_MAX];
    const BsvdBlk d = descs[blockIdx.x];
    const int n = d.n;
    int np = 1;
    while (np < n) np <<= 1;
    const double* cn = ar + d.cn;
    for (int k = threadIdx.x; k < np; k += BT) {
        key[k] = k < n ? float(cn[k]) : -1.f;
        idx[k] = k;
    }
    __syncthreads();
    for (int size = 2; size <= np; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < (np >> 1); t += BT) {
                const int lo = 2 * t - (t & (stride - 1)), hi = lo + stride;
                const float kl = key[lo], kh = key[hi];
                const int il = idx[lo], ih = idx[hi];
                const bool lo_first = kl > kh || (kl == kh && il < ih);
                if (lo_first != ((lo & size) == 0)) {
                    key[lo] = kh;
                    key[hi] = kl;
                    idx[lo] = ih;
                    idx[hi] = il;
                }
            }
            __syncthreads();
        }
    }
    int* pv = reinterpret_cast<int*>(ar + d.piv);
    for (int k = threadIdx.x; k < n; k += BT) {
        pv[k] = idx[k];
        pv[n + idx[k]] = k;
    }
}

// Householder QR of the panel columns [p0, p0 + w) of one block's work matrix (rows p0..m-1),
// one CTA per block, the panel in shared memory in double-float.  Writes the panel back (R on
// and above the diagonal), the explicit reflectors (unit diagonal, zeros above) and the two T
// factors of Q_p = H_p0 ... H_p0+w-1 = I - V T V^T: -T^T (trailing update) and -T (applying Q).
__global__ void __launch_bounds__(BT) bsvd_panel_kernel(const BsvdBlk* __restrict__ descs,
                                                        double* __restrict__ ar, int p0, int pw) {
    extern __shared__ __align__(16) unsigned char smem[];
    const BsvdBlk d = descs[blockIdx.x];
    if (p0 >= d.n) return;
    const int m = d.m, w = min(pw, d.n - p0), r = m - p0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    df2* P = reinterpret_cast<df2*>(smem);  // r x w, ld r
    __shared__ df2 tau[32];
    __shared__ df2 red[BT / 32];
    __shared__ float colmax[BT / 32];
    __shared__ df2 hh[3];
    __shared__ df2 T[32 * 32];
    __shared__ df2 G[32 * 32];
    double* X = ar + d.xq;
    for (int c = warp; c < w; c += BT / 32) {
        const double* xc = X + p0 + int64_t(p0 + c) * m;
        df2* pc = P + int64_t(c) * r;
        for (int i = lane; i < r; i += 32) pc[i] = df_from_double(xc[i]);
    }
    __syncthreads();
    for (int j = 0; j < w; ++j) {
        df2* pj = P + int64_t(j) * r;
        // the column is scaled by an exact power of two to a largest entry in [1/2, 1), so
        // that no square leaves the FP32 range (entries of graded blocks reach 1e-20 and less)
        float mx = 0.f;
        for (int i = j + threadIdx.x; i < r; i += BT) mx = fmaxf(mx, fabsf(pj[i].hi));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        __syncthreads();
        if (lane == 0) colmax[warp] = mx;
        __syncthreads();
        mx = 0.f;
        for (int q = 0; q < BT / 32; ++q) mx = fmaxf(mx, colmax[q]);
        int ex = 0;
        if (mx > 0.f) frexpf(mx, &ex);
        // a column below 2^-100 (already far under any kept singular value) is left as it is
        if (ex < -100) mx = 0.f;
        df2 sq{0.f, 0.f};
        for (int i = j + 1 + threadIdx.x; i < r; i += BT) {
            const df2 x = df_ldexp(pj[i], -ex);
            sq = df_fma(x, x, sq);
        }
        sq = block_sum_df(sq, red);
        if (threadIdx.x == 0) {
            const df2 alpha = df_ldexp(pj[j], -ex);
            if (sq.hi == 0.f || mx == 0.f) {
                hh[0] = df2{0.f, 0.f};
                hh[1] = pj[j];
                hh[2] = df2{0.f, 0.f};
            } else {
                // in the scaled column: beta' = -sign(alpha') |x'|, tau = (beta' - alpha') /
                // beta', v = x / (alpha - beta) = x' / (alpha' - beta'), R_jj = beta' 2^ex
                df2 beta = df_sqrt(df_fma(alpha, alpha, sq));
                if (alpha.hi >= 0.f) beta = df_neg(beta);
                hh[0] = df_mul(df_add(beta, df_neg(alpha)), df_recip(beta));
                hh[1] = df_ldexp(beta, ex);
                hh[2] = df_ldexp(df_recip(df_add(alpha, df_neg(beta))), -ex);
            }
            tau[j] = hh[0];
        }
        __syncthreads();
        const df2 tj = hh[0], sc = hh[2];
        for (int i = j + 1 + threadIdx.x; i < r; i += BT) pj[i] = df_mul(pj[i], sc);
        __syncthreads();
        if (threadIdx.x == 0) pj[j] = hh[1];
        for (int c = j + 1 + warp; c < w; c += BT / 32) {
            df2* pc = P + int64_t(c) * r;
            df2 acc{0.f, 0.f};
            for (int i = j + 1 + lane; i < r; i += 32) acc = df_fma(pj[i], pc[i], acc);
            acc = warp_sum_df(acc);
            const df2 wc = df_mul(df_add(acc, pc[j]), tj);
            __syncwarp();
            if (lane == 0) pc[j] = df_add(pc[j], df_neg(wc));
            for (int i = j + 1 + lane; i < r; i += 32) pc[i] = df_add(pc[i], df_neg(df_mul(wc, pj[i])));
        }
        __syncthreads();
    }
    // Gram of the reflectors: G[i][j] = v_i . v_j (i < j), v_i(i) = 1, v_i(l < i) = 0
    for (int q = warp; q < w * w; q += BT / 32) {
        const int i = q % w, j = q / w;
        if (i >= j) continue;
        const df2* vi = P + int64_t(i) * r;
        const df2* vj = P + int64_t(j) * r;
        df2 acc{0.f, 0.f};
        for (int l = j + 1 + lane; l < r; l += 32) acc = df_fma(vi[l], vj[l], acc);
        acc = warp_sum_df(acc);
        if (lane == 0) G[i + j * 32] = df_add(acc, vi[j]);
    }
    __syncthreads();
    // T (upper triangular): T[j][j] = tau_j, T[0:j, j] = -tau_j T[0:j, 0:j] G[0:j, j]
    for (int j = 0; j < w; ++j) {
        if (threadIdx.x < j) {
            const int i = threadIdx.x;
            df2 acc{0.f, 0.f};
            for (int k = i; k < j; ++k) acc = df_fma(T[i + k * 32], G[k + j * 32], acc);
            T[i + j * 32] = df_neg(df_mul(tau[j], acc));
        }
        if (threadIdx.x >= j && threadIdx.x < 32)
            T[threadIdx.x + j * 32] = threadIdx.x == j ? tau[j] : df2{0.f, 0.f};
        __syncthreads();
    }
    // write back
    double* Vp = ar + d.vp + int64_t(p0) * m;
    for (int c = warp; c < w; c += BT / 32) {
        double* xc = X + p0 + int64_t(p0 + c) * m;
        double* vc = Vp + int64_t(c) * r;
        const df2* pc = P + int64_t(c) * r;
        for (int i = lane; i < r; i += 32) {
            const double v = df_to_double(pc[i]);
            xc[i] = v;
            vc[i] = i == c ? 1.0 : (i > c ? v : 0.0);
        }
    }
    double* Tm = ar + d.tm + int64_t(p0) * 64;
    for (int e = threadIdx.x; e < w * w; e += BT) {
        const int i = e % w, j = e / w;
        Tm[e] = -df_to_double(T[j + i * 32]);         // -T^T
        Tm[w * w + e] = -df_to_double(T[i + j * 32]);  // -T
    }
}

// element-wise set-up kernels of the Jacobi phases (grid: chunks x blocks)
__global__ void bsvd_elem_kernel(const BsvdBlk* __restrict__ descs, int op, double* __restrict__ ar) {
    const BsvdBlk d = descs[blockIdx.y];
    const int n = d.n;
    const int64_t nn = int64_t(n) * n;
    const double* X = ar + d.xq;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < nn;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int i = int(e % n), j = int(e / n);
        if (op == 0) {
            const double rt = (j <= i) ? X[j + int64_t(i) * d.m] : 0.0;  // R^T[i, j] = R[j, i]
            ar[d.rt64 + e] = rt;
            reinterpret_cast<float*>(ar + d.r32)[e] = float(rt);
            reinterpret_cast<float*>(ar + d.v32)[e] = (i == j) ? 1.f : 0.f;
        } else if (op == 1) {
            ar[d.v64 + e] = double(reinterpret_cast<const float*>(ar + d.v32)[e]);
        } else if (op == 2) {
            const double g = ar[d.g64 + e];
            ar[d.g64 + e] = (i == j ? 1.5 : 0.0) - 0.5 * g;
        } else {
            reinterpret_cast<df2*>(ar + d.ydf)[e] = df_from_double(ar[d.y64 + e]);
            reinterpret_cast<df2*>(ar + d.vdf)[e] = df_from_double(ar[d.v64 + e]);
        }
    }
}

// ------------------------------------------------------------------------------------
// cooperative one-sided Jacobi by rounds of column-block pairs
// ------------------------------------------------------------------------------------
template <class T>
struct JOp;
template <>
struct JOp<float> {
    __device__ static float zero() { return 0.f; }
    __device__ static float fma(float a, float b, float c) { return fmaf(a, b, c); }
    __device__ static float add(float a, float b) { return a + b; }
    __device__ static float shfl(float a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    __device__ static float hi(float a) { return a; }
    __device__ static float diff_hi(float b, float a) { return b - a; }
    struct Rot {
        float c, s;
    };
    __device__ static Rot rot(float t) {
        const float c = rsqrtf(1.f + t * t);
        return Rot{c, c * t};
    }
    __device__ static void apply(const Rot& R, float& p, float& q) {
        const float x = p, y = q;
        p = R.c * x - R.s * y;
        q = R.s * x + R.c * y;
    }
    __device__ static float ld(const float* p) { return __ldcg(p); }
};
template <>
struct JOp<df2> {
    __device__ static df2 zero() { return df2{0.f, 0.f}; }
    __device__ static df2 fma(df2 a, df2 b, df2 c) { return df_fma(a, b, c); }
    __device__ static df2 add(df2 a, df2 b) { return df_add(a, b); }
    __device__ static df2 shfl(df2 a, int o) { return df_shfl_xor(a, o); }
    __device__ static float hi(df2 a) { return a.hi; }
    __device__ static float diff_hi(df2 b, df2 a) {
        const df2 d = df_add(b, df_neg(a));
        return d.hi + d.lo;
    }
    struct Rot {
        df2 c, s;
    };
    // the angle comes from FP32 (it only has to reduce the pair's cosine by many orders);
    // c and s are formed in double-float so that the rotation is orthogonal to ~1e-14
    __device__ static Rot rot(float t) {
        const df2 t2{t, 0.f};
        const df2 c = df_rsqrt(df_add(df2{1.f, 0.f}, df_mul(t2, t2)));
        return Rot{c, df_mul(c, t2)};
    }
    __device__ static void apply(const Rot& R, df2& p, df2& q) {
        const df2 x = p, y = q;
        p = df_add(df_mul(R.c, x), df_neg(df_mul(R.s, y)));
        q = df_add(df_mul(R.s, x), df_mul(R.c, y));
    }
    __device__ static df2 ld(const df2* p) {
        const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
        return df2{v.x, v.y};
    }
};

// registers per thread for the resident column of a cross task (X and V: 2 RM values), set
// so that n * B <= 512 RM (the block width is chosen from this, see bj_block)
template <class T>
struct JRegs;
template <>
struct JRegs<float> {
    static constexpr int RM = 36;
};
template <>
struct JRegs<df2> {
    static constexpr int RM = 18;
};

__device__ __forceinline__ bool group_barrier(unsigned* bar, unsigned target, int* err, int* s_fail) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        const long long t0 = clock64();
        while (true) {
            if (*reinterpret_cast<volatile unsigned*>(bar) >= target) break;
            if (*reinterpret_cast<volatile int*>(err) != 0 || clock64() - t0 > BJ_WAIT) {
                atomicExch(err, 3);
                *s_fail = 1;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    return *reinterpret_cast<volatile int*>(s_fail) == 0;
}

__device__ __forceinline__ int rr_player(int nn, int r, int pos) {
    return pos == 0 ? 0 : 1 + ((pos - 1 + r) % (nn - 1));
}

// One CTA's part of the Jacobi sweeps of one matrix (see the file comment).  B = columns per
// block; a cross task rotates the B x B column pairs (I_a, J_b) in B sub-rounds of B disjoint
// pairs, a diagonal task the pairs inside one block (round-robin, B - 1 sub-rounds of B/2).
template <class T, int B>
__global__ void __launch_bounds__(BT, 1)
bj_kernel(const BjDesc* __restrict__ descs, int nd, float tol, int max_sweeps, int use_maxcos,
          int* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem[];
    int di = 0;
    while (di < nd && !(int(blockIdx.x) >= descs[di].cta0 &&
                        int(blockIdx.x) < descs[di].cta0 + descs[di].ncta))
        ++di;
    if (di >= nd) return;
    const BjDesc d = descs[di];
    const int lc = int(blockIdx.x) - d.cta0;
    const int n = d.n;
    T* xs = reinterpret_cast<T*>(smem);       // B staged columns of X, n rows each
    T* vs = xs + int64_t(B) * n;               // B staged columns of V
    __shared__ int gcol[2 * B];
    __shared__ int s_rot, s_fail;
    __shared__ unsigned s_maxcos;
    __shared__ T red[BT / 32][3];
    T* X = static_cast<T*>(d.X);
    T* V = static_cast<T*>(d.V);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_rot = 0;
        // test hook (tn_ctx_inject_wait_timeout, code 2): CTA 0 of the first group leaves
        // before its first barrier, so that the group's barrier waits run out
        s_fail = (di == 0 && lc == 0 && atomicCAS(err + 1, 2, 0) == 2) ? 1 : 0;
        s_maxcos = 0u;
    }
    __syncthreads();
    if (s_fail) return;
    const int nbe = d.nb + (d.nb & 1);
    unsigned nbar = 0;
    int sweep = 0;

    // load / store the columns of blocks I (local 0..B-1) and J (local B..2B-1, J < 0: none)
    auto load = [&](int I, int J) {
        if (threadIdx.x < 2 * B) {
            const int c = threadIdx.x;
            const int blk = c < B ? I : J;
            const int g = (blk < 0) ? -1 : blk * B + (c % B);
            gcol[c] = (g >= 0 && g < n) ? g : -1;
        }
        __syncthreads();
        // one warp per column (no integer division in the address arithmetic)
        const int nc = J < 0 ? B : 2 * B;
        for (int c = warp; c < nc; c += BT / 32) {
            const int g = gcol[c];
            if (g < 0) continue;
            const T* xg = X + int64_t(g) * n;
            const T* vg = V + int64_t(g) * n;
            T* xl = xs + int64_t(c) * n;
            T* vl = vs + int64_t(c) * n;
            for (int i = lane; i < n; i += 32) {
                xl[i] = JOp<T>::ld(xg + i);
                vl[i] = JOp<T>::ld(vg + i);
            }
        }
        __syncthreads();
    };
    auto store = [&](int J) {
        const int nc = J < 0 ? B : 2 * B;
        for (int c = warp; c < nc; c += BT / 32) {
            const int g = gcol[c];
            if (g < 0) continue;
            T* xg = X + int64_t(g) * n;
            T* vg = V + int64_t(g) * n;
            const T* xl = xs + int64_t(c) * n;
            const T* vl = vs + int64_t(c) * n;
            for (int i = lane; i < n; i += 32) {
                xg[i] = xl[i];
                vg[i] = vl[i];
            }
        }
        __syncthreads();
    };
    // one sub-round: npair disjoint local pairs (li[a], lj[a]) given by pair_of(a)
    auto subround = [&](int npair, auto pair_of) {
        const int G = BT / npair;          // threads per pair (a multiple of 32)
        const int a = threadIdx.x / G;
        const int sub = threadIdx.x % G;
        const int wpp = G / 32;            // warps per pair
        int li = 0, lj = 0;
        pair_of(a, li, lj);
        const bool act = gcol[li] >= 0 && gcol[lj] >= 0;
        T sa = JOp<T>::zero(), sb = JOp<T>::zero(), sg = JOp<T>::zero();
        T* xi = xs + int64_t(li) * n;
        T* xj = xs + int64_t(lj) * n;
        if (act)
            for (int t = sub; t < n; t += G) {
                const T p = xi[t], q = xj[t];
                sa = JOp<T>::fma(p, p, sa);
                sb = JOp<T>::fma(q, q, sb);
                sg = JOp<T>::fma(p, q, sg);
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sa = JOp<T>::add(sa, JOp<T>::shfl(sa, o));
            sb = JOp<T>::add(sb, JOp<T>::shfl(sb, o));
            sg = JOp<T>::add(sg, JOp<T>::shfl(sg, o));
        }
        if (wpp > 1) {
            if (lane == 0) {
                red[warp][0] = sa;
                red[warp][1] = sb;
                red[warp][2] = sg;
            }
            __syncthreads();
            const int w0 = (a * G) / 32;
            sa = red[w0][0];
            sb = red[w0][1];
            sg = red[w0][2];
            for (int k = 1; k < wpp; ++k) {
                sa = JOp<T>::add(sa, red[w0 + k][0]);
                sb = JOp<T>::add(sb, red[w0 + k][1]);
                sg = JOp<T>::add(sg, red[w0 + k][2]);
            }
        }
        const float ah = JOp<T>::hi(sa), bh = JOp<T>::hi(sb), gh = JOp<T>::hi(sg);
        // the block is scaled to a largest entry in [1/2, 1), so sigma_max >= 1/2: columns
        // whose squared norm is below 1e-36 (under 2e-18 sigma_max, far below any kept value)
        // are not rotated; their squares sit at the bottom of the FP32 range, where the
        // rotation test is rounding noise and would never settle
        bool rot = act && ah > 1e-36f && bh > 1e-36f && fabsf(gh) > tol * sqrtf(ah) * sqrtf(bh);
        float tt = 0.f;
        if (rot) {
            const float zeta = JOp<T>::diff_hi(sb, sa) / (2.f * gh);
            const float az = fabsf(zeta);
            // |zeta| large (graded columns): tan = 1/(2 zeta) avoids zeta^2 overflow
            tt = az > 1e15f ? 0.5f / zeta : (zeta >= 0.f ? 1.f : -1.f) / (az + sqrtf(1.f + zeta * zeta));
            rot = isfinite(tt) && tt != 0.f;
        }
        if (rot) {
            const typename JOp<T>::Rot R = JOp<T>::rot(tt);
            for (int t = sub; t < n; t += G) JOp<T>::apply(R, xi[t], xj[t]);
            T* vi = vs + int64_t(li) * n;
            T* vj = vs + int64_t(lj) * n;
            for (int t = sub; t < n; t += G) JOp<T>::apply(R, vi[t], vj[t]);
            if (sub == 0) {
                s_rot = 1;
                const float cosr = fabsf(gh) / (sqrtf(ah) * sqrtf(bh));
                atomicMax(&s_maxcos, __float_as_uint(cosr));
            }
        }
        __syncthreads();
    };
    auto flush_flags = [&]() {
        if (threadIdx.x == 0 && s_rot) {
            atomicOr(&d.flags[sweep % 3], 1);
            atomicMax(reinterpret_cast<unsigned*>(&d.flags[3 + sweep % 3]), s_maxcos);
            s_rot = 0;
            s_maxcos = 0u;
        }
    };

    // Cross task of blocks I < J: the B column pairs (I_a, J_(a+k) mod B), k = 0..B-1.  The
    // group of G threads of pair a keeps column I_a of X and V in registers for the whole
    // task (RM elements per thread), the J columns are staged in shared memory and move from
    // group to group, so each rotation reads its J column twice and writes it once.
    auto cross_task = [&](int I, int J) {
        constexpr int G = BT / B;
        constexpr int RM = JRegs<T>::RM;
        const int a = threadIdx.x / G, sub = threadIdx.x % G;
        const int wpp = G / 32;
        const int gi = I * B + a;
        const bool own = gi < n;
        T xr[RM], vr[RM];
#pragma unroll
        for (int r = 0; r < RM; ++r) {
            const int t = sub + G * r;
            const bool ok = own && t < n;
            xr[r] = ok ? JOp<T>::ld(X + int64_t(gi) * n + t) : JOp<T>::zero();
            vr[r] = ok ? JOp<T>::ld(V + int64_t(gi) * n + t) : JOp<T>::zero();
        }
        if (threadIdx.x < B) {
            const int g = J * B + int(threadIdx.x);
            gcol[threadIdx.x] = g < n ? g : -1;
        }
        __syncthreads();
        for (int c = warp; c < B; c += BT / 32) {
            const int g = gcol[c];
            if (g < 0) continue;
            const T* xg = X + int64_t(g) * n;
            const T* vg = V + int64_t(g) * n;
            T* xl = xs + int64_t(c) * n;
            T* vl = vs + int64_t(c) * n;
            for (int i = lane; i < n; i += 32) {
                xl[i] = JOp<T>::ld(xg + i);
                vl[i] = JOp<T>::ld(vg + i);
            }
        }
        __syncthreads();
        for (int k = 0; k < B; ++k) {
            const int c = (a + k) % B;
            const bool act = own && gcol[c] >= 0;
            T* xc = xs + int64_t(c) * n;
            T* vc = vs + int64_t(c) * n;
            T sa = JOp<T>::zero(), sb = JOp<T>::zero(), sg = JOp<T>::zero();
            if (act) {
#pragma unroll
                for (int r = 0; r < RM; ++r) {
                    const int t = sub + G * r;
                    if (t < n) {
                        const T q = xc[t];
                        sa = JOp<T>::fma(xr[r], xr[r], sa);
                        sb = JOp<T>::fma(q, q, sb);
                        sg = JOp<T>::fma(xr[r], q, sg);
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sa = JOp<T>::add(sa, JOp<T>::shfl(sa, o));
                sb = JOp<T>::add(sb, JOp<T>::shfl(sb, o));
                sg = JOp<T>::add(sg, JOp<T>::shfl(sg, o));
            }
            if (wpp > 1) {
                if (lane == 0) {
                    red[warp][0] = sa;
                    red[warp][1] = sb;
                    red[warp][2] = sg;
                }
                __syncthreads();
                const int w0 = (a * G) / 32;
                sa = red[w0][0];
                sb = red[w0][1];
                sg = red[w0][2];
                for (int q = 1; q < wpp; ++q) {
                    sa = JOp<T>::add(sa, red[w0 + q][0]);
                    sb = JOp<T>::add(sb, red[w0 + q][1]);
                    sg = JOp<T>::add(sg, red[w0 + q][2]);
                }
            }
            const float ah = JOp<T>::hi(sa), bh = JOp<T>::hi(sb), gh = JOp<T>::hi(sg);
            bool rot = act && ah > 1e-36f && bh > 1e-36f && fabsf(gh) > tol * sqrtf(ah) * sqrtf(bh);
            float tt = 0.f;
            if (rot) {
                const float zeta = JOp<T>::diff_hi(sb, sa) / (2.f * gh);
                const float az = fabsf(zeta);
                tt = az > 1e15f ? 0.5f / zeta : (zeta >= 0.f ? 1.f : -1.f) / (az + sqrtf(1.f + zeta * zeta));
                rot = isfinite(tt) && tt != 0.f;
            }
            if (rot) {
                const typename JOp<T>::Rot R = JOp<T>::rot(tt);
#pragma unroll
                for (int r = 0; r < RM; ++r) {
                    const int t = sub + G * r;
                    if (t < n) {
                        T q = xc[t];
                        JOp<T>::apply(R, xr[r], q);
                        xc[t] = q;
                        T w = vc[t];
                        JOp<T>::apply(R, vr[r], w);
                        vc[t] = w;
                    }
                }
                if (sub == 0) {
                    s_rot = 1;
                    const float cosr = fabsf(gh) / (sqrtf(ah) * sqrtf(bh));
                    atomicMax(&s_maxcos, __float_as_uint(cosr));
                }
            }
            __syncthreads();
        }
        if (own) {
#pragma unroll
            for (int r = 0; r < RM; ++r) {
                const int t = sub + G * r;
                if (t < n) {
                    X[int64_t(gi) * n + t] = xr[r];
                    V[int64_t(gi) * n + t] = vr[r];
                }
            }
        }
        for (int c = warp; c < B; c += BT / 32) {
            const int g = gcol[c];
            if (g < 0) continue;
            T* xg = X + int64_t(g) * n;
            T* vg = V + int64_t(g) * n;
            const T* xl = xs + int64_t(c) * n;
            const T* vl = vs + int64_t(c) * n;
            for (int i = lane; i < n; i += 32) {
                xg[i] = xl[i];
                vg[i] = vl[i];
            }
        }
        __syncthreads();
    };

    for (sweep = 0; sweep < max_sweeps; ++sweep) {
        if (lc == 0 && threadIdx.x == 0) {
            d.flags[(sweep + 1) % 3] = 0;
            d.flags[3 + (sweep + 1) % 3] = 0;
        }
        // diagonal round: the pairs inside each block
        for (int I = lc; I < d.nb; I += d.ncta) {
            load(I, -1);
            for (int k = 0; k < B - 1; ++k)
                subround(B / 2, [&](int a, int& li, int& lj) {
                    const int p = rr_player(B, k, a), q = rr_player(B, k, B - 1 - a);
                    li = min(p, q);
                    lj = max(p, q);
                });
            store(-1);
            flush_flags();
        }
        if (!group_barrier(d.bar, (++nbar) * unsigned(d.ncta), err, &s_fail)) return;
        for (int r = 0; r < nbe - 1; ++r) {
            for (int t = lc; t < nbe / 2; t += d.ncta) {
                int I = rr_player(nbe, r, t), J = rr_player(nbe, r, nbe - 1 - t);
                if (I > J) {
                    const int u = I;
                    I = J;
                    J = u;
                }
                if (J >= d.nb) continue;
                cross_task(I, J);
                flush_flags();
            }
            if (!group_barrier(d.bar, (++nbar) * unsigned(d.ncta), err, &s_fail)) return;
        }
        const int rotated = *reinterpret_cast<volatile int*>(&d.flags[sweep % 3]);
        const float maxcos =
            __uint_as_float(*reinterpret_cast<volatile unsigned*>(&d.flags[3 + sweep % 3]));
        if (!rotated) break;
        // quadratic convergence: a sweep whose largest rotated cosine is below 1e-7 leaves
        // nothing above the tolerance for the next one
        if (use_maxcos && maxcos < 1.0e-7f) {
            ++sweep;
            break;
        }
    }
    if (lc == 0 && threadIdx.x == 0 && d.sweeps) *d.sweeps = sweep;
}

// singular values = column norms of Y (double-float), sorted descending with the
// permutation (PY = P Y and QV = [V; 0] are written by bsvd_outputs_kernel)
__global__ void __launch_bounds__(BT) bsvd_finish_kernel(const BsvdBlk* __restrict__ descs,
                                                         double* __restrict__ ar,
                                                         double* __restrict__ qv,
                                                         double* __restrict__ py,
                                                         double* __restrict__ S,
                                                         int* __restrict__ perm) {
    extern __shared__ __align__(16) unsigned char smem[];
    const BsvdBlk d = descs[blockIdx.x];
    const int n = d.n, m = d.m;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* h = reinterpret_cast<double*>(smem);
    const df2* Y = reinterpret_cast<const df2*>(ar + d.ydf);
    const int ex = int(ar[d.scl]);  // undo the power-of-two scaling of the block
    for (int j = warp; j < n; j += BT / 32) {
        const df2* yj = Y + int64_t(j) * n;
        df2 a{0.f, 0.f};
        for (int t = lane; t < n; t += 32) a = df_fma(yj[t], yj[t], a);
        a = warp_sum_df(a);
        if (lane == 0) h[j] = ldexp(sqrt(df_to_double(a)), ex);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += BT) {
        const double sj = h[j];
        int rank = 0;
        for (int k = 0; k < n; ++k) {
            const double sk = h[k];
            rank += (sk > sj) || (sk == sj && k < j);
        }
        S[d.s_off + rank] = sj;
        perm[d.s_off + rank] = j;
    }
    (void)m;
}

// PY = P Y (scaled back, rows in the source column order) and QV = [V; 0]: element-wise, spread over many CTAs per block (the
// conversions from double-float use the FP64 pipe)
__global__ void bsvd_outputs_kernel(const BsvdBlk* __restrict__ descs, const double* __restrict__ ar,
                                    double* __restrict__ qv, double* __restrict__ py) {
    const BsvdBlk d = descs[blockIdx.y];
    const int n = d.n, m = d.m;
    const int ex = int(ar[d.scl]);
    const df2* Y = reinterpret_cast<const df2*>(ar + d.ydf);
    const df2* Vd = reinterpret_cast<const df2*>(ar + d.vdf);
    double* P = py + d.v_off;
    double* Z = qv + d.x_off;
    const int* ip = reinterpret_cast<const int*>(ar + d.piv) + n;  // work column of source c
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int j = gw; j < n; j += nw) {
        const df2* yj = Y + int64_t(j) * n;
        double* pj = P + int64_t(j) * n;
        for (int c = lane; c < n; c += 32) pj[c] = ldexp(df_to_double(yj[ip[c]]), ex);
        double* zj = Z + int64_t(j) * m;
        const df2* vj = Vd + int64_t(j) * n;
        for (int i = lane; i < m; i += 32) zj[i] = (i < n) ? df_to_double(vj[i]) : 0.0;
    }
}

int grid_chunks(int64_t work) {
    int64_t g = (work + 255) / 256;
    if (g > 1184) g = 1184;
    return int(g < 1 ? 1 : g);
}

template <class T, int B>
size_t bj_smem(int maxn) {
    return size_t(B) * size_t(maxn) * sizeof(T) * 2;  // B staged columns of X and of V
}

template <class T, int B>
void bj_launch(const BjDesc* d, int nd, int nctas, int maxn, float tol, int max_sweeps,
               int use_maxcos, int* err, cudaStream_t s) {
    const size_t shm = bj_smem<T, B>(maxn);
    TN_CUDA(cudaFuncSetAttribute(bj_kernel<T, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(shm)));
    void* args[] = {(void*)&d, (void*)&nd, (void*)&tol, (void*)&max_sweeps, (void*)&use_maxcos,
                    (void*)&err};
    TN_CUDA(cudaLaunchCooperativeKernel((const void*)bj_kernel<T, B>, dim3(nctas), dim3(BT), args,
                                        shm, s));
}

template <class T, int B>
int bj_capacity(int maxn) {
    const size_t shm = bj_smem<T, B>(maxn);
    TN_CUDA(cudaFuncSetAttribute(bj_kernel<T, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(shm)));
    int dev = 0, nsm = 0, per = 0;
    TN_CUDA(cudaGetDevice(&dev));
    TN_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    TN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, bj_kernel<T, B>, BT, shm));
    return nsm * per;
}

}  // namespace

int bsvd_panel_width(int mmax) {
    // the panel (m x w double-float) must fit the shared memory budget
    for (int w = 32; w >= 4; w /= 2)
        if (int64_t(mmax) * w * 8 <= PANEL_SMEM) return w;
    return 0;
}

// Column blocks as wide as the registers of the resident column and the shared memory of the
// staged columns allow: n B <= 512 RM and 2 B n sizeof(T) <= SMEM_MAX (FP32: B in {16, 8, 4},
// double-float: B in {16, 8, 4, 2}, the polish with half the FP32 width or more).
int bsvd_max_n() { return 3568; }

static int bj_block(int maxn, int precision) {
    const int rm = precision == 0 ? JRegs<float>::RM : JRegs<df2>::RM;
    const int esz = precision == 0 ? 4 : 8;
    const int bmin = precision == 0 ? 4 : 2;
    for (int b = 16; b >= bmin; b /= 2)
        if (int64_t(maxn) * b <= int64_t(BT) * rm && int64_t(2) * b * maxn * esz <= SMEM_MAX)
            return b;
    return 0;
}

void launch_bsvd_gather(const BsvdBlk* d, int nb, int64_t mnmax, const double* src, double* ar,
                        cudaStream_t s) {
    if (nb <= 0) return;
    bsvd_scale_kernel<<<nb, BT, 0, s>>>(d, src, ar);
    TN_CUDA(cudaGetLastError());
    count_launch();
    bsvd_colnorm_kernel<<<dim3(16, nb), 256, 0, s>>>(d, src, ar);
    TN_CUDA(cudaGetLastError());
    count_launch();
    bsvd_presort_kernel<<<nb, BT, 0, s>>>(d, ar);
    TN_CUDA(cudaGetLastError());
    count_launch();
    bsvd_gather_kernel<<<dim3(grid_chunks(mnmax), nb), 256, 0, s>>>(d, src, ar);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_bsvd_panel(const BsvdBlk* d, int nb, int p0, int pw, int rmax, double* ar,
                       cudaStream_t s) {
    if (nb <= 0) return;
    const size_t shm = size_t(rmax) * pw * 8;  // the panel rows of the tallest block
    TN_REQUIRE(pw >= 1 && pw <= 32 && shm <= size_t(PANEL_SMEM), "block SVD: panel too large");
    TN_CUDA(cudaFuncSetAttribute(bsvd_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(shm)));
    bsvd_panel_kernel<<<nb, BT, shm, s>>>(d, ar, p0, pw);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_bsvd_elem(const BsvdBlk* d, int nb, int64_t nnmax, int op, double* ar, cudaStream_t s) {
    if (nb <= 0) return;
    bsvd_elem_kernel<<<dim3(grid_chunks(nnmax), nb), 256, 0, s>>>(d, op, ar);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

int bsvd_jacobi_block(int maxn, int precision) { return bj_block(maxn, precision); }

int bsvd_jacobi_capacity(int maxn, int precision) {
    switch (bsvd_jacobi_block(maxn, precision) + 100 * precision) {
        case 16: return bj_capacity<float, 16>(maxn);
        case 8: return bj_capacity<float, 8>(maxn);
        case 4: return bj_capacity<float, 4>(maxn);
        case 116: return bj_capacity<df2, 16>(maxn);
        case 108: return bj_capacity<df2, 8>(maxn);
        case 104: return bj_capacity<df2, 4>(maxn);
        case 102: return bj_capacity<df2, 2>(maxn);
        default: throw Error(-1, "block SVD: block too large for the Jacobi kernel");
    }
}

void launch_bsvd_jacobi(const BjDesc* d, int nd, int nctas, int maxn, int precision, int* err,
                        cudaStream_t s) {
    if (nd <= 0) return;
    TN_REQUIRE(maxn <= bsvd_max_n(), "block SVD: block too large for the Jacobi kernel");
    // rotation threshold above the rounding noise of a double-float dot product
    const float tdf = 3.55e-15f * sqrtf(float(maxn > 1 ? maxn : 1)) * 32.f;
    switch (bsvd_jacobi_block(maxn, precision) + 100 * precision) {
        case 16: bj_launch<float, 16>(d, nd, nctas, maxn, 2.0e-5f, 30, 0, err, s); break;
        case 8: bj_launch<float, 8>(d, nd, nctas, maxn, 2.0e-5f, 30, 0, err, s); break;
        case 4: bj_launch<float, 4>(d, nd, nctas, maxn, 2.0e-5f, 30, 0, err, s); break;
        case 116: bj_launch<df2, 16>(d, nd, nctas, maxn, tdf, 30, 1, err, s); break;
        case 108: bj_launch<df2, 8>(d, nd, nctas, maxn, tdf, 30, 1, err, s); break;
        case 104: bj_launch<df2, 4>(d, nd, nctas, maxn, tdf, 30, 1, err, s); break;
        case 102: bj_launch<df2, 2>(d, nd, nctas, maxn, tdf, 30, 1, err, s); break;
        default: throw Error(-1, "block SVD: block too large for the Jacobi kernel");
    }
    count_launch();
}

void launch_bsvd_finish(const BsvdBlk* d, int nb, double* ar, double* qv, double* py, double* S,
                        int* perm, cudaStream_t s) {
    if (nb <= 0) return;
    const size_t shm = size_t(bsvd_max_n()) * 8;
    TN_CUDA(cudaFuncSetAttribute(bsvd_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(shm)));
    bsvd_finish_kernel<<<nb, BT, shm, s>>>(d, ar, qv, py, S, perm);
    TN_CUDA(cudaGetLastError());
    bsvd_outputs_kernel<<<dim3(64, nb), 256, 0, s>>>(d, ar, qv, py);
    TN_CUDA(cudaGetLastError());
    count_launch(2);
}

}  // namespace tn
