// Batched one-sided Jacobi SVD of the charge blocks of a two-site tensor (Hestenes' method
// with round-robin parallel ordering; FP32 presolve, FP64 polish), followed by the
// extraction of the truncated factors into the left/right site tensors.  The truncation decision itself is
// made on the host from the sorted singular values (tiny, integer-valued result).
#include <cuda_runtime.h>

#include "df_arith.cuh"
#include "tn_internal.h"

namespace tn {
namespace {
using namespace dfa;

constexpr int SVD_THREADS = 512;
// Round-robin tournament: nn (even) players, round r in [0, nn-1), pair k in [0, nn/2).
__device__ __forceinline__ void rr_pair(int nn, int r, int k, int& i, int& j) {
    auto player = [&](int pos) { return pos == 0 ? 0 : 1 + ((pos - 1 + r) % (nn - 1)); };
    i = player(k);
    j = player(nn - 1 - k);
    if (i > j) { int t = i; i = j; j = t; }
}

// Reduction over the 8 lanes of a pair group (xor offsets stay inside the group).
template <class T>
__device__ __forceinline__ T gsum8(T v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v;
}

// One-sided Jacobi sweeps on the columns of x (m x n, column-major, leading dim m) with
// the rotations accumulated into v (n x n).  T is the working precision of every operation
// (on GB300 one warp-wide FP64 instruction occupies the SM's FP64 pipe for many cycles,
// so the FP32 presolve must not touch FP64).  Each warp works on 4 disjoint column pairs
// at a time, 8 lanes per pair.  Returns the number of sweeps run; all threads must call it.
template <class T>
__device__ int jacobi_sweeps(T* x, T* v, int m, int n, T tol, int max_sweeps, int* rotated) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int grp = lane >> 3, sub = lane & 7;
    const int nn = n + (n & 1);
    const int npairs = nn / 2;
    const int slots = nwarps * 4;
    int sweep = 0;
    if (n < 2) return 0;
    for (sweep = 0; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) *rotated = 0;
        __syncthreads();
        for (int r = 0; r < nn - 1; ++r) {
            for (int base = 0; base < npairs; base += slots) {
                const int k = base + warp * 4 + grp;
                int i = 0, j = 0;
                const bool live = k < npairs;
                if (live) rr_pair(nn, r, k, i, j);
                const bool act = live && j < n;
                T a = 0, bb = 0, g = 0;
                T* xi = x + int64_t(i) * m;
                T* xj = x + int64_t(j) * m;
                if (act)
                    for (int t = sub; t < m; t += 8) {
                        const T p = xi[t], q = xj[t];
                        a = fma(p, p, a);
                        bb = fma(q, q, bb);
                        g = fma(p, q, g);
                    }
                a = gsum8(a);
                bb = gsum8(bb);
                g = gsum8(g);
                bool rot = act && a > T(0) && bb > T(0) && (fabs(g) > tol * sqrt(a) * sqrt(bb));
                T tt = T(0);
                if (rot) {
                    const T zeta = (bb - a) / (T(2) * g);
                    const T az = fabs(zeta);
                    // |zeta| large (graded columns): tan = 1/(2 zeta) avoids zeta^2 overflow
                    tt = az > T(1e15) ? T(0.5) / zeta
                                      : (zeta >= T(0) ? T(1) : T(-1)) / (az + sqrt(T(1) + zeta * zeta));
                    rot = isfinite(tt) && tt != T(0);  // a no-op rotation is not a rotation
                }
                if (rot) {
                    const T c = T(1) / sqrt(T(1) + tt * tt);
                    const T sn = c * tt;
                    for (int t = sub; t < m; t += 8) {
                        const T p = xi[t], q = xj[t];
                        xi[t] = c * p - sn * q;
                        xj[t] = sn * p + c * q;
                    }
                    T* vi = v + int64_t(i) * n;
                    T* vj = v + int64_t(j) * n;
                    for (int t = sub; t < n; t += 8) {
                        const T p = vi[t], q = vj[t];
                        vi[t] = c * p - sn * q;
                        vj[t] = sn * p + c * q;
                    }
                    if (sub == 0) *rotated = 1;
                }
            }
            __syncthreads();
        }
        const int done = !*rotated;
        __syncthreads();
        if (done) break;
    }
    return sweep;
}

// One-sided Jacobi sweeps in double-float on the columns of x (m x n) with rotations
// accumulated into v (n x n); same pairing and layout as jacobi_sweeps.  The rotation
// angle comes from FP32 (it only has to zero the pair to ~1e-7 of itself, which a sweep
// squares), while c and s are formed in double-float from that angle so that every
// rotation is orthogonal to double-float precision.  No FP64 instruction is executed.
// A sweep whose largest rotated |cos| (g / sqrt(a b)) stays below 1e-7 leaves, by the
// quadratic convergence of one-sided Jacobi, nothing above tol for the next sweep: the
// loop then stops without the confirming sweep.
__device__ int jacobi_sweeps_df(df2* x, df2* v, int m, int n, float tol, int max_sweeps,
                                int* rotated, unsigned* maxcos_bits) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int grp = lane >> 3, sub = lane & 7;
    const int nn = n + (n & 1);
    const int npairs = nn / 2;
    const int slots = nwarps * 4;
    int sweep = 0;
    if (n < 2) return 0;
    for (sweep = 0; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) {
            *rotated = 0;
            *maxcos_bits = 0u;
        }
        __syncthreads();
        for (int r = 0; r < nn - 1; ++r) {
            for (int base = 0; base < npairs; base += slots) {
                const int k = base + warp * 4 + grp;
                int i = 0, j = 0;
                const bool live = k < npairs;
                if (live) rr_pair(nn, r, k, i, j);
                const bool act = live && j < n;
                df2 a{0.f, 0.f}, bb{0.f, 0.f}, g{0.f, 0.f};
                df2* xi = x + int64_t(i) * m;
                df2* xj = x + int64_t(j) * m;
                if (act)
                    for (int t = sub; t < m; t += 8) {
                        const df2 p = xi[t], q = xj[t];
                        a = df_fma(p, p, a);
                        bb = df_fma(q, q, bb);
                        g = df_fma(p, q, g);
                    }
#pragma unroll
                for (int o = 4; o > 0; o >>= 1) {
                    a = df_add(a, df_shfl_xor(a, o));
                    bb = df_add(bb, df_shfl_xor(bb, o));
                    g = df_add(g, df_shfl_xor(g, o));
                }
                bool rot = act && a.hi > 0.f && bb.hi > 0.f &&
                           (fabsf(g.hi) > tol * sqrtf(a.hi) * sqrtf(bb.hi));
                float tt = 0.f;
                if (rot) {
                    const df2 d = df_add(bb, df_neg(a));
                    const float zeta = (d.hi + d.lo) / (2.f * g.hi);
                    const float az = fabsf(zeta);
                    // |zeta| large (graded columns): tan = 1/(2 zeta) avoids zeta^2 overflow
                    tt = az > 1e15f ? 0.5f / zeta
                                    : (zeta >= 0.f ? 1.f : -1.f) / (az + sqrtf(1.f + zeta * zeta));
                    rot = isfinite(tt) && tt != 0.f;  // a no-op rotation is not a rotation
                }
                if (rot) {
                    const df2 t2{tt, 0.f};
                    const df2 c = df_rsqrt(df_add(df2{1.f, 0.f}, df_mul(t2, t2)));
                    const df2 sn = df_mul(c, t2);
                    for (int t = sub; t < m; t += 8) {
                        const df2 p = xi[t], q = xj[t];
                        xi[t] = df_add(df_mul(c, p), df_neg(df_mul(sn, q)));
                        xj[t] = df_add(df_mul(sn, p), df_mul(c, q));
                    }
                    df2* vi = v + int64_t(i) * n;
                    df2* vj = v + int64_t(j) * n;
                    for (int t = sub; t < n; t += 8) {
                        const df2 p = vi[t], q = vj[t];
                        vi[t] = df_add(df_mul(c, p), df_neg(df_mul(sn, q)));
                        vj[t] = df_add(df_mul(sn, p), df_mul(c, q));
                    }
                    if (sub == 0) {
                        *rotated = 1;
                        const float cosr = fabsf(g.hi) / (sqrtf(a.hi) * sqrtf(bb.hi));
                        atomicMax(maxcos_bits, __float_as_uint(cosr));  // positive floats order as ints
                    }
                }
            }
            __syncthreads();
        }
        const int done = !*rotated;
        const bool converged = *rotated && __uint_as_float(*maxcos_bits) < 1.0e-7f;
        __syncthreads();
        if (done) break;
        if (converged) {
            ++sweep;
            break;
        }
    }
    return sweep;
}

// sum of one double-float per thread over the CTA (fixed order)
__device__ df2 df_block_sum(df2 v, df2* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = df_add(v, df_shfl_xor(v, o));
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    df2 s{0.f, 0.f};
    for (int w = 0; w < nwarps; ++w) s = df_add(s, red[w]);
    return s;
}

// Preconditioned mixed-precision one-sided Jacobi SVD, one CTA per block (work matrix
// A = M or M^T, m x n with m >= n):
//  1. QR with column pivoting A P = Q R (double-float Householder; A is factored in shared
//     memory when m n double-floats fit the region of the Jacobi matrices, which is free
//     until step 2, and the reflectors are then kept in the global work buffer X);
//  2. FP32 one-sided Jacobi on R^T, accumulating V in float: graded R^T makes cyclic Jacobi
//     converge in a few sweeps (Drmac & Veselic, SIMAX 29, 2008);
//  3. V re-orthonormalised in double-float (one classical Gram-Schmidt pass);
//  4. Y = R^T V and a double-float one-sided Jacobi polish of Y with V accumulation
//     (quadratic convergence from the FP32 start: Higham, Tisseur, Webb & Zhou, SIMAX 42,
//     2021); double-float (FP32 pairs, ~48 bits) runs on the FP32 pipe, which issues 64
//     times the FP64 rate of GB300;
//  5. PY = P Y, then QV = Q [V; 0] (reflectors applied in reverse order; QV in shared
//     memory when it fits there, Y being dead by then).
// Then A = QV * diag(s) * (PY / s)^T: QV is the orthonormal factor on the A-row side,
// PY = (A-column side) * diag(s).  Outputs: QV in W (m x n), PY in V (n x n), singular
// values sorted descending in S with the sorting permutation in perm.  The n x n Jacobi
// matrices live in shared memory when 2 n^2 doubles fit, else in the global scratch P/V.
__global__ void __launch_bounds__(SVD_THREADS)
svd_qrj_kernel(const SvdBlockDesc* __restrict__ desc, const double* __restrict__ src,
               double* __restrict__ X, double* __restrict__ W, double* __restrict__ V,
               double* __restrict__ P, double* __restrict__ S, int* __restrict__ perm,
               int* __restrict__ sweeps_out, int smem_region) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int rotated;
    __shared__ unsigned maxcos;
    __shared__ int piv;
    __shared__ double red[SVD_THREADS / 32];
    const SvdBlockDesc d = desc[blockIdx.x];
    const int m = d.m, n = d.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    // optional phase clocks (diagnostics): 8 stamps per block after the sweep counters
    long long* clk = sweeps_out ? reinterpret_cast<long long*>(sweeps_out + ((gridDim.x + 1) & ~1)) +
                                      blockIdx.x * 8
                                : nullptr;
    auto stamp = [&](int i) {
        if (clk && threadIdx.x == 0) clk[i] = clock64();
    };
    stamp(0);
    // aux: column norms / tau / Gram-Schmidt coefficients (3n doubles) + column perm (n ints)
    double* cn = reinterpret_cast<double*>(smem + smem_region);
    double* tau = cn + n;
    double* h = tau + n;
    int* cp = reinterpret_cast<int*>(h + n);
    float* cnf = reinterpret_cast<float*>(cn);      // column norms (pivoting only needs FP32)
    df2* taud = reinterpret_cast<df2*>(tau);        // Householder tau in double-float
    __shared__ df2 hhd[3];                          // tau, beta, scale of the current reflector
    const bool in_smem = int64_t(2) * n * n * 8 <= smem_region;
    // the m x n work matrix (double-float) in shared memory while the Jacobi region is free
    const bool a_smem = int64_t(m) * n * 8 <= smem_region;
    df2* const Ag = reinterpret_cast<df2*>(X + d.x_off);  // reflectors after step 1
    df2* A = a_smem ? reinterpret_cast<df2*>(smem) : Ag;
    double* Pm = in_smem ? reinterpret_cast<double*>(smem) : P + d.v_off;
    double* Qm = in_smem ? reinterpret_cast<double*>(smem) + int64_t(n) * n : V + d.v_off;
    const double* M = src + d.src_off;
    // 0. A = M (or M^T) in double-float, column norms
    for (int64_t e = threadIdx.x; e < int64_t(m) * n; e += blockDim.x) {
        const int i = int(e % m), k = int(e / m);
        A[e] = df_from_double(d.trans ? M[k + int64_t(i) * d.rows] : M[i + int64_t(k) * d.rows]);
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) cp[j] = j;
    __syncthreads();
    for (int j = warp; j < n; j += nwarps) {
        const df2* a = A + int64_t(j) * m;
        df2 t{0.f, 0.f};
        for (int i = lane; i < m; i += 32) t = df_fma(a[i], a[i], t);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = df_add(t, df_shfl_xor(t, o));
        if (lane == 0) cnf[j] = t.hi;
    }
    __syncthreads();
    // 1. Householder QR with column pivoting, double-float
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            float best = -1.f;
            int bi = k;
            for (int j = k + lane; j < n; j += 32)
                if (cnf[j] > best) { best = cnf[j]; bi = j; }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) piv = bi;
        }
        __syncthreads();
        const int p = piv;
        if (p != k) {
            df2* a = A + int64_t(k) * m;
            df2* b2 = A + int64_t(p) * m;
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const df2 t = a[i]; a[i] = b2[i]; b2[i] = t;
            }
            if (threadIdx.x == 0) {
                const float t = cnf[k]; cnf[k] = cnf[p]; cnf[p] = t;
                const int u = cp[k]; cp[k] = cp[p]; cp[p] = u;
            }
        }
        __syncthreads();
        df2* ak = A + int64_t(k) * m;
        if (warp == 0) {
            df2 sq{0.f, 0.f};
            for (int i = k + 1 + lane; i < m; i += 32) sq = df_fma(ak[i], ak[i], sq);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sq = df_add(sq, df_shfl_xor(sq, o));
            if (lane == 0) {
                const df2 alpha = ak[k];
                if (sq.hi == 0.f) {
                    hhd[0] = df2{0.f, 0.f}; hhd[1] = alpha; hhd[2] = df2{0.f, 0.f};
                } else {
                    df2 beta = df_sqrt(df_fma(alpha, alpha, sq));
                    if (alpha.hi >= 0.f) beta = df_neg(beta);
                    hhd[0] = df_mul(df_add(beta, df_neg(alpha)), df_recip(beta));
                    hhd[1] = beta;
                    hhd[2] = df_recip(df_add(alpha, df_neg(beta)));
                }
                taud[k] = hhd[0];
            }
        }
        __syncthreads();
        const df2 tk = hhd[0], sc = hhd[2];
        for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) ak[i] = df_mul(ak[i], sc);
        __syncthreads();
        if (threadIdx.x == 0) ak[k] = hhd[1];
        for (int j = k + 1 + warp; j < n; j += nwarps) {
            df2* aj = A + int64_t(j) * m;
            df2 w{0.f, 0.f};
            for (int i = k + 1 + lane; i < m; i += 32) w = df_fma(ak[i], aj[i], w);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) w = df_add(w, df_shfl_xor(w, o));
            w = df_mul(df_add(w, aj[k]), tk);
            df2 nrm{0.f, 0.f};
            __syncwarp();  // every lane has read aj[k] before lane 0 updates it
            if (lane == 0) aj[k] = df_add(aj[k], df_neg(w));
            for (int i = k + 1 + lane; i < m; i += 32) {
                const df2 x = df_add(aj[i], df_neg(df_mul(w, ak[i])));
                aj[i] = x;
                nrm = df_fma(x, x, nrm);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) nrm = df_add(nrm, df_shfl_xor(nrm, o));
            if (lane == 0) cnf[j] = nrm.hi;
        }
        __syncthreads();
    }
    if (a_smem) {  // R and the reflectors to the global work buffer; the region is reused
        for (int64_t e = threadIdx.x; e < int64_t(m) * n; e += blockDim.x) Ag[e] = A[e];
        __syncthreads();
        A = Ag;
    }
    stamp(1);
    // 2. R^T as double-float into the W scratch (unused until step 5); FP32 Jacobi on
    //    R^T (n x n lower triangular) in the P region
    df2* rt = reinterpret_cast<df2*>(W + d.x_off);
    // the FP32 pair of n x n arrays fits shared memory up to twice the size the
    // double-float phases need
    const bool f32_smem = int64_t(2) * n * n * 4 <= smem_region;
    float* x32 = f32_smem ? reinterpret_cast<float*>(smem) : reinterpret_cast<float*>(Pm);
    float* v32 = x32 + int64_t(n) * n;
    for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) {
        const int i = int(e % n), j = int(e / n);
        const df2 r = (j <= i) ? A[j + int64_t(i) * m] : df2{0.f, 0.f};  // R^T[i,j] = R[j,i]
        rt[e] = r;
        x32[e] = r.hi;
        v32[e] = (i == j) ? 1.f : 0.f;
    }
    __syncthreads();
    const int sw32 = jacobi_sweeps<float>(x32, v32, n, n, 2.0e-5f, 30, &rotated);
    __syncthreads();
    stamp(2);
    // 3. V in double-float in the Q region, one classical Gram-Schmidt pass (V32 is
    //    orthogonal to ~1e-6, so one pass reaches double-float orthogonality)
    df2* v = reinterpret_cast<df2*>(Qm);
    df2* hd = reinterpret_cast<df2*>(h);
    df2* redd = reinterpret_cast<df2*>(red);
    for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) v[e] = df2{v32[e], 0.f};
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        df2* vj = v + int64_t(j) * n;
        for (int i = warp; i < j; i += nwarps) {
            const df2* vi = v + int64_t(i) * n;
            df2 a{0.f, 0.f};
            for (int t = lane; t < n; t += 32) a = df_fma(vi[t], vj[t], a);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a = df_add(a, df_shfl_xor(a, o));
            if (lane == 0) hd[i] = a;
        }
        __syncthreads();
        df2 ss{0.f, 0.f};
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            df2 acc = vj[t];
            for (int i = 0; i < j; ++i) acc = df_add(acc, df_neg(df_mul(hd[i], v[t + int64_t(i) * n])));
            vj[t] = acc;
            ss = df_fma(acc, acc, ss);
        }
        ss = df_block_sum(ss, redd);
        const df2 inv = ss.hi > 0.f ? df_rsqrt(ss) : df2{0.f, 0.f};
        for (int t = threadIdx.x; t < n; t += blockDim.x) vj[t] = df_mul(vj[t], inv);
        __syncthreads();
    }
    stamp(3);
    // 4. Y = R^T V (double-float) in the P region (the float arrays there are dead), then
    //    the double-float Jacobi polish
    df2* y = reinterpret_cast<df2*>(Pm);
    for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) {
        const int i = int(e % n), j = int(e / n);
        const df2* vj = v + int64_t(j) * n;
        df2 acc{0.f, 0.f};
        for (int k = 0; k <= i; ++k) acc = df_fma(rt[i + int64_t(k) * n], vj[k], acc);
        y[e] = acc;
    }
    __syncthreads();
    stamp(4);
    // rotation threshold above the rounding noise of a double-float dot product
    const float tol = 3.55e-15f * sqrtf(float(n > 1 ? n : 1)) * 32.f;
    const int sw64 = jacobi_sweeps_df(y, v, n, n, tol, 30, &rotated, &maxcos);
    stamp(5);
    __syncthreads();
    // singular values and sorting permutation
    for (int j = warp; j < n; j += nwarps) {
        const df2* yj = y + int64_t(j) * n;
        df2 a{0.f, 0.f};
        for (int t = lane; t < n; t += 32) a = df_fma(yj[t], yj[t], a);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = df_add(a, df_shfl_xor(a, o));
        if (lane == 0) h[j] = sqrt(df_to_double(a));
    }
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double sj = h[j];
        int rank = 0;
        for (int k = 0; k < n; ++k) {
            const double sk = h[k];
            rank += (sk > sj) || (sk == sj && k < j);
        }
        S[d.s_off + rank] = sj;
        perm[d.s_off + rank] = j;
    }
    stamp(6);
    // 5b. PY = P Y into the V output (row cp[r] of P Y is row r of Y).  Y lives in shared
    // memory or in the P scratch, never in V; V (the double-float rotations) is read
    // below, so PY goes through the P scratch when V is not in shared memory.
    double* py = V + d.v_off;
    const bool v_in_V = !in_smem;  // v (Qm) is the V output region itself
    double* pyw = v_in_V ? P + d.v_off : py;
    if (v_in_V) {  // y is in P (Pm): stage PY in the W scratch instead (R^T there is dead)
        double* wt = W + d.x_off;
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) {
            const int r = int(e % n), j = int(e / n);
            wt[cp[r] + int64_t(j) * n] = df_to_double(y[e]);
        }
        __syncthreads();
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) pyw[e] = wt[e];
    } else {
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) {
            const int r = int(e % n), j = int(e / n);
            pyw[cp[r] + int64_t(j) * n] = df_to_double(y[e]);
        }
    }
    __syncthreads();
    // 5a. QV = Q [V; 0] (double-float; in shared memory when it fits, Y being dead), then
    // FP64 into W
    const bool qv_smem = in_smem && int64_t(m) * n * 8 <= smem_region;
    df2* qv = reinterpret_cast<df2*>(W + d.x_off);
    if (qv_smem) {
        // v sits in the upper half of the region that qv will cover: stage it in W first
        df2* vt = qv;
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) vt[e] = v[e];
        __syncthreads();
        df2* qs = reinterpret_cast<df2*>(smem);
        for (int64_t e = threadIdx.x; e < int64_t(m) * n; e += blockDim.x) {
            const int i = int(e % m), j = int(e / m);
            qs[e] = (i < n) ? vt[i + int64_t(j) * n] : df2{0.f, 0.f};
        }
        qv = qs;
    } else {
        for (int64_t e = threadIdx.x; e < int64_t(m) * n; e += blockDim.x) {
            const int i = int(e % m), j = int(e / m);
            qv[e] = (i < n) ? v[i + int64_t(j) * n] : df2{0.f, 0.f};
        }
    }
    __syncthreads();
    for (int k = n - 1; k >= 0; --k) {
        const df2 tk = taud[k];
        if (tk.hi == 0.f) continue;  // uniform: tau lives in shared memory
        const df2* ak = A + int64_t(k) * m;
        for (int j = warp; j < n; j += nwarps) {
            df2* wj = qv + int64_t(j) * m;
            df2 w{0.f, 0.f};
            for (int i = k + 1 + lane; i < m; i += 32) w = df_fma(ak[i], wj[i], w);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) w = df_add(w, df_shfl_xor(w, o));
            w = df_mul(df_add(w, wj[k]), tk);
            __syncwarp();
            if (lane == 0) wj[k] = df_add(wj[k], df_neg(w));
            for (int i = k + 1 + lane; i < m; i += 32) wj[i] = df_add(wj[i], df_neg(df_mul(w, ak[i])));
        }
        __syncthreads();
    }
    {
        double* qvd = W + d.x_off;  // same bytes element by element, or from shared memory
        for (int64_t e = threadIdx.x; e < int64_t(m) * n; e += blockDim.x) {
            const df2 t = qv[e];
            qvd[e] = df_to_double(t);
        }
    }
    if (v_in_V) {  // PY from the P scratch into the V output (v is dead now)
        __syncthreads();
        for (int64_t e = threadIdx.x; e < int64_t(n) * n; e += blockDim.x) py[e] = pyw[e];
    }
    stamp(7);
    if (threadIdx.x == 0 && sweeps_out) sweeps_out[blockIdx.x] = (sw32 << 16) | sw64;
}

// Truncated factors from (QV, PY): for trans = 0 the block is QV diag(s) (PY/s)^T, for
// trans = 1 it is (PY/s) diag(s) QV^T.  ortho 0 keeps the left factor orthonormal,
// ortho 1 the right one; the singular values go to the other side scaled by inv_norm.
__global__ void svd_extract_kernel(const ExtractDesc* __restrict__ desc,
                                   const double* __restrict__ QV, const double* __restrict__ PY,
                                   const double* __restrict__ S, const int* __restrict__ perm,
                                   double* __restrict__ left, double* __restrict__ right,
                                   int ortho, double inv_norm) {
    const ExtractDesc d = desc[blockIdx.x];
    const int rows = d.rows, cols = d.cols, n = d.n, k = d.k;
    const double* qv = QV + d.x_off;  // m x n, m = max(rows, cols)
    const double* py = PY + d.v_off;  // n x n
    const int m = d.trans ? cols : rows;
    const double* s = S + d.s_off;
    const int* pm = perm + d.s_off;
    double* L = left + d.left_off;
    double* R = right + d.right_off;
    const int64_t nl = int64_t(rows) * k;
    for (int64_t e = threadIdx.x; e < nl; e += blockDim.x) {
        const int i = int(e % rows), c = int(e / rows);
        const int pc = pm[c];
        double u;
        if (!d.trans) {
            const double q = qv[i + int64_t(pc) * m];
            u = (ortho == 0) ? q : q * s[c] * inv_norm;
        } else {
            const double y = py[i + int64_t(pc) * n];
            u = (ortho == 0) ? y / s[c] : y * inv_norm;
        }
        L[e] = u;
    }
    const int64_t nr = int64_t(k) * cols;
    for (int64_t e = threadIdx.x; e < nr; e += blockDim.x) {
        const int c = int(e % k), j = int(e / k);
        const int pc = pm[c];
        double w;
        if (!d.trans) {
            const double y = py[j + int64_t(pc) * n];
            w = (ortho == 0) ? y * inv_norm : y / s[c];
        } else {
            const double q = qv[j + int64_t(pc) * m];
            w = (ortho == 0) ? q * s[c] * inv_norm : q;
        }
        R[e] = w;
    }
}

// rows, cols: the complex block; QV / PY hold the realified block's factors (m = 2 rows or
// 2 cols after orientation, n = the realified n)
__global__ void svd_extract_complex_kernel(const ExtractDesc* __restrict__ desc,
                                           const double* __restrict__ QV,
                                           const double* __restrict__ PY,
                                           const double* __restrict__ S,
                                           const int* __restrict__ perm, double* __restrict__ left,
                                           int64_t lplane, double* __restrict__ right,
                                           int64_t rplane, int ortho, double inv_norm) {
    const ExtractDesc d = desc[blockIdx.x];
    const int rows = d.rows, cols = d.cols, n = d.n, k = d.k;
    const double* qv = QV + d.x_off;
    const double* py = PY + d.v_off;
    const int m = d.trans ? 2 * cols : 2 * rows;
    const double* s = S + d.s_off;
    const int* pm = perm + d.s_off;
    double* Lr = left + d.left_off;
    double* Li = Lr + lplane;
    double* Rr = right + d.right_off;
    double* Ri = Rr + rplane;
    const int64_t nl = int64_t(rows) * k;
    for (int64_t e = threadIdx.x; e < nl; e += blockDim.x) {
        const int i = int(e % rows), c = int(e / rows);
        const int pc = pm[2 * c];
        const double sg = s[2 * c];
        double ur, ui;
        if (!d.trans) {  // U column
            const double a = qv[i + int64_t(pc) * m], b = qv[rows + i + int64_t(pc) * m];
            const double f = (ortho == 0) ? 1.0 : sg * inv_norm;
            ur = a * f;
            ui = b * f;
        } else {         // U S column
            const double a = py[i + int64_t(pc) * n], b = py[rows + i + int64_t(pc) * n];
            if (ortho == 0) {
                ur = a / sg;
                ui = b / sg;
            } else {
                ur = a * inv_norm;
                ui = b * inv_norm;
            }
        }
        Lr[e] = ur;
        Li[e] = ui;
    }
    const int64_t nr = int64_t(k) * cols;
    for (int64_t e = threadIdx.x; e < nr; e += blockDim.x) {
        const int c = int(e % k), j = int(e / k);
        const int pc = pm[2 * c];
        const double sg = s[2 * c];
        double vr, vi;  // the entry of S V^H (ortho 0) or V^H (ortho 1)
        if (!d.trans) {  // V S column
            const double a = py[j + int64_t(pc) * n], b = py[cols + j + int64_t(pc) * n];
            if (ortho == 0) {
                vr = a * inv_norm;
                vi = -b * inv_norm;
            } else {
                vr = a / sg;
                vi = -b / sg;
            }
        } else {         // V column
            const double a = qv[j + int64_t(pc) * m], b = qv[cols + j + int64_t(pc) * m];
            const double f = (ortho == 0) ? sg * inv_norm : 1.0;
            vr = a * f;
            vi = -b * f;
        }
        Rr[e] = vr;
        Ri[e] = vi;
    }
}

}  // namespace

void launch_svd_extract_complex(const ExtractDesc* d, int nb, const double* QV, const double* PY,
                                const double* S, const int* perm, double* left, int64_t lplane,
                                double* right, int64_t rplane, int ortho, double inv_norm,
                                cudaStream_t s) {
    if (nb <= 0) return;
    svd_extract_complex_kernel<<<nb, 256, 0, s>>>(d, QV, PY, S, perm, left, lplane, right, rplane,
                                                  ortho, inv_norm);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_svd_jacobi(const SvdBlockDesc* d, int nb, int max_n, const double* src, double* X,
                       double* W, double* V, double* P, double* S, int* perm, int* sweeps_out,
                       cudaStream_t s) {
    if (nb <= 0) return;
    const int64_t limit = 227 * 1024 - 2048;
    const int64_t aux = int64_t(max_n > 0 ? max_n : 1) * (3 * 8 + 4) + 16;
    TN_REQUIRE(aux < 96 * 1024, "SVD block too large (more than 3000 columns)");
    int64_t region = int64_t(2) * max_n * max_n * 8;
    if (region + aux > limit) region = ((limit - aux) / 16) * 16;  // smaller blocks still fit
    const size_t shm = size_t(region + aux);
    TN_CUDA(cudaFuncSetAttribute(svd_qrj_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(shm)));
    svd_qrj_kernel<<<nb, SVD_THREADS, shm, s>>>(d, src, X, W, V, P, S, perm, sweeps_out,
                                                int(region));
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_svd_extract(const ExtractDesc* d, int nb, const double* QV, const double* PY,
                        const double* S, const int* perm, double* left, double* right, int ortho,
                        double inv_norm, cudaStream_t s) {
    if (nb <= 0) return;
    svd_extract_kernel<<<nb, 256, 0, s>>>(d, QV, PY, S, perm, left, right, ortho, inv_norm);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace tn
