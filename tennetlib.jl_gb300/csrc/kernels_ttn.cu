// Kernels of the tree tensor network (TTN) sweep.  Every kernel works on a batch of
// instances at once (blockIdx.y or blockIdx.x selects the instance through a descriptor
// table), so that the lockstep sweep of many independent TTNs issues one launch per step:
//  * batched Krylov vector kernels (fused Gram-Schmidt pass, scaling, linear combination)
//    with warp-shuffle reductions and a deterministic last-block finalisation;
//  * Householder QR: one CTA per matrix for small matrices, and for tall matrices the
//    column kernels of a blocked factorisation (reflector, panel dots, panel update,
//    explicit V and the triangular factor T) whose trailing updates run as grouped GEMMs;
//  * leg permutation (move one leg of a tensor to the end and back) and small helpers.
#include <cuda_runtime.h>

#include "ttn_internal.h"

namespace tn {
namespace {

constexpr int BT = 256;  // threads of the vector kernels

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------------------------
// batched Krylov kernels
// ------------------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(BT)
bgs_pass_kernel(const BGsDesc* __restrict__ descs, double sign, int dots, int norm,
                double* __restrict__ part_all, unsigned* __restrict__ tickets) {
    __shared__ const double* sV[BK_MAX];
    __shared__ double hs[BK_MAX];
    __shared__ double red[BT / 32][K + 1];
    __shared__ int last;
    const BGsDesc& D = descs[blockIdx.y];
    const int kk = D.kk;
    const int64_t n = D.n;
    double* __restrict__ w = D.w;
    if (threadIdx.x < kk) {
        sV[threadIdx.x] = D.V[threadIdx.x];
        hs[threadIdx.x] = D.hin ? sign * D.hin[threadIdx.x] : 0.0;
    }
    __syncthreads();
    double acc[K + 1];
#pragma unroll
    for (int k = 0; k <= K; ++k) acc[k] = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        double x = w[i];
        if (D.hin) {
            for (int k = 0; k < kk; ++k) x = fma(hs[k], sV[k][i], x);
            w[i] = x;
        }
        if (dots) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (k < kk) acc[k] = fma(sV[k][i], x, acc[k]);
        }
        if (norm) acc[K] = fma(x, x, acc[K]);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nres = (dots ? kk : 0) + (norm ? 1 : 0);
#pragma unroll
    for (int k = 0; k <= K; ++k) {
        const double v = warp_sum(acc[k]);
        if (lane == 0) red[wid][k] = v;
    }
    __syncthreads();
    double* part = part_all + int64_t(blockIdx.y) * (BK_MAX + 1) * gridDim.x;
    if (threadIdx.x < nres) {
        const int src = (dots && threadIdx.x < kk) ? threadIdx.x : K;
        double sum = 0.0;
        for (int j = 0; j < BT / 32; ++j) sum += red[j][src];
        part[int64_t(threadIdx.x) * gridDim.x + blockIdx.x] = sum;
    }
    __threadfence();
    __syncthreads();
    unsigned* ticket = tickets + blockIdx.y;
    if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int j = wid; j < nres; j += BT / 32) {
        double sum = 0.0;
        for (int bb = lane; bb < (int)gridDim.x; bb += 32)
            sum += reinterpret_cast<volatile double*>(part)[int64_t(j) * gridDim.x + bb];
        sum = warp_sum(sum);
        if (lane == 0) D.out[j] = sum;
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

__global__ void __launch_bounds__(BT) bscale_kernel(const BScaleDesc* __restrict__ descs) {
    const BScaleDesc& D = descs[blockIdx.y];
    double s = D.scale;
    if (D.denom_sq) {
        const double q = *D.denom_sq;
        s = q > 0.0 ? D.scale / sqrt(q) : 0.0;
    }
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < D.n; i += stride) {
        const double v = D.src[i] * s;
        D.dst[i] = v;
        if (D.dst2) D.dst2[i] = v;
    }
}

__global__ void __launch_bounds__(BT) blincomb_kernel(const BLinDesc* __restrict__ descs) {
    __shared__ const double* sV[BK_MAX];
    __shared__ double cs[BK_MAX];
    const BLinDesc& D = descs[blockIdx.y];
    if (threadIdx.x < D.kk) {
        sV[threadIdx.x] = D.V[threadIdx.x];
        cs[threadIdx.x] = D.coef[threadIdx.x];
    }
    __syncthreads();
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < D.n; i += stride) {
        double x = 0.0;
        for (int k = 0; k < D.kk; ++k) x = fma(cs[k], sV[k][i], x);
        D.dst[i] = x;
    }
}

// ------------------------------------------------------------------------------------
// leg permutation: t viewed as (P, D, Q) <-> (P, Q, D)
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(BT) permute_kernel(const PermDesc* __restrict__ descs) {
    const PermDesc& D = descs[blockIdx.y];
    const int64_t total = D.P * D.D * D.Q;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
        // e indexes the (P, Q, D) side
        const int64_t p = e % D.P;
        const int64_t r = e / D.P;
        const int64_t q = r % D.Q;
        const int64_t a = r / D.Q;
        const int64_t f = p + D.P * (a + D.D * q);  // (P, D, Q) side
        if (D.to_end) D.dst[e] = D.src[f];
        else          D.dst[f] = D.src[e];
    }
}

__global__ void __launch_bounds__(BT) concat_kernel(const ConcatDesc* __restrict__ descs) {
    const ConcatDesc& D = descs[blockIdx.y];
    const int64_t Dt = D.D1 + D.D2;
    const int64_t total = D.P * Dt * D.Q;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
        const int64_t p = e % D.P;
        const int64_t r = e / D.P;
        const int64_t k = r % Dt;
        const int64_t q = r / Dt;
        D.dst[e] = k < D.D1 ? D.a[p + D.P * (k + D.D1 * q)]
                            : D.b[p + D.P * ((k - D.D1) + D.D2 * q)];
    }
}

// ------------------------------------------------------------------------------------
// Householder reflector of x = (alpha, tail), LAPACK dlarfg convention:
//   H = I - tau v v^T, v = (1, tail * scale), H x = (beta, 0).
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void make_reflector(double alpha, double sig, double& tau,
                                               double& scale, double& beta) {
    if (sig == 0.0) {
        tau = 0.0;
        scale = 0.0;
        beta = alpha;
        return;
    }
    const double nrm = sqrt(alpha * alpha + sig);
    beta = alpha >= 0.0 ? -nrm : nrm;
    tau = (beta - alpha) / beta;
    scale = 1.0 / (alpha - beta);
}

__device__ __forceinline__ double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (wid == 0) {
        s = lane < int(blockDim.x >> 5) ? red[lane] : 0.0;
        s = warp_sum(s);
        if (lane == 0) red[32] = s;
    }
    __syncthreads();
    return red[32];
}

// One CTA factors one m x n matrix A (lda = m): R (kmin x n) is written out, A is
// overwritten by the explicit Q (m x kmin), kmin = min(m, n).  Unblocked Householder QR
// (LAPACK dgeqr2) followed by the backward accumulation of Q (dorg2r).
__global__ void __launch_bounds__(1024) qr_small_kernel(const QrDesc* __restrict__ descs) {
    __shared__ double red[33];
    __shared__ double sc[3];
    const QrDesc& D = descs[blockIdx.x];
    double* __restrict__ A = D.A;
    double* __restrict__ tau = D.tau;
    const int m = D.m, n = D.n, kmin = m < n ? m : n;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < kmin; ++j) {
        double* col = A + int64_t(j) * m;
        double s = 0.0;
        for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) s = fma(col[i], col[i], s);
        s = block_sum(s, red);
        if (threadIdx.x == 0) {
            double t, scale, beta;
            make_reflector(col[j], s, t, scale, beta);
            sc[0] = t;
            sc[1] = scale;
            sc[2] = beta;
        }
        __syncthreads();
        const double t = sc[0], scale = sc[1];
        for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] *= scale;
        __syncthreads();
        if (t != 0.0) {
            for (int k = j + 1 + wid; k < n; k += nw) {
                double* ck = A + int64_t(k) * m;
                double d = lane == 0 ? ck[j] : 0.0;
                for (int i = j + 1 + lane; i < m; i += 32) d = fma(col[i], ck[i], d);
                d = warp_sum(d) * t;
                if (lane == 0) ck[j] -= d;
                for (int i = j + 1 + lane; i < m; i += 32) ck[i] = fma(-d, col[i], ck[i]);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            col[j] = sc[2];
            tau[j] = t;
        }
        __syncthreads();
    }
    // R = upper triangle of the first kmin rows
    for (int64_t e = threadIdx.x; e < int64_t(kmin) * n; e += blockDim.x) {
        const int r = int(e % kmin), c = int(e / kmin);
        D.R[e] = r <= c ? A[r + int64_t(c) * m] : 0.0;
    }
    __syncthreads();
    // Q = H_0 ... H_{kmin-1} [I; 0] in place (dorg2r)
    for (int i = kmin - 1; i >= 0; --i) {
        double* ci = A + int64_t(i) * m;
        const double t = tau[i];
        for (int k = i + 1 + wid; k < kmin; k += nw) {
            double* ck = A + int64_t(k) * m;
            double d = lane == 0 ? ck[i] : 0.0;
            for (int r = i + 1 + lane; r < m; r += 32) d = fma(ci[r], ck[r], d);
            d = warp_sum(d) * t;
            if (lane == 0) ck[i] -= d;
            for (int r = i + 1 + lane; r < m; r += 32) ck[r] = fma(-d, ci[r], ck[r]);
        }
        __syncthreads();
        for (int r = threadIdx.x; r < m; r += blockDim.x) {
            if (r > i) ci[r] *= -t;
            else if (r == i) ci[r] = 1.0 - t;
            else ci[r] = 0.0;
        }
        __syncthreads();
    }
}

// ---- blocked Householder: column kernels (grid: parts x instances) -------------------
// column norm of A[j+1:m, j]; the last block forms the reflector of column j
__global__ void __launch_bounds__(BT) hh_norm_kernel(const HhDesc* __restrict__ descs, int j) {
    __shared__ double red[33];
    __shared__ int last;
    const HhDesc& D = descs[blockIdx.y];
    if (j >= D.kmin) return;
    const double* col = D.A + int64_t(j) * D.m;
    double s = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = j + 1 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < D.m; i += stride)
        s = fma(col[i], col[i], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) D.part[blockIdx.x] = s;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(D.ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last || threadIdx.x >= 32) return;
    __threadfence();
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32)
        t += reinterpret_cast<volatile double*>(D.part)[b];
    t = warp_sum(t);
    if (threadIdx.x == 0) {
        double tau, scale, beta;
        make_reflector(col[j], t, tau, scale, beta);
        double* sc = D.scal + 4 * (j & 1);
        sc[0] = tau;
        sc[1] = scale;
        sc[2] = beta;
        D.tau[j] = tau;
        *D.ticket = 0u;
    }
}

// w_k = A[j, k] + scale * sum_{i>j} A[i, j] A[i, k] for the panel columns k in (j, pend);
// the last block stores tau * w_k in D.wv[k - j - 1]
__global__ void __launch_bounds__(BT) hh_dots_kernel(const HhDesc* __restrict__ descs, int j,
                                                     int pend) {
    __shared__ double red[BT / 32][HH_B];
    __shared__ int last;
    const HhDesc& D = descs[blockIdx.y];
    const int pe = pend < D.kmin ? pend : D.kmin;
    const int nk = pe - j - 1;
    if (j >= D.kmin || nk <= 0) return;
    const double* col = D.A + int64_t(j) * D.m;
    double acc[HH_B];
#pragma unroll
    for (int c = 0; c < HH_B; ++c) acc[c] = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = j + 1 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < D.m; i += stride) {
        const double v = col[i];
#pragma unroll
        for (int c = 0; c < HH_B; ++c)
            if (c < nk) acc[c] = fma(v, D.A[i + int64_t(j + 1 + c) * D.m], acc[c]);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < HH_B; ++c) {
        const double v = warp_sum(acc[c]);
        if (lane == 0) red[wid][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < nk) {
        double s = 0.0;
        for (int w = 0; w < BT / 32; ++w) s += red[w][threadIdx.x];
        D.part[int64_t(threadIdx.x) * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(D.ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    const double* sc = D.scal + 4 * (j & 1);
    const double tau = sc[0], scale = sc[1];
    for (int c = wid; c < nk; c += BT / 32) {
        double s = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32)
            s += reinterpret_cast<volatile double*>(D.part)[int64_t(c) * gridDim.x + b];
        s = warp_sum(s);
        if (lane == 0) D.wv[c] = tau * (D.A[j + int64_t(j + 1 + c) * D.m] + scale * s);
    }
    __syncthreads();
    if (threadIdx.x == 0) *D.ticket = 0u;
}

// A[i, k] -= v_i (tau w_k) for i >= j, k in (j, pend); then column j holds v (scaled) below
// the diagonal and beta on it.  When column j + 1 is in the panel, the same pass sums the
// squares of its updated entries below the diagonal and the last block forms its reflector
// (the work of hh_norm_kernel for column j + 1).
__global__ void __launch_bounds__(BT) hh_update_kernel(const HhDesc* __restrict__ descs, int j,
                                                       int pend) {
    __shared__ double red[33];
    __shared__ int last;
    const HhDesc& D = descs[blockIdx.y];
    if (j >= D.kmin) return;
    const int pe = pend < D.kmin ? pend : D.kmin;
    const int nk = pe - j - 1;
    double* col = D.A + int64_t(j) * D.m;
    const double* sc = D.scal + 4 * (j & 1);
    const double scale = sc[1], beta = sc[2];
    double nrm = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = j + int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < D.m; i += stride) {
        const double v = i == j ? 1.0 : col[i] * scale;
        for (int c = 0; c < nk; ++c) {
            double* a = D.A + i + int64_t(j + 1 + c) * D.m;
            const double x = fma(-v, D.wv[c], *a);
            *a = x;
            if (c == 0 && i > j + 1) nrm = fma(x, x, nrm);
        }
        col[i] = i == j ? beta : v;
    }
    if (nk <= 0) return;
    nrm = block_sum(nrm, red);
    if (threadIdx.x == 0) D.part[blockIdx.x] = nrm;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(D.ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last || threadIdx.x >= 32) return;
    __threadfence();
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32)
        t += reinterpret_cast<volatile double*>(D.part)[b];
    t = warp_sum(t);
    if (threadIdx.x == 0) {
        const double alpha = reinterpret_cast<volatile double*>(D.A)[(j + 1) + int64_t(j + 1) * D.m];
        double tau, sca, bet;
        make_reflector(alpha, t, tau, sca, bet);
        double* sn = D.scal + 4 * ((j + 1) & 1);
        sn[0] = tau;
        sn[1] = sca;
        sn[2] = bet;
        D.tau[j + 1] = tau;
        *D.ticket = 0u;
    }
}

// ---- cooperative panel factorisation -------------------------------------------------
// All CTAs of one launch are co-resident (cooperative launch).  Instance i owns the CTAs
// [cta0, cta0 + ncta), each a contiguous chunk of the rows [p0, m).  Per column: partial
// norms -> barrier -> every CTA forms the same reflector -> partial dots -> barrier ->
// every CTA sums the same partials in the same order -> local update.  Waits are bounded
// (about a second of clocks); a wait that gives up sets *err and the kernel returns.
constexpr long long COOP_WAIT = 2000000000LL;

__device__ __forceinline__ bool inst_barrier(unsigned* bar, unsigned target, int* err,
                                             int* s_fail) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        const long long t0 = clock64();
        while (true) {
            if (*reinterpret_cast<volatile unsigned*>(bar) >= target) break;
            if (*reinterpret_cast<volatile int*>(err) != 0 || clock64() - t0 > COOP_WAIT) {
                atomicExch(err, 2);
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

// One grid barrier per column: every CTA reduces, over its own rows below j, sigma^2 = sum x_i^2
// and s_c = sum x_i A[i, c] for the panel columns c right of j (x = column j), and the owner of
// row j publishes A[j, j..pe).  After the barrier every CTA forms the same reflector
// (beta, tau, scale = 1 / (alpha - beta)) and w_c = tau (A[j, c] + scale s_c) = tau v^T A[:, c],
// then updates its rows.  Partials and the published row are double-buffered by column parity:
// a CTA can only reuse a buffer after the next barrier, which every CTA reaches only once it
// has read the totals of the previous column.
__global__ void __launch_bounds__(BT, 2)
hh_panel_coop_kernel(const HhDesc* __restrict__ descs, int ninst, int p0, int* err) {
    constexpr int W1 = HH_B + 1;
    __shared__ double red[BT / 32][W1];
    __shared__ double tot[W1];
    __shared__ double wsh[HH_B];
    __shared__ double sc[3];
    __shared__ int s_fail;
    int inst = -1;
    for (int i = 0; i < ninst; ++i)
        if (int(blockIdx.x) >= descs[i].cta0 && int(blockIdx.x) < descs[i].cta0 + descs[i].ncta) inst = i;
    if (inst < 0) return;
    const HhDesc& D = descs[inst];
    if (p0 >= D.kmin) return;  // uniform over the instance's CTAs
    const int G = D.ncta, g = int(blockIdx.x) - D.cta0;
    // test hook (tn_ctx_inject_wait_timeout, code 3): the first CTA of the first instance leaves
    // before its first barrier, so that the other CTAs' barrier waits run out
    if (threadIdx.x == 0) s_fail = (inst == 0 && g == 0 && atomicCAS(err + 1, 3, 0) == 3) ? 1 : 0;
    __syncthreads();
    if (s_fail) return;
    const int pe = (p0 + HH_B) < D.kmin ? (p0 + HH_B) : D.kmin;
    const int64_t m = D.m;
    const int64_t chunk = (m - p0 + G - 1) / G;
    const int64_t r0 = p0 + int64_t(g) * chunk;
    const int64_t r1 = (r0 + chunk) < m ? (r0 + chunk) : m;
    double* parts = D.part;                          // 2 x G x W1: [sigma^2, s_0, s_1, ...]
    double* pubs = D.part + 2 * int64_t(G) * W1;     // 2 x W1: A[j, j], A[j, j+1], ...
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned nb = 0;
    for (int j = p0; j < pe; ++j) {
        const int buf = j & 1;
        double* col = D.A + int64_t(j) * m;
        const int nk = pe - j - 1;
        double ss = 0.0;
        double acc[HH_B];
#pragma unroll
        for (int c = 0; c < HH_B; ++c) acc[c] = 0.0;
        for (int64_t i = (r0 > j + 1 ? r0 : j + 1) + threadIdx.x; i < r1; i += BT) {
            const double x = col[i];
            ss = fma(x, x, ss);
            const double* arow = D.A + i + int64_t(j + 1) * m;
            // groups of 8 columns past nk are skipped whole
#pragma unroll
            for (int cg = 0; cg < HH_B; cg += 8) {
                if (cg >= nk) break;
#pragma unroll
                for (int c = cg; c < cg + 8; ++c)
                    if (c < nk) acc[c] = fma(x, arow[int64_t(c) * m], acc[c]);
            }
        }
        ss = warp_sum(ss);
        if (lane == 0) red[wid][0] = ss;
#pragma unroll
        for (int c = 0; c < HH_B; ++c) {
            if (c >= ((nk + 7) & ~7)) break;
            const double v = warp_sum(acc[c]);
            if (lane == 0) red[wid][1 + c] = v;
        }
        __syncthreads();
        if (threadIdx.x <= nk) {
            double t = 0.0;
            for (int w = 0; w < BT / 32; ++w) t += red[w][threadIdx.x];
            parts[(int64_t(buf) * G + g) * W1 + threadIdx.x] = t;
            if (j >= r0 && j < r1) pubs[buf * W1 + threadIdx.x] = col[j + int64_t(threadIdx.x) * m];
        }
        if (!inst_barrier(D.bar, (++nb) * unsigned(G), err, &s_fail)) return;
        // totals: every CTA sums the G partials in the same fixed order (lane-strided, then a
        // warp tree), so the reflectors are identical everywhere
        // (L2 loads: the partials were written by other SMs before the barrier's fences)
        const double* pall = parts + int64_t(buf) * G * W1;
        const double* pub = pubs + buf * W1;
        for (int c = wid; c <= nk; c += BT / 32) {
            double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
            int b = lane;
            for (; b + 96 < G; b += 128) {
                t0 += __ldcg(pall + int64_t(b) * W1 + c);
                t1 += __ldcg(pall + int64_t(b + 32) * W1 + c);
                t2 += __ldcg(pall + int64_t(b + 64) * W1 + c);
                t3 += __ldcg(pall + int64_t(b + 96) * W1 + c);
            }
            for (; b < G; b += 32) t0 += __ldcg(pall + int64_t(b) * W1 + c);
            const double t = warp_sum((t0 + t1) + (t2 + t3));
            if (lane == 0) tot[c] = t;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double tau, scale, beta;
            make_reflector(__ldcg(pub), tot[0], tau, scale, beta);
            sc[0] = tau;
            sc[1] = scale;
            sc[2] = beta;
        }
        __syncthreads();
        const double tau = sc[0], scale = sc[1], beta = sc[2];
        if (threadIdx.x < nk) wsh[threadIdx.x] = tau * (__ldcg(pub + 1 + threadIdx.x) + scale * tot[1 + threadIdx.x]);
        __syncthreads();
        const int64_t i0 = r0 > j ? r0 : j;
        if (nk > 0) {
            for (int64_t i = i0 + threadIdx.x; i < r1; i += BT) {
                const double v = i == j ? 1.0 : col[i] * scale;
                for (int c = 0; c < nk; ++c) {
                    double* a = D.A + i + int64_t(j + 1 + c) * m;
                    *a = fma(-v, wsh[c], *a);
                }
            }
        }
        for (int64_t i = i0 + threadIdx.x; i < r1; i += BT) col[i] = i == j ? beta : col[i] * scale;
        if (g == 0 && threadIdx.x == 0) D.tau[j] = tau;
        __syncthreads();
    }
}

// columns [p0, p0 + pb) of the explicit unit lower-trapezoidal V (m x kmin, ld m): zero above
// the diagonal, one on it, the stored reflector below
__global__ void __launch_bounds__(BT) hh_build_v_kernel(const HhDesc* __restrict__ descs, int p0,
                                                        int pb_max) {
    const HhDesc& D = descs[blockIdx.y];
    if (p0 >= D.kmin) return;
    const int pb = (D.kmin - p0) < pb_max ? (D.kmin - p0) : pb_max;
    const int64_t m = D.m;
    const int64_t total = m * pb;
    double* V = D.V + p0 * m;
    const double* A = D.A + p0 * m;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
        const int64_t r = e % m;
        const int64_t dg = p0 + e / m;  // the diagonal row of this column
        V[e] = r < dg ? 0.0 : (r == dg ? 1.0 : A[e]);
    }
}

// Gram matrix G = V^T V of the panel (partial sums per block, deterministic finalisation)
// and the negated triangular factor -T of the block reflector I - V T V^T (LAPACK dlarft,
// forward, columnwise), written to D.T (HH_B x HH_B, column-major, ld HH_B)
__global__ void __launch_bounds__(HH_B * HH_B) hh_gram_t_kernel(const HhDesc* __restrict__ descs,
                                                                int p0, int pb_max) {
    __shared__ double tile[64][HH_B + 1];
    __shared__ double G[HH_B][HH_B + 1];
    __shared__ double T[HH_B][HH_B + 1];
    __shared__ int last;
    const HhDesc& D = descs[blockIdx.y];
    if (p0 >= D.kmin) return;
    const int pb = (D.kmin - p0) < pb_max ? (D.kmin - p0) : pb_max;
    const int64_t rows = D.m - p0;
    const double* V = D.V + hh_panel_voff(D.m, p0);
    const int64_t ldv = D.m;
    const int a = threadIdx.x % HH_B, b = threadIdx.x / HH_B;
    // the Gram is symmetric: threads [0, NPAIR) take the pairs ga <= gb (whole warps idle past)
    constexpr int NPAIR = HH_B * (HH_B + 1) / 2;
    const int t = threadIdx.x;
    int gb = int((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
    while ((gb + 1) * (gb + 2) / 2 <= t) ++gb;
    while (gb > 0 && gb * (gb + 1) / 2 > t) --gb;
    const int ga = t - gb * (gb + 1) / 2;
    const bool mine = t < NPAIR;
    double acc = 0.0;
    for (int64_t r0 = int64_t(blockIdx.x) * 64; r0 < rows; r0 += int64_t(gridDim.x) * 64) {
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * HH_B; e += blockDim.x) {
            const int rr = e % 64, c = e / 64;
            const int64_t r = r0 + rr;
            tile[rr][c] = (r < rows && c < pb) ? V[r + int64_t(c) * ldv] : 0.0;
        }
        __syncthreads();
        if (mine) {
#pragma unroll 8
            for (int rr = 0; rr < 64; ++rr) acc = fma(tile[rr][ga], tile[rr][gb], acc);
        }
    }
    D.part[int64_t(blockIdx.x) * (HH_B * HH_B) + threadIdx.x] = acc;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(D.ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (mine) {
        double s = 0.0;
        for (int bb = 0; bb < (int)gridDim.x; ++bb)
            s += reinterpret_cast<volatile double*>(D.part)[int64_t(bb) * (HH_B * HH_B) + threadIdx.x];
        G[ga][gb] = s;
        G[gb][ga] = s;
    }
    T[a][b] = 0.0;
    __syncthreads();
    // T[0:j, j] = -tau_j T[0:j, 0:j] G[0:j, j]; T[j, j] = tau_j
    for (int jj = 0; jj < pb; ++jj) {
        const double tj = D.tau[p0 + jj];
        double v = 0.0;
        if (threadIdx.x < jj) {
            const int r = threadIdx.x;
            for (int c = r; c < jj; ++c) v = fma(T[r][c], G[c][jj], v);
        }
        __syncthreads();
        if (threadIdx.x < jj) T[threadIdx.x][jj] = -tj * v;
        if (threadIdx.x == 0) T[jj][jj] = tj;
        __syncthreads();
    }
    D.T[int64_t(p0 / HH_B) * HH_B * HH_B + a + b * HH_B] = (a < pb && b < pb) ? -T[a][b] : 0.0;
    if (threadIdx.x == 0) *D.ticket = 0u;
}

// -T of the whole block reflector H_0 H_1 ... H_{kmin-1} = I - V T V^T (forward,
// columnwise) from the per-panel factors T_p and G = V^T V, one 32-column block at a time:
// T[0:q0, q] = -T[0:q0, 0:q0] (G[0:q0, q] T_q) (Schreiber and Van Loan's merge of two block
// reflectors).  One CTA per instance; Y = G[0:q0, q] T_q goes through a global scratch
// (row-major, ld HH_B) so that every row's 32 products come from two cache lines.
constexpr int TALL_THREADS = 256;
__global__ void __launch_bounds__(TALL_THREADS) hh_tall_kernel(const HhDesc* __restrict__ descs) {
    const HhDesc& D = descs[blockIdx.x];
    const int k = D.kmin;
    double* T = D.Tall;  // holds +T while it is built, negated at the end
    const double* G = D.G;
    double* Y = D.Yscr;
    __shared__ double Tq[HH_B][HH_B + 1];
    const int np = (k + HH_B - 1) / HH_B;
    // diagonal blocks +T_p (the per-panel factors hold -T_p), zero elsewhere
    for (int64_t e = threadIdx.x; e < int64_t(k) * k; e += blockDim.x) {
        const int r = int(e % k), c = int(e / k), p = c / HH_B;
        T[e] = r / HH_B == p
                   ? -D.T[int64_t(p) * HH_B * HH_B + (r % HH_B) + (c % HH_B) * HH_B]
                   : 0.0;
    }
    __syncthreads();
    for (int q = 1; q < np; ++q) {
        const int q0 = q * HH_B;
        const int qb = (k - q0) < HH_B ? (k - q0) : HH_B;
        for (int e = threadIdx.x; e < HH_B * HH_B; e += blockDim.x)
            Tq[e % HH_B][e / HH_B] = -D.T[int64_t(q) * HH_B * HH_B + e];
        __syncthreads();
        // Y (q0 x HH_B) = G[0:q0, q0:q0+qb] T_q (T_q upper triangular; zero columns past qb)
        for (int e = threadIdx.x; e < q0 * HH_B; e += blockDim.x) {
            const int r = e % q0, c = e / q0;
            double y = 0.0;
            if (c < qb)
                for (int cc = 0; cc <= c; ++cc) y = fma(G[r + int64_t(q0 + cc) * k], Tq[cc][c], y);
            Y[int64_t(r) * HH_B + c] = y;
        }
        __syncthreads();
        // T[0:q0, q0:q0+qb] = -T[0:q0, 0:q0] Y (T upper triangular)
        for (int r = threadIdx.x; r < q0; r += blockDim.x) {
            double acc[HH_B];
#pragma unroll
            for (int c = 0; c < HH_B; ++c) acc[c] = 0.0;
            for (int cp = r; cp < q0; ++cp) {
                const double t = T[r + int64_t(cp) * k];
                const double* y = Y + int64_t(cp) * HH_B;
#pragma unroll
                for (int c = 0; c < HH_B; ++c) acc[c] = fma(t, y[c], acc[c]);
            }
#pragma unroll
            for (int c = 0; c < HH_B; ++c)
                if (c < qb) T[r + int64_t(q0 + c) * k] = -acc[c];
        }
        __syncthreads();
    }
    for (int64_t e = threadIdx.x; e < int64_t(k) * k; e += blockDim.x) T[e] = -T[e];
}

// R (kmin x n) = upper triangle of the factored A; Q (m x kmin, ld m) = [I; 0]
__global__ void __launch_bounds__(BT) hh_finish_kernel(const HhDesc* __restrict__ descs) {
    const HhDesc& D = descs[blockIdx.y];
    const int64_t totr = int64_t(D.kmin) * D.n;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < totr; e += stride) {
        const int r = int(e % D.kmin), c = int(e / D.kmin);
        D.R[e] = r <= c ? D.A[r + int64_t(c) * D.m] : 0.0;
    }
}

__global__ void __launch_bounds__(BT) hh_init_q_kernel(const HhDesc* __restrict__ descs) {
    const HhDesc& D = descs[blockIdx.y];
    const int64_t tot = int64_t(D.m) * D.kmin;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < tot; e += stride) {
        const int64_t r = e % D.m, c = e / D.m;
        D.Q[e] = r == c ? 1.0 : 0.0;
    }
}

int grid_x(int64_t n, int cap) {
    int64_t g = (n + BT - 1) / BT;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return int(g);
}

}  // namespace

int ttn_parts() { return TTN_PARTS; }

void launch_bgs_pass(const BGsDesc* d, int ninst, int kmax, int64_t nmax, double sign, bool dots,
                     bool norm, double* part, unsigned* tickets, cudaStream_t s) {
    if (ninst <= 0) return;
    TN_REQUIRE(kmax <= BK_MAX, "too many Krylov vectors for one batched kernel");
    const dim3 g(grid_x(nmax, TTN_PARTS), ninst);
    const int dd = dots ? 1 : 0, nm = norm ? 1 : 0;
    if (kmax <= 4)
        bgs_pass_kernel<4><<<g, BT, 0, s>>>(d, sign, dd, nm, part, tickets);
    else if (kmax <= 8)
        bgs_pass_kernel<8><<<g, BT, 0, s>>>(d, sign, dd, nm, part, tickets);
    else if (kmax <= 16)
        bgs_pass_kernel<16><<<g, BT, 0, s>>>(d, sign, dd, nm, part, tickets);
    else
        bgs_pass_kernel<32><<<g, BT, 0, s>>>(d, sign, dd, nm, part, tickets);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_bscale(const BScaleDesc* d, int ninst, int64_t nmax, cudaStream_t s) {
    if (ninst <= 0) return;
    bscale_kernel<<<dim3(grid_x(nmax, 2 * TTN_PARTS), ninst), BT, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_blincomb(const BLinDesc* d, int ninst, int64_t nmax, cudaStream_t s) {
    if (ninst <= 0) return;
    blincomb_kernel<<<dim3(grid_x(nmax, 2 * TTN_PARTS), ninst), BT, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_permute(const PermDesc* d, int ninst, int64_t nmax, cudaStream_t s) {
    if (ninst <= 0) return;
    permute_kernel<<<dim3(grid_x(nmax, 4 * TTN_PARTS), ninst), BT, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_concat(const ConcatDesc* d, int ninst, int64_t nmax, cudaStream_t s) {
    if (ninst <= 0) return;
    concat_kernel<<<dim3(grid_x(nmax, 4 * TTN_PARTS), ninst), BT, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_qr_small(const QrDesc* d, int ninst, cudaStream_t s) {
    if (ninst <= 0) return;
    qr_small_kernel<<<ninst, 1024, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_hh_column(const HhDesc* d, int ninst, int64_t mmax, int j, int p0, int pend,
                      cudaStream_t s) {
    const int g = grid_x(mmax, 4 * TTN_PARTS);
    if (j == p0) {  // inside a panel the update of column j - 1 formed this reflector
        hh_norm_kernel<<<dim3(g, ninst), BT, 0, s>>>(d, j);
        TN_CUDA(cudaGetLastError());
        count_launch();
    }
    hh_dots_kernel<<<dim3(g, ninst), BT, 0, s>>>(d, j, pend);
    TN_CUDA(cudaGetLastError());
    hh_update_kernel<<<dim3(g, ninst), BT, 0, s>>>(d, j, pend);
    TN_CUDA(cudaGetLastError());
    count_launch(2);
}

// co-resident CTAs of the cooperative panel kernel on the current device (cached per device)
int hh_coop_capacity() {
    constexpr int MAXDEV = 64;
    static int cap[MAXDEV] = {};
    int dev = 0;
    TN_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAXDEV) throw Error(-1, "device index out of range");
    if (cap[dev] <= 0) {
        int nsm = 0, per = 0;
        TN_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        TN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, hh_panel_coop_kernel, BT, 0));
        cap[dev] = nsm * per;
    }
    return cap[dev];
}

void launch_hh_panel_coop(const HhDesc* d, int ninst, int nctas, int p0, int* err,
                          cudaStream_t s) {
    void* args[] = {(void*)&d, (void*)&ninst, (void*)&p0, (void*)&err};
    TN_CUDA(cudaLaunchCooperativeKernel((const void*)hh_panel_coop_kernel, dim3(nctas), dim3(BT),
                                        args, 0, s));
    count_launch();
}

void launch_hh_panel_end(const HhDesc* d, int ninst, int64_t mmax, int p0, int pb,
                         cudaStream_t s) {
    hh_build_v_kernel<<<dim3(grid_x(mmax * pb, 2 * TTN_PARTS), ninst), BT, 0, s>>>(d, p0, pb);
    TN_CUDA(cudaGetLastError());
    int g = int((mmax + 63) / 64);
    if (g > TTN_PARTS) g = TTN_PARTS;
    if (g < 1) g = 1;
    hh_gram_t_kernel<<<dim3(g, ninst), HH_B * HH_B, 0, s>>>(d, p0, pb);
    TN_CUDA(cudaGetLastError());
    count_launch(2);
}

void launch_hh_tall(const HhDesc* d, int ninst, cudaStream_t s) {
    if (ninst <= 0) return;
    hh_tall_kernel<<<ninst, TALL_THREADS, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_hh_finish(const HhDesc* d, int ninst, int64_t mnmax, cudaStream_t s) {
    hh_finish_kernel<<<dim3(grid_x(mnmax, 2 * TTN_PARTS), ninst), BT, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    hh_init_q_kernel<<<dim3(grid_x(mnmax, 2 * TTN_PARTS), ninst), BT, 0, s>>>(d);
    TN_CUDA(cudaGetLastError());
    count_launch(2);
}

}  // namespace tn
