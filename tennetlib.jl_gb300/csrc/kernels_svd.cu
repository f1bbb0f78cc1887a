// Batched FP64 one-sided Jacobi SVD of the charge blocks of a two-site tensor
// (Hestenes' method with round-robin parallel ordering), followed by the extraction of the
// truncated factors into the left/right site tensors.  The truncation decision itself is
// made on the host from the sorted singular values (tiny, integer-valued result).
#include <cuda_runtime.h>

#include "tn_internal.h"

namespace tn {
namespace {

constexpr int SVD_THREADS = 512;
constexpr int SVD_MAX_SWEEPS = 40;

__global__ void svd_prepare_kernel(const SvdBlockDesc* __restrict__ desc,
                                   const double* __restrict__ src, double* __restrict__ X,
                                   double* __restrict__ V) {
    const SvdBlockDesc d = desc[blockIdx.x];
    const double* M = src + d.src_off;
    double* x = X + d.x_off;
    double* v = V + d.v_off;
    const int64_t mn = int64_t(d.m) * d.n;
    for (int64_t e = threadIdx.x; e < mn; e += blockDim.x) {
        const int i = int(e % d.m), j = int(e / d.m);
        x[e] = d.trans ? M[j + int64_t(i) * d.rows] : M[i + int64_t(j) * d.rows];
    }
    const int64_t nn = int64_t(d.n) * d.n;
    for (int64_t e = threadIdx.x; e < nn; e += blockDim.x) {
        const int i = int(e % d.n), j = int(e / d.n);
        v[e] = (i == j) ? 1.0 : 0.0;
    }
}

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Round-robin tournament: nn (even) players, round r in [0, nn-1), pair k in [0, nn/2).
__device__ __forceinline__ void rr_pair(int nn, int r, int k, int& i, int& j) {
    auto player = [&](int pos) { return pos == 0 ? 0 : 1 + ((pos - 1 + r) % (nn - 1)); };
    i = player(k);
    j = player(nn - 1 - k);
    if (i > j) { int t = i; i = j; j = t; }
}

__global__ void __launch_bounds__(SVD_THREADS)
svd_jacobi_kernel(const SvdBlockDesc* __restrict__ desc, double* __restrict__ X,
                  double* __restrict__ V, double* __restrict__ S, int* __restrict__ perm,
                  int* __restrict__ sweeps_out) {
    extern __shared__ double raw[];  // n column norms
    __shared__ int rotated;
    const SvdBlockDesc d = desc[blockIdx.x];
    const int m = d.m, n = d.n;
    double* x = X + d.x_off;
    double* v = V + d.v_off;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const double tol = 2.220446049250313e-16 * sqrt(double(m > 1 ? m : 1)) * 2.0;
    const int nn = n + (n & 1);
    int sweep = 0;
    if (n > 1) {
        for (sweep = 0; sweep < SVD_MAX_SWEEPS; ++sweep) {
            if (threadIdx.x == 0) rotated = 0;
            __syncthreads();
            for (int r = 0; r < nn - 1; ++r) {
                for (int k = warp; k < nn / 2; k += nwarps) {
                    int i, j;
                    rr_pair(nn, r, k, i, j);
                    if (j >= n) continue;
                    double* xi = x + int64_t(i) * m;
                    double* xj = x + int64_t(j) * m;
                    double a = 0.0, bb = 0.0, g = 0.0;
                    for (int t = lane; t < m; t += 32) {
                        const double p = xi[t], q = xj[t];
                        a = fma(p, p, a);
                        bb = fma(q, q, bb);
                        g = fma(p, q, g);
                    }
                    a = wsum(a);
                    bb = wsum(bb);
                    g = wsum(g);
                    if (!(fabs(g) > tol * sqrt(a) * sqrt(bb))) continue;
                    const double zeta = (bb - a) / (2.0 * g);
                    const double tt = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                    const double c = 1.0 / sqrt(1.0 + tt * tt);
                    const double s = c * tt;
                    for (int t = lane; t < m; t += 32) {
                        const double p = xi[t], q = xj[t];
                        xi[t] = c * p - s * q;
                        xj[t] = s * p + c * q;
                    }
                    double* vi = v + int64_t(i) * n;
                    double* vj = v + int64_t(j) * n;
                    for (int t = lane; t < n; t += 32) {
                        const double p = vi[t], q = vj[t];
                        vi[t] = c * p - s * q;
                        vj[t] = s * p + c * q;
                    }
                    if (lane == 0) rotated = 1;
                }
                __syncthreads();
            }
            const int done = !rotated;
            __syncthreads();
            if (done) break;
        }
    }
    // column norms
    for (int j = warp; j < n; j += nwarps) {
        const double* xj = x + int64_t(j) * m;
        double a = 0.0;
        for (int t = lane; t < m; t += 32) a = fma(xj[t], xj[t], a);
        a = wsum(a);
        if (lane == 0) raw[j] = sqrt(a);
    }
    __syncthreads();
    // sort descending by rank counting (stable on ties)
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double sj = raw[j];
        int rank = 0;
        for (int k = 0; k < n; ++k) {
            const double sk = raw[k];
            rank += (sk > sj) || (sk == sj && k < j);
        }
        S[d.s_off + rank] = sj;
        perm[d.s_off + rank] = j;
    }
    if (threadIdx.x == 0 && sweeps_out) sweeps_out[blockIdx.x] = sweep;
}

__global__ void svd_extract_kernel(const ExtractDesc* __restrict__ desc,
                                   const double* __restrict__ X, const double* __restrict__ V,
                                   const double* __restrict__ S, const int* __restrict__ perm,
                                   double* __restrict__ left, double* __restrict__ right,
                                   int ortho, double inv_norm) {
    const ExtractDesc d = desc[blockIdx.x];
    const int rows = d.rows, cols = d.cols, n = d.n, k = d.k;
    const double* x = X + d.x_off;
    const double* v = V + d.v_off;
    const double* s = S + d.s_off;
    const int* pm = perm + d.s_off;
    double* L = left + d.left_off;
    double* R = right + d.right_off;
    // left factor: rows x k
    const int64_t nl = int64_t(rows) * k;
    for (int64_t e = threadIdx.x; e < nl; e += blockDim.x) {
        const int i = int(e % rows), c = int(e / rows);
        const int pc = pm[c];
        double u;
        if (!d.trans) {
            const double xv = x[i + int64_t(pc) * rows];
            u = (ortho == 0) ? xv / s[c] : xv * inv_norm;
        } else {
            const double vv = v[i + int64_t(pc) * n];
            u = (ortho == 0) ? vv : vv * s[c] * inv_norm;
        }
        L[e] = u;
    }
    // right factor: k x cols
    const int64_t nr = int64_t(k) * cols;
    for (int64_t e = threadIdx.x; e < nr; e += blockDim.x) {
        const int c = int(e % k), j = int(e / k);
        const int pc = pm[c];
        double w;
        if (!d.trans) {
            const double vv = v[j + int64_t(pc) * n];
            w = (ortho == 0) ? vv * s[c] * inv_norm : vv;
        } else {
            const double xv = x[j + int64_t(pc) * cols];
            w = (ortho == 0) ? xv * inv_norm : xv / s[c];
        }
        R[e] = w;
    }
}

}  // namespace

void launch_svd_prepare(const SvdBlockDesc* d, int nb, const double* src, double* X, double* V,
                        cudaStream_t s) {
    if (nb <= 0) return;
    svd_prepare_kernel<<<nb, 256, 0, s>>>(d, src, X, V);
    TN_CUDA(cudaGetLastError());
}

void launch_svd_jacobi(const SvdBlockDesc* d, int nb, int max_n, double* X, double* V,
                       double* S, int* perm, int* sweeps_out, cudaStream_t s) {
    if (nb <= 0) return;
    size_t shm = size_t(max_n > 0 ? max_n : 1) * sizeof(double);
    TN_REQUIRE(shm <= 200 * 1024, "SVD block too large (more than 25600 columns)");
    if (shm > 48 * 1024)
        TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(shm)));
    svd_jacobi_kernel<<<nb, SVD_THREADS, shm, s>>>(d, X, V, S, perm, sweeps_out);
    TN_CUDA(cudaGetLastError());
}

void launch_svd_extract(const ExtractDesc* d, int nb, int, int, const double* X,
                        const double* V, const double* S, const int* perm, double* left,
                        double* right, int ortho, double inv_norm, cudaStream_t s) {
    if (nb <= 0) return;
    svd_extract_kernel<<<nb, 256, 0, s>>>(d, X, V, S, perm, left, right, ortho, inv_norm);
    TN_CUDA(cudaGetLastError());
}

}  // namespace tn
