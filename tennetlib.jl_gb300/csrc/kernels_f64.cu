// FP64 kernels of the sweep engine:
//  * grouped block-sparse GEMM (CUDA-core DFMA) -- the FP64 GPU path of every contraction
//    of the two-site effective Hamiltonian and of the environment updates;
//  * block linear combination -- the MPO step between the two GEMM stages;
//  * Krylov vector kernels (multi-dot, multi-axpy, scaling, linear combination) with
//    warp-shuffle reductions and a deterministic two-stage finalisation.
#include <cuda_runtime.h>

#include "tn_internal.h"

namespace tn {

// ------------------------------------------------------------------------------------
// grouped GEMM: one CTA per 64x64 output tile, 256 threads, 4x4 outputs per thread
// ------------------------------------------------------------------------------------
namespace {
constexpr int BK = 16;

__global__ void __launch_bounds__(256)
gemm_f64_kernel(const Seg* __restrict__ segs, const Task* __restrict__ tasks,
                const Tile* __restrict__ tiles, Bases b) {
    __shared__ double As[BK][GEMM_BM + 1];
    __shared__ double Bs[BK][GEMM_BN + 1];
    const Tile t = tiles[blockIdx.x];
    const Task tk = tasks[t.task];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int si = 0; si < tk.nseg; ++si) {
        const Seg sg = segs[tk.seg0 + si];
        const double* __restrict__ A = b.p[sg.abuf] + sg.aoff;
        const double* __restrict__ B = b.p[sg.bbuf] + sg.boff;
        for (int k0 = 0; k0 < sg.k; k0 += BK) {
            for (int e = tid; e < GEMM_BM * BK; e += 256) {
                int i, kk;
                if (!sg.ta) { i = e % GEMM_BM; kk = e / GEMM_BM; }
                else        { kk = e % BK; i = e / BK; }
                const int gi = t.m0 + i, gk = k0 + kk;
                double v = 0.0;
                if (gi < tk.m && gk < sg.k)
                    v = sg.ta ? A[gk + int64_t(gi) * sg.lda] : A[gi + int64_t(gk) * sg.lda];
                As[kk][i] = sg.sgn < 0 ? -v : v;
            }
            for (int e = tid; e < GEMM_BN * BK; e += 256) {
                int j, kk;
                if (!sg.tb) { kk = e % BK; j = e / BK; }
                else        { j = e % GEMM_BN; kk = e / GEMM_BN; }
                const int gj = t.n0 + j, gk = k0 + kk;
                double v = 0.0;
                if (gj < tk.n && gk < sg.k)
                    v = sg.tb ? B[gj + int64_t(gk) * sg.ldb] : B[gk + int64_t(gj) * sg.ldb];
                Bs[kk][j] = v;
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                double a[4], bb[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) bb[j] = Bs[kk][ty + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
            }
            __syncthreads();
        }
    }
    double* __restrict__ C = b.p[tk.cbuf] + tk.coff;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int gj = t.n0 + ty + 16 * j;
        if (gj >= tk.n) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int gi = t.m0 + tx + 16 * i;
            if (gi < tk.m) {
                double* c = C + gi + int64_t(gj) * tk.ldc;
                *c = tk.accum ? *c + acc[i][j] : acc[i][j];
            }
        }
    }
}

__global__ void __launch_bounds__(256)
combine_kernel(const CombOut* __restrict__ outs, const CombTerm* __restrict__ terms,
               const CombTile* __restrict__ tiles, Bases b) {
    const CombTile t = tiles[blockIdx.x];
    const CombOut o = outs[t.out];
    const int r = t.r0 + (threadIdx.x & 31);
    const int cb = t.c0 + (threadIdx.x >> 5);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const bool rok = r < o.rows;
    for (int ti = 0; ti < o.nt; ++ti) {
        const CombTerm tm = terms[o.t0 + ti];
        const double* __restrict__ src = b.p[tm.sbuf] + tm.soff;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = cb + 8 * j;
            if (rok && c < o.cols) acc[j] = fma(tm.coef, src[r + int64_t(c) * tm.lds], acc[j]);
        }
    }
    double* __restrict__ dst = b.p[o.dbuf] + o.doff;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = cb + 8 * j;
        if (rok && c < o.cols) dst[r + int64_t(c) * o.ldd] = acc[j];
    }
}

// ------------------------------------------------------------------------------------
// Krylov vector kernels
// ------------------------------------------------------------------------------------
constexpr int KMAX = 32;
struct VecPtrs {
    const double* p[KMAX];
};
constexpr int BLAS_THREADS = 256;
constexpr int BLAS_PARTS = 2 * 152;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int K>
__global__ void __launch_bounds__(BLAS_THREADS)
multi_dot_kernel(VecPtrs V, int kk, const double* __restrict__ w, int64_t n,
                 double* __restrict__ part) {
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double x = w[i];
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < kk) acc[k] = fma(V.p[k][i], x, acc[k]);
    }
    __shared__ double red[BLAS_THREADS / 32][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double v = warp_sum(acc[k]);
        if (lane == 0) red[wid][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kk) {
        double s = 0.0;
        for (int j = 0; j < BLAS_THREADS / 32; ++j) s += red[j][threadIdx.x];
        part[int64_t(threadIdx.x) * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void finalize_dot_kernel(const double* __restrict__ part, int nparts, int kk,
                                    double* __restrict__ out) {
    // one warp per result, fixed summation order
    const int k = blockIdx.x;
    if (k >= kk) return;
    double s = 0.0;
    for (int j = threadIdx.x; j < nparts; j += 32) s += part[int64_t(k) * nparts + j];
    s = warp_sum(s);
    if (threadIdx.x == 0) out[k] = s;
}

__global__ void __launch_bounds__(BLAS_THREADS)
multi_axpy_kernel(double* __restrict__ w, VecPtrs V, int kk, const double* __restrict__ h,
                  double sign, int64_t n) {
    __shared__ double hs[KMAX];
    if (threadIdx.x < kk) hs[threadIdx.x] = sign * h[threadIdx.x];
    __syncthreads();
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        double x = w[i];
        for (int k = 0; k < kk; ++k) x = fma(hs[k], V.p[k][i], x);
        w[i] = x;
    }
}

__global__ void __launch_bounds__(BLAS_THREADS)
scale_into_kernel(double* __restrict__ dst, const double* __restrict__ src,
                  const double* __restrict__ denom_sq, double hscale, int64_t n) {
    double s = hscale;
    if (denom_sq) s = hscale / sqrt(*denom_sq);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = src[i] * s;
}

__global__ void __launch_bounds__(BLAS_THREADS)
lincomb_kernel(double* __restrict__ dst, VecPtrs V, int kk, const double* __restrict__ coef,
               int64_t n) {
    __shared__ double cs[KMAX];
    if (threadIdx.x < kk) cs[threadIdx.x] = coef[threadIdx.x];
    __syncthreads();
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        double x = 0.0;
        for (int k = 0; k < kk; ++k) x = fma(cs[k], V.p[k][i], x);
        dst[i] = x;
    }
}

// One fused Gram-Schmidt pass over a Krylov residual w:
//   (optional)  w += sign * sum_k hin[k] V_k
//   (optional)  out[k] = V_k . w   for k < kk          (with the updated w)
//   (optional)  out[kk or 0] = w . w
// Partial sums of every block go to `part`; the last block to finish (atomic ticket)
// adds them in block order, so results are deterministic, and resets the ticket.
template <int K>
__global__ void __launch_bounds__(BLAS_THREADS)
gs_pass_kernel(VecPtrs V, int kk, double* __restrict__ w, const double* __restrict__ hin,
               double sign, int64_t n, int dots, int norm, double* __restrict__ part,
               double* __restrict__ out, unsigned* __restrict__ ticket) {
    __shared__ double hs[KMAX];
    __shared__ double red[BLAS_THREADS / 32][K + 1];
    __shared__ int last;
    if (hin && threadIdx.x < kk) hs[threadIdx.x] = sign * hin[threadIdx.x];
    __syncthreads();
    double acc[K + 1];
#pragma unroll
    for (int k = 0; k <= K; ++k) acc[k] = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        double x = w[i];
        if (hin) {
            for (int k = 0; k < kk; ++k) x = fma(hs[k], V.p[k][i], x);
            w[i] = x;
        }
        if (dots) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (k < kk) acc[k] = fma(V.p[k][i], x, acc[k]);
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
    if (threadIdx.x < nres) {
        const int src = (dots && threadIdx.x < kk) ? threadIdx.x : K;
        double sum = 0.0;
        for (int j = 0; j < BLAS_THREADS / 32; ++j) sum += red[j][src];
        part[int64_t(threadIdx.x) * gridDim.x + blockIdx.x] = sum;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int j = wid; j < nres; j += BLAS_THREADS / 32) {
        double sum = 0.0;
        for (int bb = lane; bb < (int)gridDim.x; bb += 32)
            sum += reinterpret_cast<volatile double*>(part)[int64_t(j) * gridDim.x + bb];
        sum = warp_sum(sum);
        if (lane == 0) out[j] = sum;
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

__global__ void __launch_bounds__(BLAS_THREADS)
block_dot_kernel(const BlockDot* __restrict__ descs, double* __restrict__ out) {
    __shared__ double red[BLAS_THREADS / 32];
    const BlockDot D = descs[blockIdx.x];
    const int64_t n = int64_t(D.rows) * D.cols;
    double acc = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int r = int(e % D.rows), c = int(e / D.rows);
        acc = fma(D.x[r + int64_t(c) * D.ldx], D.y[r + int64_t(c) * D.ldy], acc);
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < BLAS_THREADS / 32; ++w) s += red[w];
        out[blockIdx.x] = s;
    }
}

int grid_for(int64_t n) {
    int64_t g = (n + BLAS_THREADS - 1) / BLAS_THREADS;
    if (g > BLAS_PARTS) g = BLAS_PARTS;
    if (g < 1) g = 1;
    return int(g);
}

VecPtrs make_ptrs(const double* const* V, int K) {
    VecPtrs p{};
    TN_REQUIRE(K <= KMAX, "too many Krylov vectors for one kernel (max 32)");
    for (int k = 0; k < K; ++k) p.p[k] = V[k];
    return p;
}
}  // namespace

void launch_gemm_f64(const GemmPlan& p, const Bases& b, cudaStream_t s) {
    if (p.tiles.empty()) return;
    gemm_f64_kernel<<<unsigned(p.tiles.size()), 256, 0, s>>>(
        p.dsegs.as<Seg>(), p.dtasks.as<Task>(), p.dtiles.as<Tile>(), b);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_combine(const CombPlan& p, const Bases& b, cudaStream_t s) {
    if (p.tiles.empty()) return;
    combine_kernel<<<unsigned(p.tiles.size()), 256, 0, s>>>(
        p.douts.as<CombOut>(), p.dterms.as<CombTerm>(), p.dtiles.as<CombTile>(), b);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

int blas_nparts() { return BLAS_PARTS; }

void launch_block_dots(const BlockDot* d, int n, double* out, cudaStream_t s) {
    if (n <= 0) return;
    block_dot_kernel<<<n, BLAS_THREADS, 0, s>>>(d, out);
    TN_CUDA(cudaGetLastError());
    count_launch();
}

void launch_multi_dot(const double* const* V, int K, const double* w, int64_t n,
                      double* part, double* out, cudaStream_t s) {
    if (K <= 0) return;
    VecPtrs P = make_ptrs(V, K);
    const int g = BLAS_PARTS;  // fixed part count: deterministic, finalize reads g parts
    if (K <= 4)
        multi_dot_kernel<4><<<g, BLAS_THREADS, 0, s>>>(P, K, w, n, part);
    else if (K <= 8)
        multi_dot_kernel<8><<<g, BLAS_THREADS, 0, s>>>(P, K, w, n, part);
    else if (K <= 16)
        multi_dot_kernel<16><<<g, BLAS_THREADS, 0, s>>>(P, K, w, n, part);
    else
        multi_dot_kernel<32><<<g, BLAS_THREADS, 0, s>>>(P, K, w, n, part);
    TN_CUDA(cudaGetLastError());
    count_launch();
    finalize_dot_kernel<<<K, 32, 0, s>>>(part, g, K, out);
    TN_CUDA(cudaGetLastError());
    count_launch();
    count_krylov_bytes(int64_t(K + 1) * n * 8);
}

void launch_multi_axpy(double* w, const double* const* V, int K, const double* h, double sign,
                       int64_t n, cudaStream_t s) {
    if (K <= 0 || n <= 0) return;
    multi_axpy_kernel<<<grid_for(n), BLAS_THREADS, 0, s>>>(w, make_ptrs(V, K), K, h, sign, n);
    TN_CUDA(cudaGetLastError());
    count_launch();
    count_krylov_bytes(int64_t(K + 2) * n * 8);
}

void launch_gs_pass(const double* const* V, int K, double* w, const double* hin, double sign,
                    int64_t n, bool dots, bool norm, double* part, double* out, unsigned* ticket,
                    cudaStream_t s) {
    VecPtrs P = K > 0 ? make_ptrs(V, K) : VecPtrs{};
    const int g = BLAS_PARTS;
    const int d = dots ? 1 : 0, nm = norm ? 1 : 0;
    if (K <= 4)
        gs_pass_kernel<4><<<g, BLAS_THREADS, 0, s>>>(P, K, w, hin, sign, n, d, nm, part, out, ticket);
    else if (K <= 8)
        gs_pass_kernel<8><<<g, BLAS_THREADS, 0, s>>>(P, K, w, hin, sign, n, d, nm, part, out, ticket);
    else if (K <= 16)
        gs_pass_kernel<16><<<g, BLAS_THREADS, 0, s>>>(P, K, w, hin, sign, n, d, nm, part, out, ticket);
    else
        gs_pass_kernel<32><<<g, BLAS_THREADS, 0, s>>>(P, K, w, hin, sign, n, d, nm, part, out, ticket);
    TN_CUDA(cudaGetLastError());
    count_launch();
    count_krylov_bytes(int64_t(1 + ((hin || dots) ? K : 0) + (hin ? 1 : 0)) * n * 8);
}

void launch_scale_into(double* dst, const double* src, const double* denom_sq,
                       double host_scale, int64_t n, cudaStream_t s) {
    if (n <= 0) return;
    scale_into_kernel<<<grid_for(n), BLAS_THREADS, 0, s>>>(dst, src, denom_sq, host_scale, n);
    TN_CUDA(cudaGetLastError());
    count_launch();
    count_krylov_bytes(2 * n * 8);
}

void launch_lincomb(double* dst, const double* const* V, int K, const double* coef, int64_t n,
                    cudaStream_t s) {
    if (n <= 0) return;
    lincomb_kernel<<<grid_for(n), BLAS_THREADS, 0, s>>>(dst, make_ptrs(V, K), K, coef, n);
    TN_CUDA(cudaGetLastError());
    count_launch();
    count_krylov_bytes(int64_t(K + 1) * n * 8);
}

}  // namespace tn
