// Internal declarations of the tree tensor network (TTN) sweep: the tree, the batched
// kernel descriptors and their launchers.
#pragma once

#include <cstdint>
#include <map>
#include <utility>
#include <vector>

#include "tn_internal.h"

namespace tn {

constexpr int BK_MAX = 32;      // Krylov vectors per batched kernel
constexpr int TTN_PARTS = 152;  // partial sums per instance of the batched reductions
constexpr int HH_B = 32;        // panel width of the blocked Householder QR

// A tree of nodes 0..nn-1 with physical sites attached.  The legs of node v are its sites
// (ascending), then its neighbours (ascending).
struct TtnTree {
    int N = 0, d = 0, nn = 0;
    std::vector<std::vector<int>> nbr, sites;
    std::vector<int> site_node;
    std::vector<std::pair<int, int>> edges;  // (a, b), a < b
    std::map<std::pair<int, int>, int> eidx;
    int nlegs(int v) const { return int(sites[v].size() + nbr[v].size()); }
    int leg_nbr(int v, int u) const;
    int leg_site(int v, int n) const;
    int edge(int a, int b) const;
    std::vector<int> path(int a, int b) const;   // shortest path a .. b
    std::vector<char> side(int v, int u) const;  // sites on v's side of the edge (v, u)
};

// ---- batched Krylov descriptors -----------------------------------------------------
struct BGsDesc {                 // one instance of a fused Gram-Schmidt pass
    const double* V[BK_MAX];
    double* w;
    const double* hin;           // w += sign * V hin first (device, or null)
    double* out;                 // dots V^T w (kk values), then |w|^2
    int64_t n;
    int32_t kk, pad;
};
struct BScaleDesc {              // dst (and dst2) = src * scale [/ sqrt(*denom_sq)]
    const double* src;
    double* dst;
    double* dst2;
    const double* denom_sq;
    double scale;
    int64_t n;
};
struct BLinDesc {                // dst = sum_k coef[k] V[k]
    const double* V[BK_MAX];
    const double* coef;
    double* dst;
    int64_t n;
    int32_t kk, pad;
};
struct PermDesc {                // (P, D, Q) <-> (P, Q, D)
    const double* src;
    double* dst;
    int64_t P, D, Q;
    int32_t to_end, pad;
};
struct ConcatDesc {              // dst (P, D1 + D2, Q) = [a (P, D1, Q) | b (P, D2, Q)]
    const double* a;
    const double* b;
    double* dst;
    int64_t P, D1, D2, Q;
};
struct QrDesc {                  // small QR: A (m x n, ld m) -> Q in place, R out
    double* A;
    double* R;
    double* tau;
    int32_t m, n;
};
struct HhDesc {                  // blocked Householder QR of A (m x n, ld m, m >= n)
    double* A;                   // factored in place; then overwritten by Q (= Q below)
    double* Q;
    double* R;                   // kmin x n
    double* V;                   // explicit reflectors, m x kmin, ld m (see hh_panel_voff)
    double* T;                   // per panel -T (HH_B x HH_B)
    double* G;                   // V^T V of all reflectors (kmin x kmin, ld kmin)
    double* Tall;                // -T of the whole block reflector (kmin x kmin, ld kmin)
    double* Yscr;                // scratch of the -T kernel (>= kmin * HH_B)
    double* tau;                 // kmin
    double* scal;                // tau, scale, beta of column j at scal + 4 (j & 1)
    double* wv;                  // current column: tau * w_k of the panel columns
    double* part;                // partial sums (>= HH_B*HH_B*TTN_PARTS)
    unsigned* ticket;
    unsigned* bar;               // barrier counter of the cooperative panel kernel
    int32_t m, n, kmin;
    int32_t cta0, ncta;          // CTAs [cta0, cta0 + ncta) of the cooperative panel kernel
    int32_t pad;
};

// The reflectors form one unit lower-trapezoidal matrix V (m x kmin, ld m; zero above the
// diagonal, one on it).  Offset of the panel starting at column p0, from its diagonal row:
// that panel's reflectors are the (m - p0) x HH_B block below, with ld m.
__host__ __device__ inline int64_t hh_panel_voff(int m, int p0) {
    return int64_t(p0) + int64_t(p0) * m;
}

int ttn_parts();
void launch_bgs_pass(const BGsDesc* d, int ninst, int kmax, int64_t nmax, double sign, bool dots,
                     bool norm, double* part, unsigned* tickets, cudaStream_t s);
void launch_bscale(const BScaleDesc* d, int ninst, int64_t nmax, cudaStream_t s);
void launch_blincomb(const BLinDesc* d, int ninst, int64_t nmax, cudaStream_t s);
void launch_permute(const PermDesc* d, int ninst, int64_t nmax, cudaStream_t s);
// the direct sum of subspace expansion along one leg; nmax >= every P (D1 + D2) Q
void launch_concat(const ConcatDesc* d, int ninst, int64_t nmax, cudaStream_t s);
void launch_qr_small(const QrDesc* d, int ninst, cudaStream_t s);
void launch_hh_column(const HhDesc* d, int ninst, int64_t mmax, int j, int p0, int pend,
                      cudaStream_t s);
void launch_hh_panel_end(const HhDesc* d, int ninst, int64_t mmax, int p0, int pb,
                         cudaStream_t s);
void launch_hh_finish(const HhDesc* d, int ninst, int64_t mnmax, cudaStream_t s);
// -T of the whole block reflector from G = V^T V and the per-panel T (one CTA per instance)
void launch_hh_tall(const HhDesc* d, int ninst, cudaStream_t s);
// CTAs that the cooperative panel kernel may use (all co-resident on the device)
int hh_coop_capacity();
// one panel [p0, p0 + HH_B) of every instance in one cooperative launch of nctas CTAs
// (instance i owns CTAs [cta0, cta0 + ncta)); grid-wide waits are bounded and set *err
void launch_hh_panel_coop(const HhDesc* d, int ninst, int nctas, int p0, int* err,
                          cudaStream_t s);

}  // namespace tn
