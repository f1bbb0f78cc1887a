// Host-side objects of the sweep engine (behind the opaque handles of tennet.h).
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/tennet.h"
#include "tn_internal.h"

namespace tn {

// CUDA-event interval timer: intervals are recorded on the stream and resolved only at the
// next synchronisation point, so timing adds no host round trips.
enum TimeCat { T_HEFF = 0, T_ENV, T_SVD, T_LANCZOS, T_SWEEP, T_GEMM, T_PACK, T_QRPANEL, T_QRGEMM,
               T_NCAT };
struct EventTimer {
    cudaStream_t s = nullptr;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    struct Iv { int cat; int a, b; };
    std::vector<Iv> ivs;
    int mark();
    void add(int cat, int a, int b) { ivs.push_back(Iv{cat, a, b}); }
    // sums the recorded intervals (ms) per category into acc and forgets them; the caller
    // must have synchronised the stream.
    void collect(double* acc);
    ~EventTimer();
};

struct Scratch;  // fixed-capacity device scratch used by the allocation-free entry points

// work buffers of the multi-SM block SVD (bsvd.cpp), kept by the context between bonds
struct BsvdWork {
    DevBuf arena, blks, flags, bars, sweeps;
    DevBuf bjd[2];
};
struct BsvdStats {
    double gemm_flops = 0;    // algorithmic flops of the SVD's grouped GEMMs
    double jacobi_flops = 0;  // flops of the Jacobi rotations (dots and column updates)
    int sweeps32 = 0, sweeps_df = 0;
    double small_flops = 0;   // algorithmic flops of the one-CTA block SVDs
};

// Autotuned schedule of a bond's block SVD: which charge blocks take the one-CTA kernel and
// which the multi-SM pipeline.  Keyed on the bond's block-size histogram through its largest
// block that the pipeline accepts (32-column buckets); the candidate thresholds of a key are
// timed once each (CUDA events around the whole SVD) on the first bonds with that key, then
// the fastest is used for every later bond with it.
struct SvdTuner {
    struct Entry {
        std::vector<int> cand;  // column thresholds (INT_MAX: every block on one CTA)
        std::vector<float> ms;  // measured milliseconds, -1 until tried
        int next = 0, best = -1;
    };
    std::map<int, Entry> table;
    cudaEvent_t a = nullptr, b = nullptr;
    SvdTuner() = default;
    SvdTuner(const SvdTuner&) = delete;
    SvdTuner& operator=(const SvdTuner&) = delete;
    ~SvdTuner();
};

// overlap environment of psi against a projector state on one link: one D_psi(q) x D_M(q)
// block (column-major) per charge q that both links carry
struct OvEnv {
    std::vector<int> q, da, db;
    std::vector<int64_t> off;
    int64_t size = 0;
    DevBuf buf;
    int find(int charge) const;
};

}  // namespace tn

struct tn_ctx;
namespace tn {
// helpers of engine.cpp shared with the tree tensor network sweep
void sym_eig_host(int n, const std::vector<double>& A, std::vector<double>& D,
                  std::vector<double>& U);  // ascending; A, U row-major
std::unique_ptr<SplitPlan> make_split_plan(const GemmPlan& g, int slices, cudaStream_t st,
                                           bool own_packs);
void run_split_plan(tn_ctx* ctx, SplitPlan& sp, const Bases& bs);
void check_device_error_public(tn_ctx* ctx);
int svd_truncate_dense(tn_ctx* ctx, const double* A, int m, int n, int maxdim, int mindim,
                       double cutoff, double* U, double* SVt, double* truncerr);
// SVD of large charge blocks on the whole GPU (bsvd.cpp): outputs as svd_qrj_kernel's
void big_block_svd(tn_ctx* ctx, BsvdWork& W, const std::vector<SvdBlockDesc>& blocks,
                   const double* src, double* QV, double* PY, double* S, int* perm,
                   BsvdStats* stats);
}  // namespace tn

struct tn_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    int prec = TN_PREC_FP64;
    int slices = 5;
    tn::EventTimer timer;
    tn::DevBuf err;  // device error word of bounded waits (0 = ok)
    int svd_big_n = -1;  // charge blocks with more columns take the multi-SM SVD (-1: tuned)
    tn::SvdTuner svd_tune;
    tn::BsvdWork bsvd;
    tn::DevBuf svd_counts;  // sweep counts (and debug clocks) of the one-CTA block SVDs
    tn::BsvdStats svd_stats;  // accumulated by the block SVDs (read and reset by the sweeps)
};

struct tn_mpo {
    tn_ctx* ctx = nullptr;
    int N = 0, d = 0;
    std::vector<int> pq;
    std::vector<int> wd;                   // N+1
    std::vector<std::vector<int>> delta;   // N+1
    std::vector<std::vector<double>> W;    // per site, column-major (wl, wr, d, d)
    double at(int i, int a, int b, int sp, int s) const {
        const int wl = wd[i], wr = wd[i + 1];
        return W[i][size_t(a) + size_t(wl) * (size_t(b) + size_t(wr) * (size_t(sp) + size_t(d) * s))];
    }
};

struct tn_site {
    tn::SiteLayout lay;
    tn::DevBuf buf;
};

// A complex MPS (cplx) keeps each site's blocks as two planes in one buffer: the real parts
// (lay.size values), then the imaginary parts.
struct tn_mps {
    tn_ctx* ctx = nullptr;
    int N = 0, d = 0;
    std::vector<int> pq;
    std::vector<tn::Link> links;   // N+1
    std::vector<tn_site> sites;    // N
    int center = 0;
    bool cplx = false;
    int planes() const { return cplx ? 2 : 1; }
};

struct tn_envt {
    tn::EnvLayout lay;
    tn::DevBuf buf;
};

// contraction plans of the two-site effective Hamiltonian at one position
struct Heff2Plan {
    tn::PhiLayout ph;
    tn::GemmPlan g1, g3;
    tn::GemmPlan g1c, g3c;  // complex forms (complex states)
    tn::CombPlan cbc;
    std::unique_ptr<tn::SplitPlan> s1, s3;  // split-precision plans (built on first use)
    std::unique_ptr<tn::SplitPlan> s1c, s3c;  // the same of the complex forms (unsigned)
    tn::CombPlan cb;
    int64_t ysize = 0, zsize = 0;
    double flops = 0;
    // offset in T1 of Y(a, il, s1) = L(a, il) * phi[slab (s1, l)], [(a * nsec + il) * d + s1],
    // -1 where not formed (the noise term of the left move reads these blocks)
    std::vector<int64_t> yoff;
};

// contraction plans of the one-site effective Hamiltonian at one position; the one-site
// tensor is taken in the right-grouped layout
struct Heff1Plan {
    tn::SiteLayout lay;
    tn::GemmPlan g1, g3;
    tn::CombPlan cb;
    tn::GemmPlan g1c, g3c;  // complex forms (complex states)
    tn::CombPlan cbc;
    std::unique_ptr<tn::SplitPlan> s1, s3;
    std::unique_ptr<tn::SplitPlan> s1c, s3c;  // the same of the complex forms (unsigned)
    int64_t ysize = 0, zsize = 0;
    double flops = 0;
};

// one excited-state projector (ProjMPS2): a copy of M and its overlap environments with psi,
// L[i] over sites < i (link i), R[i] over sites > i (link i + 1)
struct ProjState {
    std::unique_ptr<tn_mps> M;
    std::vector<tn::OvEnv> L, R;
};

struct tn_env;
namespace tn {
// excited-state projectors (proj.cpp)
void proj_init(tn_env* env);             // edge blocks and the environments up to lpos / rpos
void proj_left_step(tn_env* env, int i);   // LM[i+1] of every projector
void proj_right_step(tn_env* env, int i);  // RM[i-1]
void proj_vectors2(tn_env* env, int p, const PhiLayout& ph);    // m_k at bond p -> projm
void proj_vectors1(tn_env* env, int p, const SiteLayout& lay);  // m_k at site p (RG) -> projm
void proj_apply(tn_env* env, const double* x, double* y, int64_t n);  // y += w sum m (m . x)
}  // namespace tn

struct tn_env {
    tn_ctx* ctx = nullptr;
    std::unique_ptr<tn_mps> psi;
    const tn_mpo* H = nullptr;
    // planar complex when psi is complex: real, imaginary and negated imaginary planes (the
    // third lets every segment of the complex H_eff be a positive product)
    std::vector<tn_envt> L, R;
    int lpos = 0, rpos = 0;
    int pos = 0, nsite = 2;
    // work buffers
    tn::DevBuf t1, t2, kry, part, dots, ticket, svdX, svdW, svdV, svdP, svdS, svdPerm, desc, desc2,
        vecA, vecB, cx;  // cx: realified complex blocks
    std::unique_ptr<Heff2Plan> hp;
    int hp_pos = -1;
    std::unique_ptr<Heff1Plan> h1p;
    int h1p_pos = -1;
    tn::DevBuf vecC, vecD;
    double acc_ms[tn::T_NCAT] = {};
    double gemm_flops = 0;
    int64_t gemm_launches = 0;
    int64_t matvecs = 0;
    double heff_flops = 0;
    // excited-state projectors (ProjMPO_MPS2): states, weight, the projected vectors of the
    // current position (K x n) and work buffers
    std::vector<ProjState> proj;
    double proj_weight = 0.0;
    tn::DevBuf projm, projc, projt1, projt2;
    // kept spectrum (squared singular values, descending) of every bond from the last full
    // sweep, bond b between sites b and b + 1 (SweepData.lasteigs)
    std::vector<std::vector<double>> bond_eigs;
};
