// Host driver of the multi-SM SVD of large charge blocks (kernels in kernels_bsvd.cu).
//
// For the blocks of one bond it lays out a work arena, orders each block's columns by
// decreasing norm (a static column pivoting), runs the blocked Householder QR (panel kernel
// + three grouped GEMMs per panel of up to 32 columns), the cooperative FP32 Jacobi presolve
// on R^T, two Newton-Schulz steps V <- V (3 I - V^T V) / 2 and Y = R^T V by grouped
// GEMMs, the cooperative double-float polish, and Q [V; 0] by grouped GEMMs.  The GEMMs run in
// the context's precision: FP64 on CUDA cores, or bf16 slices on the tensor cores with seven
// slices per operand (56 bits, FP64-equivalent products); the two w x w T products always run
// in FP64.  Results land where the one-CTA kernel puts them: QV (m x n) at x_off of the QV
// buffer, PY (n x n, rows in the source column order) at v_off, singular values and
// permutation at s_off.
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "engine.h"

namespace tn {
namespace {

constexpr int SVD_SLICES = 7;  // bf16 slices per operand of the SVD GEMMs on the split path

int64_t align32(int64_t x) { return (x + 31) & ~int64_t(31); }

constexpr int KC = 256;  // rows per k chunk of the W1 = V^T C products (split k)

struct Mm {  // one GEMM task of a grouped plan: C (+)= op(A) op(B), offsets in doubles
    int cbuf;
    int64_t coff;
    int m, n, ldc, accum;
    int abuf;
    int64_t aoff;
    int lda, ta;
    int bbuf;
    int64_t boff;
    int ldb, tb, k;
    int cont = 0;  // 1: one more segment of the previous task (its C fields are ignored)
};

struct GemmRun {
    tn_ctx* ctx;
    Bases bs;
    bool split;
    double flops = 0;
    void run(const std::vector<Mm>& mm, bool force_fp64 = false) {
        if (mm.empty()) return;
        GemmPlan g;
        for (const Mm& t : mm) {
            if (!t.cont) g.add_task(t.cbuf, t.coff, t.m, t.n, t.ldc, t.accum);
            g.add_seg(t.abuf, t.aoff, t.lda, t.ta, t.bbuf, t.boff, t.ldb, t.tb, t.k);
        }
        flops += g.flops;
        cudaStream_t st = ctx->stream;
        if (!split || force_fp64) {
            g.finalize(st);
            launch_gemm_f64(g, bs, st);
            return;
        }
        auto sp = make_split_plan(g, SVD_SLICES, st, true);
        launch_split_pack(sp->dajobs.as<PackJob>(), (int)sp->ajobs.size(), sp->daks.as<KTileSrc>(),
                          bs, sp->ap, sp->eap, sp->slices, split_tile_rows_a(), st, sp->a_maxnkt,
                          sp->amax.as<unsigned long long>(), sp->ea_n);
        launch_split_pack(sp->dbjobs.as<PackJob>(), (int)sp->bjobs.size(), sp->dbks.as<KTileSrc>(),
                          bs, sp->bp, sp->ebp, sp->slices, split_tile_rows_b(), st, sp->b_maxnkt,
                          sp->bmax.as<unsigned long long>(), sp->eb_n);
        launch_split_gemm(sp->ditems.as<SplitItem>(), (int)sp->items.size(),
                          sp->dtasks.as<SplitTask>(), sp->ap, sp->bp, sp->eap, sp->ebp, bs,
                          sp->slices, ctx->err.as<int>(), ctx->nsm, st);
    }
};

// CTAs of each matrix's Jacobi group: in proportion to n^3, at most one per block pair
void assign_ctas(std::vector<BjDesc>& bj, int cap) {
    double tot = 0;
    for (auto& d : bj) tot += double(d.n) * d.n * d.n;
    int used = 0;
    const int nd = int(bj.size());
    for (auto& d : bj) {
        const int nbe = d.nb + (d.nb & 1);
        int c = int(double(std::max(cap - nd, 0)) * double(d.n) * d.n * d.n / std::max(tot, 1.0));
        c = std::max(1, std::min(c, nbe / 2));
        d.cta0 = used;
        d.ncta = c;
        used += c;
    }
    TN_REQUIRE(used <= cap, "block SVD: more Jacobi groups than co-resident CTAs");
}

}  // namespace

void big_block_svd(tn_ctx* ctx, BsvdWork& W, const std::vector<SvdBlockDesc>& blocks,
                   const double* src, double* QV, double* PY, double* S, int* perm,
                   BsvdStats* stats) {
    if (blocks.empty()) return;
    cudaStream_t st = ctx->stream;
    const int nb = int(blocks.size());
    int mmax = 1, nmax = 1;
    for (const auto& b : blocks) {
        mmax = std::max(mmax, b.m);
        nmax = std::max(nmax, b.n);
    }
    // panel schedule shared by all blocks: at column p0 the widest panel (32, 16, 8 or 4
    // columns) whose rows (those of the tallest block below p0) fit the panel kernel's
    // shared memory; panels widen as the QR proceeds down the tall blocks
    std::vector<std::pair<int, int>> panels;
    for (int p0 = 0; p0 < nmax;) {
        const int w = bsvd_panel_width(mmax - p0);
        TN_REQUIRE(w > 0, "block SVD: block too tall for the panel kernel");
        panels.emplace_back(p0, w);
        p0 += w;
    }
    TN_REQUIRE(nmax <= bsvd_max_n(), "block SVD: block too wide for the Jacobi kernel");
    // arena layout
    std::vector<BsvdBlk> bd(nb);
    std::vector<int64_t> w1(nb), w2(nb);
    int64_t off = 0;
    auto take = [&](int64_t n) {
        const int64_t o = off;
        off += align32(n);
        return o;
    };
    int64_t mnmax = 1, nnmax = 1;
    for (int j = 0; j < nb; ++j) {
        const SvdBlockDesc& s = blocks[j];
        BsvdBlk& d = bd[j];
        d = BsvdBlk{};
        d.src_off = s.src_off;
        d.rows = s.rows;
        d.cols = s.cols;
        d.trans = s.trans;
        d.m = s.m;
        d.n = s.n;
        d.x_off = s.x_off;
        d.v_off = s.v_off;
        d.s_off = s.s_off;
        const int64_t m = s.m, n = s.n;
        d.xq = take(m * n);
        d.vp = take(m * n);    // reflectors of the panel at column p0: at p0 m, (m - p0) x w
        d.tm = take(64 * n);   // its -T^T and -T (2 w^2 <= 64 w): at 64 p0
        d.rt64 = take(n * n);
        d.v64 = take(n * n);
        d.g64 = take(n * n);
        d.v64b = take(n * n);
        d.y64 = take(n * n);
        d.r32 = take((n * n + 1) / 2);
        d.v32 = take((n * n + 1) / 2);
        d.ydf = take(n * n);
        d.vdf = take(n * n);
        d.scl = take(1);
        d.cn = take(n);
        d.piv = take(n);
        w1[j] = take(32 * std::max(n, int64_t(1)) * ((m + KC - 1) / KC));  // one per k chunk
        w2[j] = take(32 * std::max(n, int64_t(1)));
        mnmax = std::max(mnmax, m * n);
        nnmax = std::max(nnmax, n * n);
    }
    W.arena.alloc(size_t(std::max<int64_t>(off, 32)) * 8, st);
    W.blks.alloc(bd.size() * sizeof(BsvdBlk), st);
    TN_CUDA(cudaMemcpyAsync(W.blks.p, bd.data(), bd.size() * sizeof(BsvdBlk),
                            cudaMemcpyHostToDevice, st));
    double* ar = W.arena.d();
    const BsvdBlk* dblk = W.blks.as<BsvdBlk>();
    GemmRun G{ctx, Bases{}, ctx->prec == TN_PREC_SPLIT};
    G.bs.p[0] = ar;
    G.bs.p[1] = QV;
    const int AR = 0, QB = 1;

    // ---- blocked Householder QR -------------------------------------------------------
    launch_bsvd_gather(dblk, nb, mnmax, src, ar, st);
    for (const auto& pp : panels) {
        const int p0 = pp.first, pw = pp.second;
        launch_bsvd_panel(dblk, nb, p0, pw, mmax - p0, ar, st);
        std::vector<Mm> g1, g2, g3;
        for (int j = 0; j < nb; ++j) {
            const BsvdBlk& d = bd[j];
            if (p0 >= d.n) continue;
            const int w = std::min(pw, d.n - p0), r = d.m - p0, nt = d.n - p0 - w;
            if (nt <= 0) continue;
            const int64_t vpo = d.vp + int64_t(p0) * d.m;
            const int64_t co = d.xq + p0 + int64_t(p0 + w) * d.m;
            const int64_t tmo = d.tm + int64_t(p0) * 64;
            // W1_c = V_c^T C_c over row chunks c of KC rows (split k: the output has only w
            // rows, so one long-k product would occupy few CTAs), W2 = (-T^T) sum_c W1_c
            // (one task, a segment per chunk), C += V W2
            const int nch = (r + KC - 1) / KC;
            for (int c = 0; c < nch; ++c) {
                const int r0 = c * KC, rc = std::min(KC, r - r0);
                const int64_t wc = w1[j] + int64_t(c) * w * nt;
                g1.push_back(Mm{AR, wc, w, nt, w, 0, AR, vpo + r0, r, 1, AR, co + r0, d.m, 0, rc});
                Mm t2{AR, w2[j], w, nt, w, 0, AR, tmo, w, 0, AR, wc, w, 0, w};
                t2.cont = c > 0;
                g2.push_back(t2);
            }
            g3.push_back(Mm{AR, co, r, nt, d.m, 1, AR, vpo, r, 0, AR, w2[j], w, 0, w});
        }
        G.run(g1);
        G.run(g2, true);
        G.run(g3);
    }
    // ---- Jacobi on R^T ------------------------------------------------------------------
    launch_bsvd_elem(dblk, nb, nnmax, 0, ar, st);
    W.flags.alloc(size_t(nb) * 8 * sizeof(int), st);
    W.bars.alloc(size_t(nb) * sizeof(unsigned) * 2, st);
    W.sweeps.alloc(size_t(nb) * 2 * sizeof(int), st);
    std::vector<BjDesc> bj(nb);
    auto jacobi = [&](int prec) {
        const int B = bsvd_jacobi_block(nmax, prec);
        for (int j = 0; j < nb; ++j) {
            const BsvdBlk& d = bd[j];
            BjDesc& q = bj[j];
            q = BjDesc{};
            q.X = prec == 0 ? static_cast<void*>(ar + d.r32) : static_cast<void*>(ar + d.ydf);
            q.V = prec == 0 ? static_cast<void*>(ar + d.v32) : static_cast<void*>(ar + d.vdf);
            q.n = d.n;
            q.nb = (d.n + B - 1) / B;
            q.bar = W.bars.as<unsigned>() + j;
            q.flags = W.flags.as<int>() + 8 * j;
            q.sweeps = W.sweeps.as<int>() + 2 * j + prec;
        }
        const int cap = bsvd_jacobi_capacity(nmax, prec);
        TN_REQUIRE(cap >= 1, "block SVD: the Jacobi kernel does not fit an SM");
        TN_CUDA(cudaMemsetAsync(W.flags.p, 0, size_t(nb) * 8 * sizeof(int), st));
        TN_CUDA(cudaMemsetAsync(W.bars.p, 0, size_t(nb) * sizeof(unsigned) * 2, st));
        DevBuf& dd = W.bjd[prec];
        dd.alloc(bj.size() * sizeof(BjDesc), st);
        // matrices in chunks of at most `cap` groups (one co-resident launch each)
        for (int j0 = 0; j0 < nb; j0 += cap) {
            const int j1 = std::min(nb, j0 + cap);
            std::vector<BjDesc> chunk(bj.begin() + j0, bj.begin() + j1);
            assign_ctas(chunk, cap);
            int nctas = 0;
            for (auto& q : chunk) nctas = std::max(nctas, q.cta0 + q.ncta);
            BjDesc* dptr = dd.as<BjDesc>() + j0;
            TN_CUDA(cudaMemcpyAsync(dptr, chunk.data(), chunk.size() * sizeof(BjDesc),
                                    cudaMemcpyHostToDevice, st));
            launch_bsvd_jacobi(dptr, j1 - j0, nctas, nmax, prec, ctx->err.as<int>(), st);
        }
    };
    jacobi(0);
    launch_bsvd_elem(dblk, nb, nnmax, 1, ar, st);
    // two Newton-Schulz steps: V <- V (1.5 I - 0.5 V^T V), back in v64
    for (int it = 0; it < 2; ++it) {
        std::vector<Mm> gram, upd;
        for (int j = 0; j < nb; ++j) {
            const BsvdBlk& d = bd[j];
            const int64_t vin = it == 0 ? d.v64 : d.v64b, vout = it == 0 ? d.v64b : d.v64;
            gram.push_back(Mm{AR, d.g64, d.n, d.n, d.n, 0, AR, vin, d.n, 1, AR, vin, d.n, 0, d.n});
            upd.push_back(Mm{AR, vout, d.n, d.n, d.n, 0, AR, vin, d.n, 0, AR, d.g64, d.n, 0, d.n});
        }
        G.run(gram);
        launch_bsvd_elem(dblk, nb, nnmax, 2, ar, st);
        G.run(upd);
    }
    {
        std::vector<Mm> y;
        for (int j = 0; j < nb; ++j) {
            const BsvdBlk& d = bd[j];
            y.push_back(Mm{AR, d.y64, d.n, d.n, d.n, 0, AR, d.rt64, d.n, 0, AR, d.v64, d.n, 0, d.n});
        }
        G.run(y);
    }
    launch_bsvd_elem(dblk, nb, nnmax, 3, ar, st);
    jacobi(1);
    launch_bsvd_finish(dblk, nb, ar, QV, PY, S, perm, st);
    // ---- QV = Q [V; 0], panels in reverse ------------------------------------------------
    for (auto it = panels.rbegin(); it != panels.rend(); ++it) {
        const int p0 = it->first, pw = it->second;
        std::vector<Mm> g1, g2, g3;
        for (int j = 0; j < nb; ++j) {
            const BsvdBlk& d = bd[j];
            if (p0 >= d.n) continue;
            const int w = std::min(pw, d.n - p0), r = d.m - p0;
            const int64_t vpo = d.vp + int64_t(p0) * d.m;
            const int64_t zo = d.x_off + p0;
            const int64_t tmo = d.tm + int64_t(p0) * 64 + int64_t(w) * w;
            // W1_c = V_c^T Z_c over row chunks (split k), W2 = (-T) sum_c W1_c, Z += V W2
            const int nch = (r + KC - 1) / KC;
            for (int c = 0; c < nch; ++c) {
                const int r0 = c * KC, rc = std::min(KC, r - r0);
                const int64_t wc = w1[j] + int64_t(c) * w * d.n;
                g1.push_back(Mm{AR, wc, w, d.n, w, 0, AR, vpo + r0, r, 1, QB, zo + r0, d.m, 0, rc});
                Mm t2{AR, w2[j], w, d.n, w, 0, AR, tmo, w, 0, AR, wc, w, 0, w};
                t2.cont = c > 0;
                g2.push_back(t2);
            }
            g3.push_back(Mm{QB, zo, r, d.n, d.m, 1, AR, vpo, r, 0, AR, w2[j], w, 0, w});
        }
        G.run(g1);
        G.run(g2, true);
        G.run(g3);
    }
    if (stats) {
        stats->gemm_flops += G.flops;
        std::vector<int> sw(size_t(nb) * 2);
        TN_CUDA(cudaMemcpyAsync(sw.data(), W.sweeps.p, sw.size() * sizeof(int),
                                cudaMemcpyDeviceToHost, st));
        TN_CUDA(cudaStreamSynchronize(st));
        for (int j = 0; j < nb; ++j) {
            const double n = bd[j].n;
            // one-sided Jacobi: per rotated pair 3 n-long dots (6 n flops) and the rotation of
            // the two columns of X and V (12 n flops); n (n - 1) / 2 pairs per sweep
            stats->jacobi_flops += (sw[2 * j] + sw[2 * j + 1]) * 0.5 * n * (n - 1) * 18.0 * n;
            stats->sweeps32 = std::max(stats->sweeps32, sw[2 * j]);
            stats->sweeps_df = std::max(stats->sweeps_df, sw[2 * j + 1]);
        }
    }
}

}  // namespace tn
