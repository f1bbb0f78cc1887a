// Sweep engine: environments (ProjMPO restated), two-site effective Hamiltonian plans,
// thick-restart Lanczos driver, block SVD truncation and the full sweep, behind the C ABI
// of include/tennet.h.
#include "engine.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>

using namespace tn;

namespace {

thread_local std::string g_err;

int fail(const std::exception& e) {
    g_err = e.what();
    if (auto* te = dynamic_cast<const Error*>(&e)) return te->code;
    return TN_E_INVALID;
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return TN_OK;
    } catch (const std::bad_alloc&) {
        g_err = "host allocation failed";
        return TN_E_NOMEM;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// -------------------------------------------------------------------------------------
// small dense helpers (host, FP64)
// -------------------------------------------------------------------------------------

// Eigen-decomposition of a small symmetric matrix (cyclic Jacobi), ascending order.
// A is n x n row-major; on return D[n], U (row-major, columns = eigenvectors).
void sym_eig(int n, std::vector<double> A, std::vector<double>& D, std::vector<double>& U) {
    U.assign(size_t(n) * n, 0.0);
    for (int i = 0; i < n; ++i) U[size_t(i) * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += A[size_t(i) * n + j] * A[size_t(i) * n + j];
                if (i != j) off += A[size_t(i) * n + j] * A[size_t(i) * n + j];
            }
        if (off <= 1e-34 * tot || off == 0.0) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[size_t(p) * n + q];
                if (apq == 0.0) continue;
                const double app = A[size_t(p) * n + p], aqq = A[size_t(q) * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // A = J^T A J
                    const double akp = A[size_t(k) * n + p], akq = A[size_t(k) * n + q];
                    A[size_t(k) * n + p] = c * akp - s * akq;
                    A[size_t(k) * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[size_t(p) * n + k], aqk = A[size_t(q) * n + k];
                    A[size_t(p) * n + k] = c * apk - s * aqk;
                    A[size_t(q) * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double ukp = U[size_t(k) * n + p], ukq = U[size_t(k) * n + q];
                    U[size_t(k) * n + p] = c * ukp - s * ukq;
                    U[size_t(k) * n + q] = s * ukp + c * ukq;
                }
            }
    }
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return A[size_t(a) * n + a] < A[size_t(b) * n + b]; });
    D.resize(n);
    std::vector<double> U2(size_t(n) * n);
    for (int j = 0; j < n; ++j) {
        D[j] = A[size_t(idx[j]) * n + idx[j]];
        for (int i = 0; i < n; ++i) U2[size_t(i) * n + j] = U[size_t(i) * n + idx[j]];
    }
    U.swap(U2);
}

// ITensors truncate! restated: P sorted descending.  Returns kept count by rank, the
// relative discarded weight and the cut value (per block, S^2 > docut is kept).
struct TruncOut {
    int n;
    double truncerr, docut;
};
TruncOut truncation_rule(std::vector<double> P, int maxdim, int mindim, double cutoff) {
    const int origm = (int)P.size();
    for (int n = origm - 1; n >= 0; --n) {
        if (P[n] >= 0) break;
        P[n] = 0.0;
    }
    int n = origm;
    double truncerr = 0.0;
    while (n > maxdim) {
        truncerr += P[n - 1];
        --n;
    }
    double scale = 0.0;
    for (double x : P) scale += x;
    if (scale == 0.0) scale = 1.0;
    while (n > mindim && truncerr + P[n - 1] <= cutoff * scale) {
        truncerr += P[n - 1];
        --n;
    }
    truncerr /= scale;
    if (n < 1) n = 1;
    double docut = 0.0;
    if (n < origm) {
        docut = 0.5 * (P[n - 1] + P[n]);
        if (std::fabs(P[n - 1] - P[n]) < 1e-3 * P[n - 1]) docut += 1e-3 * P[n - 1];
    }
    return TruncOut{n, truncerr, docut};
}

void check_params(const tn_update_params* p) {
    TN_REQUIRE(p != nullptr, "null update parameters");
    TN_REQUIRE(p->maxdim >= 1 && p->mindim >= 1, "maxdim and mindim must be >= 1");
    TN_REQUIRE(p->krylovdim >= 1 && p->krylovdim <= 31, "krylovdim must be in [1, 31]");
    TN_REQUIRE(p->maxiter >= 1, "maxiter must be >= 1");
    TN_REQUIRE(p->noise >= 0.0 && std::isfinite(p->noise), "noise must be finite and >= 0");
}

// -------------------------------------------------------------------------------------
// environments
// -------------------------------------------------------------------------------------
void sync(tn_ctx* c) { TN_CUDA(cudaStreamSynchronize(c->stream)); }

void make_trivial_env(tn_ctx* ctx, tn_envt& E, const Link& link, const std::vector<int>& delta,
                      int planes = 1) {
    E.lay = make_env_layout(link, delta);
    TN_REQUIRE(E.lay.size == 1, "boundary link and boundary MPO link must have dimension 1");
    E.buf.alloc(sizeof(double) * planes, ctx->stream);
    const double one[3] = {1.0, 0.0, 0.0};
    TN_CUDA(cudaMemcpyAsync(E.buf.p, one, sizeof(double) * planes, cudaMemcpyHostToDevice,
                            ctx->stream));
    TN_CUDA(cudaStreamSynchronize(ctx->stream));
}

// the imaginary plane of a complex buffer of `plane` values per plane into slot s + S_IM
void set_im(Bases& bs, int slot, int64_t plane) { bs.p[slot + S_IM] = bs.p[slot] + plane; }

// planes of an environment buffer: 1 (real), 3 (complex: re, im, -im)
int env_planes(const tn_mps* psi) { return psi->cplx ? 3 : 1; }

// a complex plan with every segment positive: a negative segment reads the negated
// imaginary plane of one of its operands from slot negslot[s] (s its real slot) instead
std::unique_ptr<GemmPlan> unsigned_plan(const GemmPlan& c, const int (&negslot)[S_IM]) {
    auto u = std::make_unique<GemmPlan>();
    for (const Task& t : c.tasks) {
        u->add_task(t.cbuf, t.coff, t.m, t.n, t.ldc, t.accum);
        for (int j = 0; j < t.nseg; ++j) {
            Seg sg = c.segs[size_t(t.seg0 + j)];
            if (sg.sgn < 0) {
                if (sg.abuf >= S_IM && negslot[sg.abuf - S_IM] >= 0)
                    sg.abuf = negslot[sg.abuf - S_IM];
                else if (sg.bbuf >= S_IM && negslot[sg.bbuf - S_IM] >= 0)
                    sg.bbuf = negslot[sg.bbuf - S_IM];
                else
                    TN_REQUIRE(false, "internal: no negated plane for a negative segment");
            }
            u->add_seg(sg.abuf, sg.aoff, sg.lda, sg.ta, sg.bbuf, sg.boff, sg.ldb, sg.tb, sg.k, 1);
        }
    }
    return u;
}

bool need_left(const tn_mpo* H, int site, int a, int s) {
    for (int b = 0; b < H->wd[site + 1]; ++b)
        for (int sp = 0; sp < H->d; ++sp)
            if (H->at(site, a, b, sp, s) != 0.0) return true;
    return false;
}
bool need_right(const tn_mpo* H, int site, int c, int s) {
    for (int a = 0; a < H->wd[site]; ++a)
        for (int sp = 0; sp < H->d; ++sp)
            if (H->at(site, a, c, sp, s) != 0.0) return true;
    return false;
}

// -------------------------------------------------------------------------------------
// split-precision GEMM plans
// -------------------------------------------------------------------------------------
template <class T>
void upload_vec(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
    b.alloc(std::max<size_t>(v.size() * sizeof(T), 16), s);
    if (!v.empty())
        TN_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

std::unique_ptr<SplitPlan> make_split(const GemmPlan& g, int slices, bool a_static,
                                      bool b_static, cudaStream_t st, bool own_packs = true) {
    for (const Seg& sg : g.segs)
        TN_REQUIRE(sg.sgn == 1, "internal: the split-precision GEMM takes unsigned segments");
    auto sp = std::make_unique<SplitPlan>();
    sp->slices = slices;
    sp->a_static = a_static;
    sp->b_static = b_static;
    const int KT = split_ktile(), RA = split_tile_rows_a(), RB = split_tile_rows_b();
    const int64_t TA = split_tile_bytes_a(), TB = split_tile_bytes_b();
    int64_t aoff = 0, boff = 0, eao = 0, ebo = 0;
    std::map<std::vector<int64_t>, std::pair<int64_t, int64_t>> bseen;  // B signature -> offsets
    std::map<std::vector<int64_t>, std::pair<int64_t, int64_t>> aseen;  // A signature -> offsets
    for (size_t ti = 0; ti < g.tasks.size(); ++ti) {
        const Task& t = g.tasks[ti];
        struct KT3 { int seg, k0, kv; };
        std::vector<KT3> kts;
        for (int j = 0; j < t.nseg; ++j) {
            const Seg& sg = g.segs[t.seg0 + j];
            for (int k0 = 0; k0 < sg.k; k0 += KT) kts.push_back(KT3{t.seg0 + j, k0, std::min(KT, sg.k - k0)});
        }
        const int nkt = (int)kts.size();
        const int mt = (t.m + RA - 1) / RA, nt = (t.n + RB - 1) / RB;
        // tasks whose B operand is the same matrix (e.g. one two-site slab multiplied by
        // the environment blocks of every MPO state) share one packed copy
        std::vector<int64_t> bsig;
        bsig.push_back(t.n);
        for (int j = 0; j < t.nseg; ++j) {
            const Seg& sg = g.segs[t.seg0 + j];
            bsig.insert(bsig.end(), {int64_t(sg.bbuf), sg.boff, int64_t(sg.ldb), int64_t(sg.tb),
                                     int64_t(sg.k)});
        }
        auto bit = bseen.find(bsig);
        const bool bnew = bit == bseen.end();
        // likewise for A (e.g. one node tensor multiplied on the same leg by several matrices)
        std::vector<int64_t> asig;
        asig.push_back(t.m);
        for (int j = 0; j < t.nseg; ++j) {
            const Seg& sg = g.segs[t.seg0 + j];
            asig.insert(asig.end(), {int64_t(sg.abuf), sg.aoff, int64_t(sg.lda), int64_t(sg.ta),
                                     int64_t(sg.k)});
        }
        auto ait = aseen.find(asig);
        const bool anew = ait == aseen.end();
        SplitTask stsk{};
        stsk.coff = t.coff;
        stsk.a_off = anew ? aoff : ait->second.first;
        stsk.b_off = bnew ? boff : bit->second.first;
        stsk.cbuf = t.cbuf;
        stsk.m = t.m;
        stsk.n = t.n;
        stsk.ldc = t.ldc;
        stsk.nkt = nkt;
        stsk.ea_off = anew ? int32_t(eao) : int32_t(ait->second.second);
        stsk.eb_off = bnew ? int32_t(ebo) : int32_t(bit->second.second);
        stsk.accum = t.accum;
        sp->tasks.push_back(stsk);
        const int akt0 = (int)sp->aks.size(), bkt0 = (int)sp->bks.size();
        for (const auto& k : kts) {
            const Seg& sg = g.segs[k.seg];
            if (anew) {
                KTileSrc a{};
                a.buf = sg.abuf;
                a.sr = sg.ta ? sg.lda : 1;
                a.sk = sg.ta ? 1 : sg.lda;
                a.off = sg.aoff + int64_t(k.k0) * a.sk;
                a.kvalid = k.kv;
                sp->aks.push_back(a);
            }
            if (!bnew) continue;
            KTileSrc bsrc{};
            bsrc.buf = sg.bbuf;
            bsrc.sr = sg.tb ? 1 : sg.ldb;
            bsrc.sk = sg.tb ? sg.ldb : 1;
            bsrc.off = sg.boff + int64_t(k.k0) * bsrc.sk;
            bsrc.kvalid = k.kv;
            sp->bks.push_back(bsrc);
        }
        if (anew)
            for (int mi = 0; mi < mt; ++mi)
                sp->ajobs.push_back(PackJob{aoff + int64_t(mi) * nkt * slices * TA, akt0, nkt,
                                            std::min(RA, t.m - mi * RA), mi * RA,
                                            int32_t(eao + mi * RA), 0});
        if (bnew)
            for (int ni = 0; ni < nt; ++ni)
                sp->bjobs.push_back(PackJob{boff + int64_t(ni) * nkt * slices * TB, bkt0, nkt,
                                            std::min(RB, t.n - ni * RB), ni * RB,
                                            int32_t(ebo + ni * RB), 0});
        for (int mi = 0; mi < mt; ++mi)
            for (int ni = 0; ni < nt; ++ni) sp->items.push_back(SplitItem{int32_t(ti), mi, ni, 0});
        if (anew) {
            aseen.emplace(asig, std::make_pair(aoff, eao));
            aoff += int64_t(mt) * nkt * slices * TA;
            eao += int64_t(mt) * RA;
        }
        if (bnew) {
            bseen.emplace(bsig, std::make_pair(boff, ebo));
            boff += int64_t(nt) * nkt * slices * TB;
            ebo += int64_t(nt) * RB;
        }
    }
    std::stable_sort(sp->items.begin(), sp->items.end(), [&](const SplitItem& x, const SplitItem& y) {
        return sp->tasks[x.task].nkt > sp->tasks[y.task].nkt;
    });
    sp->abytes = aoff;
    sp->bbytes = boff;
    sp->ea_n = eao;
    sp->eb_n = ebo;
    for (const auto& j : sp->ajobs) sp->a_maxnkt = std::max(sp->a_maxnkt, j.nkt);
    for (const auto& j : sp->bjobs) sp->b_maxnkt = std::max(sp->b_maxnkt, j.nkt);
    sp->amax.alloc(size_t(std::max<int64_t>(eao, 1)) * 8, st);
    sp->bmax.alloc(size_t(std::max<int64_t>(ebo, 1)) * 8, st);
    upload_vec(sp->dtasks, sp->tasks, st);
    upload_vec(sp->ditems, sp->items, st);
    upload_vec(sp->dajobs, sp->ajobs, st);
    upload_vec(sp->dbjobs, sp->bjobs, st);
    upload_vec(sp->daks, sp->aks, st);
    upload_vec(sp->dbks, sp->bks, st);
    if (own_packs) {
        sp->apack.alloc(size_t(std::max<int64_t>(aoff, 1024)), st);
        sp->bpack.alloc(size_t(std::max<int64_t>(boff, 1024)), st);
        sp->ea.alloc(size_t(std::max<int64_t>(eao, 4)) * 4, st);
        sp->eb.alloc(size_t(std::max<int64_t>(ebo, 4)) * 4, st);
        sp->ap = sp->apack.as<uint8_t>();
        sp->bp = sp->bpack.as<uint8_t>();
        sp->eap = sp->ea.as<int>();
        sp->ebp = sp->eb.as<int>();
    }
    return sp;
}

// pack the operands that need it, then run the tensor-core GEMM; times packs and MMA
void run_split(tn_ctx* ctx, SplitPlan& sp, const Bases& bs, int* mma_ev0, int* mma_ev1) {
    cudaStream_t st = ctx->stream;
    const int p0 = ctx->timer.mark();
    if (!sp.a_static || !sp.a_packed) {
        launch_split_pack(sp.dajobs.as<PackJob>(), (int)sp.ajobs.size(), sp.daks.as<KTileSrc>(), bs,
                          sp.ap, sp.eap, sp.slices, split_tile_rows_a(), st, sp.a_maxnkt,
                          sp.amax.as<unsigned long long>(), sp.ea_n);
        sp.a_packed = true;
    }
    if (!sp.b_static || !sp.b_packed) {
        launch_split_pack(sp.dbjobs.as<PackJob>(), (int)sp.bjobs.size(), sp.dbks.as<KTileSrc>(), bs,
                          sp.bp, sp.ebp, sp.slices, split_tile_rows_b(), st, sp.b_maxnkt,
                          sp.bmax.as<unsigned long long>(), sp.eb_n);
        sp.b_packed = true;
    }
    const int p1 = ctx->timer.mark();
    ctx->timer.add(T_PACK, p0, p1);
    launch_split_gemm(sp.ditems.as<SplitItem>(), (int)sp.items.size(), sp.dtasks.as<SplitTask>(),
                      sp.ap, sp.bp, sp.eap, sp.ebp, bs, sp.slices, ctx->err.as<int>(), ctx->nsm, st);
    const int p2 = ctx->timer.mark();
    if (mma_ev0) *mma_ev0 = p1;
    if (mma_ev1) *mma_ev1 = p2;
}

// grouped GEMM in the context's precision (one-shot plans: every operand packed)
void run_gemm(tn_ctx* ctx, const GemmPlan& g, const Bases& bs) {
    if (g.tasks.empty()) return;
    if (ctx->prec == TN_PREC_SPLIT) {
        auto sp = make_split(g, ctx->slices, false, false, ctx->stream);
        run_split(ctx, *sp, bs, nullptr, nullptr);
    } else {
        launch_gemm_f64(g, bs, ctx->stream);
    }
}

void check_device_error(tn_ctx* ctx) {
    int e = 0;
    TN_CUDA(cudaMemcpyAsync(&e, ctx->err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    TN_CUDA(cudaStreamSynchronize(ctx->stream));
    if (e) {
        TN_CUDA(cudaMemsetAsync(ctx->err.p, 0, sizeof(int), ctx->stream));
        throw Error(TN_E_TIMEOUT, "a bounded device wait gave up (tensor-core GEMM or "
                                  "cooperative kernel barrier)");
    }
}

// L[i+1] from L[i] and the left isometry at site i.
void env_left_step(tn_env* env, int i) {
    tn_ctx* ctx = env->ctx;
    const tn_mpo* H = env->H;
    const tn_site& A = env->psi->sites[i];
    TN_REQUIRE(A.lay.layout == LG, "left environment needs a left-grouped site tensor");
    const Link& lk = env->psi->links[i];
    const Link& rk = env->psi->links[i + 1];
    const int d = env->psi->d;
    const EnvLayout& Lin = env->L[i].lay;
    tn_envt& Lout = env->L[i + 1];
    Lout.lay = make_env_layout(rk, H->delta[i + 1]);
    const int wl = H->wd[i], wr = H->wd[i + 1];
    // T1(a, il, s) = L(a, il) * A[s](l, r)
    GemmPlan g1, g3;
    CombPlan cb;
    std::vector<int64_t> t1off(size_t(wl) * lk.nsec() * d, -1);
    int64_t t1 = 0;
    for (int ir = 0; ir < rk.nsec(); ++ir)
        for (int s = 0; s < d; ++s) {
            const int sub = A.lay.sub[size_t(ir) * d + s];
            if (sub < 0) continue;
            const int il = A.lay.subsec[size_t(ir) * d + s];
            for (int a = 0; a < wl; ++a) {
                const int64_t lo = Lin.off[size_t(a) * Lin.nsec + il];
                if (lo < 0 || !need_left(H, i, a, s)) continue;
                const int Db = lk.dim[Lin.bra[size_t(a) * Lin.nsec + il]];
                const size_t key = (size_t(a) * lk.nsec() + il) * d + s;
                t1off[key] = t1;
                g1.add_task(S_T1, t1, Db, rk.dim[ir], Db);
                g1.add_seg(S_L, lo, Db, 0, S_X, A.lay.off[ir] + sub, A.lay.rows[ir], 0, lk.dim[il]);
                t1 += int64_t(Db) * rk.dim[ir];
            }
        }
    // T2(b, ir): rows = rows of A block r' (r' = r + delta_b), cols D_r
    std::vector<int64_t> t2off(size_t(wr) * rk.nsec(), -1);
    int64_t t2 = 0;
    for (int b = 0; b < wr; ++b)
        for (int ir = 0; ir < rk.nsec(); ++ir) {
            const int64_t oo = Lout.lay.off[size_t(b) * rk.nsec() + ir];
            if (oo < 0) continue;
            const int irp = Lout.lay.bra[size_t(b) * rk.nsec() + ir];
            const int rowsA = A.lay.rows[irp];
            t2off[size_t(b) * rk.nsec() + ir] = t2;
            for (int sp = 0; sp < d; ++sp) {
                const int sub = A.lay.sub[size_t(irp) * d + sp];
                if (sub < 0) continue;
                const int ilpp = A.lay.subsec[size_t(irp) * d + sp];
                CombOut o;
                o.doff = t2 + sub;
                o.dbuf = S_T2;
                o.ldd = rowsA;
                o.rows = lk.dim[ilpp];
                o.cols = rk.dim[ir];
                o.t0 = (int)cb.terms.size();
                o.nt = 0;
                for (int a = 0; a < wl; ++a)
                    for (int s = 0; s < d; ++s) {
                        const double w = H->at(i, a, b, sp, s);
                        if (w == 0.0) continue;
                        if (A.lay.sub[size_t(ir) * d + s] < 0) continue;
                        const int il = A.lay.subsec[size_t(ir) * d + s];
                        const size_t key = (size_t(a) * lk.nsec() + il) * d + s;
                        if (t1off[key] < 0) continue;
                        if (Lin.bra[size_t(a) * Lin.nsec + il] != ilpp) continue;
                        cb.terms.push_back(CombTerm{t1off[key], S_T1, lk.dim[ilpp], w});
                        o.nt++;
                    }
                cb.flops += 2.0 * o.nt * double(o.rows) * o.cols;
                cb.outs.push_back(o);
            }
            const int Drp = rk.dim[irp];
            g3.add_task(S_Y, oo, Drp, rk.dim[ir], Drp);
            g3.add_seg(S_X, A.lay.off[irp], rowsA, 1, S_T2, t2, rowsA, 0, rowsA);
            t2 += int64_t(rowsA) * rk.dim[ir];
        }
    cudaStream_t st = ctx->stream;
    const int np = env->psi->planes();
    env->t1.alloc(size_t(std::max<int64_t>(t1, 1)) * 8 * np, st);
    env->t2.alloc(size_t(std::max<int64_t>(t2, 1)) * 8 * np, st);
    Lout.buf.alloc(size_t(std::max<int64_t>(Lout.lay.size, 1)) * 8 * env_planes(env->psi.get()),
                     st);
    Bases bs{};
    bs.p[S_L] = env->L[i].buf.d();
    bs.p[S_X] = A.buf.d();
    bs.p[S_T1] = env->t1.d();
    bs.p[S_T2] = env->t2.d();
    bs.p[S_Y] = Lout.buf.d();
    const int e0 = ctx->timer.mark();
    if (np == 2) {  // L' = A^H (L W A): the bra (the transposed site tensor of g3) conjugated
        set_im(bs, S_L, Lin.size);
        set_im(bs, S_X, A.lay.size);
        set_im(bs, S_T1, t1);
        set_im(bs, S_T2, t2);
        set_im(bs, S_Y, Lout.lay.size);
        GemmPlan c1 = complex_plan(g1, 0), c3 = complex_plan(g3, 1u << S_X);
        CombPlan cc = complex_comb(cb);
        c1.finalize(st);
        c3.finalize(st);
        cc.finalize(st);
        launch_gemm_f64(c1, bs, st);
        launch_combine(cc, bs, st);
        launch_gemm_f64(c3, bs, st);
        launch_scale_into(Lout.buf.d() + 2 * Lout.lay.size, Lout.buf.d() + Lout.lay.size,
                          nullptr, -1.0, Lout.lay.size, st);
    } else {
        g1.finalize(st);
        g3.finalize(st);
        cb.finalize(st);
        run_gemm(ctx, g1, bs);
        launch_combine(cb, bs, st);
        run_gemm(ctx, g3, bs);
    }
    if (!env->proj.empty()) proj_left_step(env, i);
    ctx->timer.add(T_ENV, e0, ctx->timer.mark());
}

// R[i-1] from R[i] and the right isometry at site i.
void env_right_step(tn_env* env, int i) {
    tn_ctx* ctx = env->ctx;
    const tn_mpo* H = env->H;
    const tn_site& B = env->psi->sites[i];
    TN_REQUIRE(B.lay.layout == RG, "right environment needs a right-grouped site tensor");
    const Link& lk = env->psi->links[i];
    const Link& rk = env->psi->links[i + 1];
    const int d = env->psi->d;
    const EnvLayout& Rin = env->R[i].lay;
    tn_envt& Rout = env->R[i - 1];
    Rout.lay = make_env_layout(lk, H->delta[i]);
    const int wl = H->wd[i], wr = H->wd[i + 1];
    GemmPlan g1, g3;
    CombPlan cb;
    // T1(c, ir, s) = R(c, ir) * B[s](l, r)^T : D_r' x D_l
    std::vector<int64_t> t1off(size_t(wr) * rk.nsec() * d, -1);
    int64_t t1 = 0;
    for (int il = 0; il < lk.nsec(); ++il)
        for (int s = 0; s < d; ++s) {
            const int sub = B.lay.sub[size_t(il) * d + s];
            if (sub < 0) continue;
            const int ir = B.lay.subsec[size_t(il) * d + s];
            for (int c = 0; c < wr; ++c) {
                const int64_t ro = Rin.off[size_t(c) * Rin.nsec + ir];
                if (ro < 0 || !need_right(H, i, c, s)) continue;
                const int Db = rk.dim[Rin.bra[size_t(c) * Rin.nsec + ir]];
                const size_t key = (size_t(c) * rk.nsec() + ir) * d + s;
                t1off[key] = t1;
                g1.add_task(S_T1, t1, Db, lk.dim[il], Db);
                g1.add_seg(S_R, ro, Db, 0, S_X, B.lay.off[il] + int64_t(sub) * lk.dim[il],
                           lk.dim[il], 1, rk.dim[ir]);
                t1 += int64_t(Db) * lk.dim[il];
            }
        }
    int64_t t2 = 0;
    for (int a = 0; a < wl; ++a)
        for (int il = 0; il < lk.nsec(); ++il) {
            const int64_t oo = Rout.lay.off[size_t(a) * lk.nsec() + il];
            if (oo < 0) continue;
            const int ilp = Rout.lay.bra[size_t(a) * lk.nsec() + il];
            const int colsB = B.lay.cols[ilp];
            for (int sp = 0; sp < d; ++sp) {
                const int sub = B.lay.sub[size_t(ilp) * d + sp];
                if (sub < 0) continue;
                const int irpp = B.lay.subsec[size_t(ilp) * d + sp];
                CombOut o;
                o.doff = t2 + sub;
                o.dbuf = S_T2;
                o.ldd = colsB;
                o.rows = rk.dim[irpp];
                o.cols = lk.dim[il];
                o.t0 = (int)cb.terms.size();
                o.nt = 0;
                for (int c = 0; c < wr; ++c)
                    for (int s = 0; s < d; ++s) {
                        const double w = H->at(i, a, c, sp, s);
                        if (w == 0.0) continue;
                        if (B.lay.sub[size_t(il) * d + s] < 0) continue;
                        const int ir = B.lay.subsec[size_t(il) * d + s];
                        const size_t key = (size_t(c) * rk.nsec() + ir) * d + s;
                        if (t1off[key] < 0) continue;
                        if (Rin.bra[size_t(c) * Rin.nsec + ir] != irpp) continue;
                        cb.terms.push_back(CombTerm{t1off[key], S_T1, rk.dim[irpp], w});
                        o.nt++;
                    }
                cb.flops += 2.0 * o.nt * double(o.rows) * o.cols;
                cb.outs.push_back(o);
            }
            const int Dlp = lk.dim[ilp];
            g3.add_task(S_Y, oo, Dlp, lk.dim[il], Dlp);
            g3.add_seg(S_X, B.lay.off[ilp], Dlp, 0, S_T2, t2, colsB, 0, colsB);
            t2 += int64_t(colsB) * lk.dim[il];
        }
    cudaStream_t st = ctx->stream;
    const int np = env->psi->planes();
    env->t1.alloc(size_t(std::max<int64_t>(t1, 1)) * 8 * np, st);
    env->t2.alloc(size_t(std::max<int64_t>(t2, 1)) * 8 * np, st);
    Rout.buf.alloc(size_t(std::max<int64_t>(Rout.lay.size, 1)) * 8 * env_planes(env->psi.get()),
                     st);
    Bases bs{};
    bs.p[S_R] = env->R[i].buf.d();
    bs.p[S_X] = B.buf.d();
    bs.p[S_T1] = env->t1.d();
    bs.p[S_T2] = env->t2.d();
    bs.p[S_Y] = Rout.buf.d();
    const int e0 = ctx->timer.mark();
    if (np == 2) {  // R' = (B W R) B^H: the bra (the untransposed site tensor of g3) conjugated
        set_im(bs, S_R, Rin.size);
        set_im(bs, S_X, B.lay.size);
        set_im(bs, S_T1, t1);
        set_im(bs, S_T2, t2);
        set_im(bs, S_Y, Rout.lay.size);
        GemmPlan c1 = complex_plan(g1, 0), c3 = complex_plan(g3, 1u << S_X);
        CombPlan cc = complex_comb(cb);
        c1.finalize(st);
        c3.finalize(st);
        cc.finalize(st);
        launch_gemm_f64(c1, bs, st);
        launch_combine(cc, bs, st);
        launch_gemm_f64(c3, bs, st);
        launch_scale_into(Rout.buf.d() + 2 * Rout.lay.size, Rout.buf.d() + Rout.lay.size,
                          nullptr, -1.0, Rout.lay.size, st);
    } else {
        g1.finalize(st);
        g3.finalize(st);
        cb.finalize(st);
        run_gemm(ctx, g1, bs);
        launch_combine(cb, bs, st);
        run_gemm(ctx, g3, bs);
    }
    if (!env->proj.empty()) proj_right_step(env, i);
    ctx->timer.add(T_ENV, e0, ctx->timer.mark());
}

void position(tn_env* env, int pos, int nsite) {
    const int N = env->psi->N;
    TN_REQUIRE(nsite == 1 || nsite == 2, "nsite must be 1 or 2");
    TN_REQUIRE(pos >= 0 && pos + nsite - 1 < N, "position out of range");
    while (env->lpos < pos) {
        env_left_step(env, env->lpos);
        env->lpos++;
    }
    env->lpos = pos;
    const int last = pos + nsite - 1;
    while (env->rpos > last) {
        env_right_step(env, env->rpos);
        env->rpos--;
    }
    env->rpos = last;
    if (env->pos != pos || env->nsite != nsite) {
        env->hp_pos = -1;
        env->h1p_pos = -1;
    }
    env->pos = pos;
    env->nsite = nsite;
}

// -------------------------------------------------------------------------------------
// two-site effective Hamiltonian
// -------------------------------------------------------------------------------------
std::unique_ptr<Heff2Plan> build_heff2(tn_env* env, int p) {
    auto P = std::make_unique<Heff2Plan>();
    const tn_mpo* H = env->H;
    const tn_mps* psi = env->psi.get();
    const int d = psi->d;
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 2];
    const EnvLayout& Lin = env->L[p].lay;
    const EnvLayout& Rin = env->R[p + 1].lay;
    P->ph = make_phi_layout(lk, rk, psi->pq);
    const PhiLayout& ph = P->ph;
    const int w0 = H->wd[p], w1 = H->wd[p + 1], w2 = H->wd[p + 2];
    // step 1: Y(a, il, s1) = L(a, il) * phi[rows (s1, l) of block m]
    std::vector<int64_t> yoff(size_t(w0) * lk.nsec() * d, -1);
    int64_t y = 0;
    for (int mi = 0; mi < ph.nblk(); ++mi)
        for (int s1 = 0; s1 < d; ++s1) {
            const int rs = ph.rsub[size_t(mi) * d + s1];
            if (rs < 0) continue;
            const int il = ph.rsec[size_t(mi) * d + s1];
            for (int a = 0; a < w0; ++a) {
                const int64_t lo = Lin.off[size_t(a) * Lin.nsec + il];
                if (lo < 0 || !need_left(H, p, a, s1)) continue;
                const int Db = lk.dim[Lin.bra[size_t(a) * Lin.nsec + il]];
                yoff[(size_t(a) * lk.nsec() + il) * d + s1] = y;
                P->g1.add_task(S_T1, y, Db, ph.cols[mi], Db);
                P->g1.add_seg(S_L, lo, Db, 0, S_X, ph.off[mi] + rs, ph.rows[mi], 0, lk.dim[il]);
                y += int64_t(Db) * ph.cols[mi];
            }
        }
    // two-site MPO G[a, c](s1' s2', s1 s2) = sum_b W1[a,b,s1',s1] W2[b,c,s2',s2]
    auto G = [&](int a, int c, int s1p, int s2p, int s1, int s2) {
        double g = 0.0;
        for (int b = 0; b < w1; ++b) {
            const double x = H->at(p, a, b, s1p, s1);
            if (x == 0.0) continue;
            g += x * H->at(p + 1, b, c, s2p, s2);
        }
        return g;
    };
    // step 2/3: Z(c, mo, s2') then out[mo][:, cols (s2', r')] = sum_c Z * R(c)^T
    int64_t z = 0;
    for (int mo = 0; mo < ph.nblk(); ++mo)
        for (int s2p = 0; s2p < d; ++s2p) {
            const int cs = ph.csub[size_t(mo) * d + s2p];
            if (cs < 0) continue;
            const int irp = ph.csec[size_t(mo) * d + s2p];
            P->g3.add_task(S_Y, ph.off[mo] + int64_t(cs) * ph.rows[mo], ph.rows[mo], rk.dim[irp],
                           ph.rows[mo]);
            struct PendingSeg { int64_t zo; int64_t ro; int Drp, Dr; };
            std::vector<PendingSeg> segs;
            for (int c = 0; c < w2; ++c) {
                const int ir = rk.find(rk.q[irp] - H->delta[p + 2][c]);
                if (ir < 0) continue;
                const int64_t ro = Rin.off[size_t(c) * Rin.nsec + ir];
                if (ro < 0 || Rin.bra[size_t(c) * Rin.nsec + ir] != irp) continue;
                const int Dr = rk.dim[ir];
                // Z block: rows(mo) x Dr; one combine output per row slab s1'
                bool nonzero = false;
                const size_t out0 = P->cb.outs.size();
                for (int s1p = 0; s1p < d; ++s1p) {
                    const int rs = ph.rsub[size_t(mo) * d + s1p];
                    if (rs < 0) continue;
                    const int ilp = ph.rsec[size_t(mo) * d + s1p];
                    CombOut o;
                    o.doff = z + rs;
                    o.dbuf = S_T2;
                    o.ldd = ph.rows[mo];
                    o.rows = lk.dim[ilp];
                    o.cols = Dr;
                    o.t0 = (int)P->cb.terms.size();
                    o.nt = 0;
                    for (int a = 0; a < w0; ++a) {
                        const int il = lk.find(lk.q[ilp] - H->delta[p][a]);
                        if (il < 0) continue;
                        for (int s1 = 0; s1 < d; ++s1) {
                            const int64_t yo = yoff[(size_t(a) * lk.nsec() + il) * d + s1];
                            if (yo < 0) continue;
                            if (Lin.bra[size_t(a) * Lin.nsec + il] != ilp) continue;
                            const int mi = ph.find(lk.q[il] + psi->pq[s1]);
                            if (mi < 0) continue;
                            for (int s2 = 0; s2 < d; ++s2) {
                                const int csub = ph.csub[size_t(mi) * d + s2];
                                if (csub < 0 || ph.csec[size_t(mi) * d + s2] != ir) continue;
                                const double g = G(a, c, s1p, s2p, s1, s2);
                                if (g == 0.0) continue;
                                P->cb.terms.push_back(
                                    CombTerm{yo + int64_t(csub) * lk.dim[ilp], S_T1, lk.dim[ilp], g});
                                o.nt++;
                            }
                        }
                    }
                    if (o.nt > 0) nonzero = true;
                    P->cb.flops += 2.0 * o.nt * double(o.rows) * o.cols;
                    P->cb.outs.push_back(o);
                }
                if (!nonzero) {  // this c contributes nothing: drop its Z block
                    P->cb.terms.resize(P->cb.outs[out0].t0);
                    P->cb.outs.resize(out0);
                    continue;
                }
                segs.push_back(PendingSeg{z, ro, rk.dim[irp], Dr});
                z += int64_t(ph.rows[mo]) * Dr;
            }
            for (const auto& sg : segs)
                P->g3.add_seg(S_T2, sg.zo, ph.rows[mo], 0, S_R, sg.ro, sg.Drp, 1, sg.Dr);
        }
    cudaStream_t st = env->ctx->stream;
    P->g1.finalize(st);
    P->g3.finalize(st);
    P->cb.finalize(st);
    P->ysize = y;
    P->zsize = z;
    P->yoff = std::move(yoff);
    P->flops = P->g1.flops + P->g3.flops + P->cb.flops;
    if (psi->cplx) {
        P->g1c = complex_plan(P->g1, 0);
        P->g3c = complex_plan(P->g3, 0);
        P->cbc = complex_comb(P->cb);
        P->g1c.finalize(st);
        P->g3c.finalize(st);
        P->cbc.finalize(st);
        P->flops = P->g1c.flops + P->g3c.flops + P->cbc.flops;
    }
    return P;
}

Heff2Plan& heff_plan(tn_env* env) {
    if (env->hp_pos != env->pos || !env->hp) {
        env->hp = build_heff2(env, env->pos);
        env->hp_pos = env->pos;
        cudaStream_t st = env->ctx->stream;
        const int np = env->psi->planes();
        env->t1.alloc(size_t(std::max<int64_t>(env->hp->ysize, 1)) * 8 * np, st);
        env->t2.alloc(size_t(std::max<int64_t>(env->hp->zsize, 1)) * 8 * np, st);
    }
    return *env->hp;
}

void heff_apply(tn_env* env, Heff2Plan& P, const double* x, double* y) {
    tn_ctx* ctx = env->ctx;
    Bases bs{};
    bs.p[S_L] = env->L[env->pos].buf.d();
    bs.p[S_R] = env->R[env->pos + 1].buf.d();
    bs.p[S_X] = const_cast<double*>(x);
    bs.p[S_Y] = y;
    bs.p[S_T1] = env->t1.d();
    bs.p[S_T2] = env->t2.d();
    const int e0 = ctx->timer.mark();
    if (env->psi->cplx) {
        const int64_t ls = env->L[env->pos].lay.size, rs = env->R[env->pos + 1].lay.size;
        set_im(bs, S_L, ls);
        set_im(bs, S_R, rs);
        set_im(bs, S_X, P.ph.size);
        set_im(bs, S_Y, P.ph.size);
        set_im(bs, S_T1, P.ysize);
        set_im(bs, S_T2, P.zsize);
        if (ctx->prec == TN_PREC_SPLIT) {
            // unsigned forms: -Im L and -Im R (third environment planes) in slots S_A, S_B
            bs.p[S_A] = bs.p[S_L] + 2 * ls;
            bs.p[S_B] = bs.p[S_R] + 2 * rs;
            if (!P.s1c) {
                const int nl[S_IM] = {S_A, -1, -1, -1, -1, -1, -1, -1};
                const int nr[S_IM] = {-1, S_B, -1, -1, -1, -1, -1, -1};
                auto u1 = unsigned_plan(P.g1c, nl);
                auto u3 = unsigned_plan(P.g3c, nr);
                P.s1c = make_split(*u1, ctx->slices, true, false, ctx->stream);   // A = L
                P.s3c = make_split(*u3, ctx->slices, false, true, ctx->stream);   // B = R
            }
            int a0 = -1, a1 = -1, b0 = -1, b1 = -1;
            run_split(ctx, *P.s1c, bs, &a0, &a1);
            launch_combine(P.cbc, bs, ctx->stream);
            run_split(ctx, *P.s3c, bs, &b0, &b1);
            ctx->timer.add(T_GEMM, a0, a1);
            ctx->timer.add(T_GEMM, b0, b1);
        } else {
            launch_gemm_f64(P.g1c, bs, ctx->stream);
            launch_combine(P.cbc, bs, ctx->stream);
            launch_gemm_f64(P.g3c, bs, ctx->stream);
        }
        ctx->timer.add(T_HEFF, e0, ctx->timer.mark());
        env->matvecs++;
        env->heff_flops += P.flops;
        env->gemm_flops += P.g1c.flops + P.g3c.flops;
        env->gemm_launches += (P.g1c.tiles.empty() ? 0 : 1) + (P.g3c.tiles.empty() ? 0 : 1);
        return;
    }
    if (ctx->prec == TN_PREC_SPLIT) {
        if (!P.s1) P.s1 = make_split(P.g1, ctx->slices, true, false, ctx->stream);   // A = L
        if (!P.s3) P.s3 = make_split(P.g3, ctx->slices, false, true, ctx->stream);   // B = R
        int a0 = -1, a1 = -1, b0 = -1, b1 = -1;
        run_split(ctx, *P.s1, bs, &a0, &a1);
        launch_combine(P.cb, bs, ctx->stream);
        run_split(ctx, *P.s3, bs, &b0, &b1);
        ctx->timer.add(T_GEMM, a0, a1);
        ctx->timer.add(T_GEMM, b0, b1);
        ctx->timer.add(T_HEFF, e0, ctx->timer.mark());
    } else {
        launch_gemm_f64(P.g1, bs, ctx->stream);
        const int e1 = ctx->timer.mark();
        launch_combine(P.cb, bs, ctx->stream);
        const int e2 = ctx->timer.mark();
        launch_gemm_f64(P.g3, bs, ctx->stream);
        const int e3 = ctx->timer.mark();
        ctx->timer.add(T_HEFF, e0, e3);
        ctx->timer.add(T_GEMM, e0, e1);
        ctx->timer.add(T_GEMM, e2, e3);
    }
    env->matvecs++;
    env->heff_flops += P.flops;
    env->gemm_flops += P.g1.flops + P.g3.flops;
    env->gemm_launches += (P.g1.tiles.empty() ? 0 : 1) + (P.g3.tiles.empty() ? 0 : 1);
}

// -------------------------------------------------------------------------------------
// one-site effective Hamiltonian (right-grouped one-site tensor)
// -------------------------------------------------------------------------------------
std::unique_ptr<Heff1Plan> build_heff1(tn_env* env, int p) {
    auto P = std::make_unique<Heff1Plan>();
    const tn_mpo* H = env->H;
    const tn_mps* psi = env->psi.get();
    const int d = psi->d;
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 1];
    const EnvLayout& Lin = env->L[p].lay;
    const EnvLayout& Rin = env->R[p].lay;
    P->lay = make_site_layout(RG, lk, rk, psi->pq);
    const SiteLayout& lay = P->lay;
    const int wl = H->wd[p], wr = H->wd[p + 1];
    // step 1: Y(a, il) = L(a, il) * v block il  (D_l' x cols(il))
    std::vector<int64_t> yoff(size_t(wl) * lk.nsec(), -1);
    int64_t y = 0;
    for (int il = 0; il < lk.nsec(); ++il) {
        if (lay.cols[il] == 0) continue;
        for (int a = 0; a < wl; ++a) {
            const int64_t lo = Lin.off[size_t(a) * Lin.nsec + il];
            if (lo < 0) continue;
            bool need = false;
            for (int s2 = 0; s2 < d; ++s2) need = need || need_left(H, p, a, s2);
            if (!need) continue;
            const int Db = lk.dim[Lin.bra[size_t(a) * Lin.nsec + il]];
            yoff[size_t(a) * lk.nsec() + il] = y;
            P->g1.add_task(S_T1, y, Db, lay.cols[il], Db);
            P->g1.add_seg(S_L, lo, Db, 0, S_X, lay.off[il], lk.dim[il], 0, lk.dim[il]);
            y += int64_t(Db) * lay.cols[il];
        }
    }
    // steps 2/3: Z(b, il', s') then out(il')[:, slab (s', r')] = sum_b Z * R(b)^T
    int64_t z = 0;
    for (int ilp = 0; ilp < lk.nsec(); ++ilp)
        for (int sp = 0; sp < d; ++sp) {
            const int csub = lay.sub[size_t(ilp) * d + sp];
            if (csub < 0) continue;
            const int irp = lay.subsec[size_t(ilp) * d + sp];
            const int Dlp = lk.dim[ilp];
            P->g3.add_task(S_Y, lay.off[ilp] + int64_t(csub) * Dlp, Dlp, rk.dim[irp], Dlp);
            struct PendingSeg { int64_t zo, ro; int Drp, Dr; };
            std::vector<PendingSeg> segs;
            for (int b = 0; b < wr; ++b) {
                const int ir = rk.find(rk.q[irp] - H->delta[p + 1][b]);
                if (ir < 0) continue;
                const int64_t ro = Rin.off[size_t(b) * Rin.nsec + ir];
                if (ro < 0 || Rin.bra[size_t(b) * Rin.nsec + ir] != irp) continue;
                const int Dr = rk.dim[ir];
                CombOut o;
                o.doff = z;
                o.dbuf = S_T2;
                o.ldd = Dlp;
                o.rows = Dlp;
                o.cols = Dr;
                o.t0 = (int)P->cb.terms.size();
                o.nt = 0;
                for (int a = 0; a < wl; ++a) {
                    const int il = lk.find(lk.q[ilp] - H->delta[p][a]);
                    if (il < 0) continue;
                    const int64_t yo = yoff[size_t(a) * lk.nsec() + il];
                    if (yo < 0 || Lin.bra[size_t(a) * Lin.nsec + il] != ilp) continue;
                    for (int s = 0; s < d; ++s) {
                        const double wv = H->at(p, a, b, sp, s);
                        if (wv == 0.0) continue;
                        const int ys = lay.sub[size_t(il) * d + s];
                        if (ys < 0 || lay.subsec[size_t(il) * d + s] != ir) continue;
                        P->cb.terms.push_back(CombTerm{yo + int64_t(ys) * Dlp, S_T1, Dlp, wv});
                        o.nt++;
                    }
                }
                if (o.nt == 0) {
                    P->cb.terms.resize(o.t0);
                    continue;
                }
                P->cb.flops += 2.0 * o.nt * double(o.rows) * o.cols;
                P->cb.outs.push_back(o);
                segs.push_back(PendingSeg{z, ro, rk.dim[irp], Dr});
                z += int64_t(Dlp) * Dr;
            }
            for (const auto& sg : segs)
                P->g3.add_seg(S_T2, sg.zo, Dlp, 0, S_R, sg.ro, sg.Drp, 1, sg.Dr);
        }
    cudaStream_t st = env->ctx->stream;
    P->g1.finalize(st);
    P->g3.finalize(st);
    P->cb.finalize(st);
    P->ysize = y;
    P->zsize = z;
    P->flops = P->g1.flops + P->g3.flops + P->cb.flops;
    if (psi->cplx) {
        P->g1c = complex_plan(P->g1, 0);
        P->g3c = complex_plan(P->g3, 0);
        P->cbc = complex_comb(P->cb);
        P->g1c.finalize(st);
        P->g3c.finalize(st);
        P->cbc.finalize(st);
        P->flops = P->g1c.flops + P->g3c.flops + P->cbc.flops;
    }
    return P;
}

Heff1Plan& heff1_plan(tn_env* env) {
    if (env->h1p_pos != env->pos || !env->h1p) {
        env->h1p = build_heff1(env, env->pos);
        env->h1p_pos = env->pos;
        cudaStream_t st = env->ctx->stream;
        const int np = env->psi->planes();
        env->t1.alloc(size_t(std::max<int64_t>(env->h1p->ysize, 1)) * 8 * np, st);
        env->t2.alloc(size_t(std::max<int64_t>(env->h1p->zsize, 1)) * 8 * np, st);
    }
    return *env->h1p;
}

void heff1_apply(tn_env* env, Heff1Plan& P, const double* x, double* y) {
    tn_ctx* ctx = env->ctx;
    Bases bs{};
    bs.p[S_L] = env->L[env->pos].buf.d();
    bs.p[S_R] = env->R[env->pos].buf.d();
    bs.p[S_X] = const_cast<double*>(x);
    bs.p[S_Y] = y;
    bs.p[S_T1] = env->t1.d();
    bs.p[S_T2] = env->t2.d();
    const int e0 = ctx->timer.mark();
    if (env->psi->cplx) {
        const int64_t ls = env->L[env->pos].lay.size, rs = env->R[env->pos].lay.size;
        set_im(bs, S_L, ls);
        set_im(bs, S_R, rs);
        set_im(bs, S_X, P.lay.size);
        set_im(bs, S_Y, P.lay.size);
        set_im(bs, S_T1, P.ysize);
        set_im(bs, S_T2, P.zsize);
        if (ctx->prec == TN_PREC_SPLIT) {
            // unsigned forms: -Im L and -Im R (third environment planes) in slots S_A, S_B
            bs.p[S_A] = bs.p[S_L] + 2 * ls;
            bs.p[S_B] = bs.p[S_R] + 2 * rs;
            if (!P.s1c) {
                const int nl[S_IM] = {S_A, -1, -1, -1, -1, -1, -1, -1};
                const int nr[S_IM] = {-1, S_B, -1, -1, -1, -1, -1, -1};
                auto u1 = unsigned_plan(P.g1c, nl);
                auto u3 = unsigned_plan(P.g3c, nr);
                P.s1c = make_split(*u1, ctx->slices, true, false, ctx->stream);   // A = L
                P.s3c = make_split(*u3, ctx->slices, false, true, ctx->stream);   // B = R
            }
            int a0 = -1, a1 = -1, b0 = -1, b1 = -1;
            run_split(ctx, *P.s1c, bs, &a0, &a1);
            launch_combine(P.cbc, bs, ctx->stream);
            run_split(ctx, *P.s3c, bs, &b0, &b1);
            ctx->timer.add(T_GEMM, a0, a1);
            ctx->timer.add(T_GEMM, b0, b1);
        } else {
            launch_gemm_f64(P.g1c, bs, ctx->stream);
            launch_combine(P.cbc, bs, ctx->stream);
            launch_gemm_f64(P.g3c, bs, ctx->stream);
        }
        ctx->timer.add(T_HEFF, e0, ctx->timer.mark());
        env->matvecs++;
        env->heff_flops += P.flops;
        env->gemm_flops += P.g1c.flops + P.g3c.flops;
        env->gemm_launches += (P.g1c.tiles.empty() ? 0 : 1) + (P.g3c.tiles.empty() ? 0 : 1);
        return;
    }
    if (ctx->prec == TN_PREC_SPLIT) {
        if (!P.s1) P.s1 = make_split(P.g1, ctx->slices, true, false, ctx->stream);
        if (!P.s3) P.s3 = make_split(P.g3, ctx->slices, false, true, ctx->stream);
        int a0 = -1, a1 = -1, b0 = -1, b1 = -1;
        run_split(ctx, *P.s1, bs, &a0, &a1);
        launch_combine(P.cb, bs, ctx->stream);
        run_split(ctx, *P.s3, bs, &b0, &b1);
        ctx->timer.add(T_GEMM, a0, a1);
        ctx->timer.add(T_GEMM, b0, b1);
    } else {
        launch_gemm_f64(P.g1, bs, ctx->stream);
        launch_combine(P.cb, bs, ctx->stream);
        launch_gemm_f64(P.g3, bs, ctx->stream);
    }
    ctx->timer.add(T_HEFF, e0, ctx->timer.mark());
    env->matvecs++;
    env->heff_flops += P.flops;
    env->gemm_flops += P.g1.flops + P.g3.flops;
    env->gemm_launches += (P.g1.tiles.empty() ? 0 : 1) + (P.g3.tiles.empty() ? 0 : 1);
}

// copy a site tensor between the left-grouped and right-grouped layouts (block copies)
void regroup(tn_ctx* ctx, const SiteLayout& src, const double* sp, const SiteLayout& dst,
             double* dp, const Link& lk, const Link& rk, int planes = 1) {
    CombPlan cb;
    const int d = src.d;
    for (int b = 0; b < src.nblk(); ++b)
        for (int s = 0; s < d; ++s) {
            const int sub = src.sub[size_t(b) * d + s];
            if (sub < 0) continue;
            const int oth = src.subsec[size_t(b) * d + s];
            const int il = src.layout == LG ? oth : b;
            const int ir = src.layout == LG ? b : oth;
            const int db = dst.layout == LG ? ir : il;
            const int dsub = dst.sub[size_t(db) * d + s];
            TN_REQUIRE(dsub >= 0, "internal: regroup layout mismatch");
            CombOut o;
            o.rows = lk.dim[il];
            o.cols = rk.dim[ir];
            o.dbuf = S_Y;
            if (dst.layout == LG) {
                o.doff = dst.off[db] + dsub;
                o.ldd = dst.rows[db];
            } else {
                o.doff = dst.off[db] + int64_t(dsub) * lk.dim[il];
                o.ldd = lk.dim[il];
            }
            o.t0 = (int)cb.terms.size();
            o.nt = 1;
            CombTerm t;
            t.sbuf = S_X;
            t.coef = 1.0;
            if (src.layout == LG) {
                t.soff = src.off[b] + sub;
                t.lds = src.rows[b];
            } else {
                t.soff = src.off[b] + int64_t(sub) * lk.dim[il];
                t.lds = lk.dim[il];
            }
            cb.terms.push_back(t);
            cb.outs.push_back(o);
        }
    cb.finalize(ctx->stream);
    for (int pl = 0; pl < planes; ++pl) {  // the same block copies on each plane
        Bases bs{};
        bs.p[S_X] = const_cast<double*>(sp) + pl * src.size;
        bs.p[S_Y] = dp + pl * dst.size;
        launch_combine(cb, bs, ctx->stream);
    }
}

// phi = site p * site p+1 in the phi layout
void form_phi(tn_env* env, int p, const PhiLayout& ph, double* out) {
    tn_mps* psi = env->psi.get();
    const tn_site& X = psi->sites[p];
    const tn_site& Y = psi->sites[p + 1];
    const Link& mk = psi->links[p + 1];
    const Link& lk = psi->links[p];
    const int d = psi->d;
    GemmPlan g;
    for (int mi = 0; mi < ph.nblk(); ++mi) {
        const int im = mk.find(ph.m[mi]);
        if (X.lay.layout == RG && Y.lay.layout == RG) {
            for (int s1 = 0; s1 < d; ++s1) {
                const int rs = ph.rsub[size_t(mi) * d + s1];
                if (rs < 0) continue;
                const int il = ph.rsec[size_t(mi) * d + s1];
                g.add_task(S_Y, ph.off[mi] + rs, lk.dim[il], ph.cols[mi], ph.rows[mi]);
                if (im < 0) continue;
                const int sub = X.lay.sub[size_t(il) * d + s1];
                if (sub < 0) continue;
                TN_REQUIRE(Y.lay.cols[im] == ph.cols[mi], "phi column layout mismatch");
                g.add_seg(S_A, X.lay.off[il] + int64_t(sub) * lk.dim[il], lk.dim[il], 0, S_B,
                          Y.lay.off[im], mk.dim[im], 0, mk.dim[im]);
            }
        } else if (X.lay.layout == LG && Y.lay.layout == LG) {
            const Link& rk = psi->links[p + 2];
            for (int s2 = 0; s2 < d; ++s2) {
                const int cs = ph.csub[size_t(mi) * d + s2];
                if (cs < 0) continue;
                const int ir = ph.csec[size_t(mi) * d + s2];
                g.add_task(S_Y, ph.off[mi] + int64_t(cs) * ph.rows[mi], ph.rows[mi], rk.dim[ir],
                           ph.rows[mi]);
                if (im < 0) continue;
                const int sub = Y.lay.sub[size_t(ir) * d + s2];
                if (sub < 0) continue;
                TN_REQUIRE(X.lay.rows[im] == ph.rows[mi], "phi row layout mismatch");
                g.add_seg(S_A, X.lay.off[im], ph.rows[mi], 0, S_B, Y.lay.off[ir] + sub,
                          Y.lay.rows[ir], 0, mk.dim[im]);
            }
        } else if (X.lay.layout == LG && Y.lay.layout == RG) {
            g.add_task(S_Y, ph.off[mi], ph.rows[mi], ph.cols[mi], ph.rows[mi]);
            if (im < 0) continue;
            g.add_seg(S_A, X.lay.off[im], ph.rows[mi], 0, S_B, Y.lay.off[im], mk.dim[im], 0,
                      mk.dim[im]);
        } else {
            throw Error(TN_E_INVALID, "two-site tensor needs the orthogonality center on the bond");
        }
    }
    Bases bs{};
    bs.p[S_A] = X.buf.d();
    bs.p[S_B] = Y.buf.d();
    bs.p[S_Y] = out;
    if (psi->cplx) {
        set_im(bs, S_A, X.lay.size);
        set_im(bs, S_B, Y.lay.size);
        set_im(bs, S_Y, ph.size);
        GemmPlan c = complex_plan(g, 0);
        c.finalize(env->ctx->stream);
        launch_gemm_f64(c, bs, env->ctx->stream);
        return;
    }
    g.finalize(env->ctx->stream);
    launch_gemm_f64(g, bs, env->ctx->stream);
}

// -------------------------------------------------------------------------------------
// Lanczos (thick restart, full re-orthogonalisation), KrylovKit eigsolve semantics
// -------------------------------------------------------------------------------------
struct EigOut {
    double energy;
    int matvecs, converged;
};

template <class MV>
EigOut lanczos_lowest(tn_env* env, MV&& apply, int64_t n, double* x0, double* result,
                      const tn_update_params* prm) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    const int kd = prm->krylovdim;
    // vector pool: kd basis + kd restart + 1 residual
    const int nvec = 2 * kd + 1;
    env->kry.alloc(size_t(nvec) * size_t(std::max<int64_t>(n, 1)) * 8, st);
    env->part.alloc(size_t(32) * blas_nparts() * 8, st);
    env->dots.alloc(128 * 8, st);
    if (!env->ticket.p) {
        env->ticket.alloc(sizeof(unsigned), st);
        TN_CUDA(cudaMemsetAsync(env->ticket.p, 0, sizeof(unsigned), st));
    }
    unsigned* tk = env->ticket.as<unsigned>();
    std::vector<double*> pool;
    for (int i = 0; i < nvec; ++i) pool.push_back(env->kry.d() + int64_t(i) * n);
    double* dv = env->dots.d();
    std::vector<double*> V;
    double* w = pool.back();
    pool.pop_back();
    auto take = [&]() {
        TN_REQUIRE(!pool.empty(), "internal: Krylov vector pool exhausted");
        double* q = pool.back();
        pool.pop_back();
        return q;
    };
    EigOut out{0.0, 0, 0};
    std::vector<double> hostd(65);

    auto gs2 = [&](int K, std::vector<double>& h, double& beta) {
        // h = V^T w ; w -= V h ; twice ; beta = |w|
        const int e0 = ctx->timer.mark();
        launch_gs_pass(V.data(), K, w, nullptr, 0.0, n, true, false, env->part.d(), dv, tk, st);
        launch_gs_pass(V.data(), K, w, dv, -1.0, n, true, false, env->part.d(), dv + 32, tk, st);
        launch_gs_pass(V.data(), K, w, dv + 32, -1.0, n, false, true, env->part.d(), dv + 64, tk, st);
        ctx->timer.add(T_LANCZOS, e0, ctx->timer.mark());
        TN_CUDA(cudaMemcpyAsync(hostd.data(), dv, 65 * 8, cudaMemcpyDeviceToHost, st));
        sync(ctx);
        h.resize(K);
        for (int i = 0; i < K; ++i) h[i] = hostd[i] + hostd[32 + i];
        beta = std::sqrt(std::max(hostd[64], 0.0));
    };

    // normalise x0 into V[0]
    {
        const double* xp = x0;
        launch_multi_dot(&xp, 1, x0, n, env->part.d(), dv + 64, st);
        double nrm2 = 0;
        TN_CUDA(cudaMemcpyAsync(&nrm2, dv + 64, 8, cudaMemcpyDeviceToHost, st));
        sync(ctx);
        TN_REQUIRE(nrm2 > 0.0, "eigensolver start vector is zero");
        double* v0 = take();
        launch_scale_into(v0, x0, nullptr, 1.0 / std::sqrt(nrm2), n, st);
        V.push_back(v0);
    }
    std::vector<double> Hm(size_t(kd + 1) * (kd + 1), 0.0);
    auto Hat = [&](int i, int j) -> double& { return Hm[size_t(i) * (kd + 1) + j]; };
    std::vector<double> h;
    double beta = 0.0;
    apply(V[0], w);
    out.matvecs++;
    gs2(1, h, beta);
    Hat(0, 0) = h[0];
    int numiter = 1;
    std::vector<double> D, U;
    int converged = 0;
    while (true) {
        const int K = (int)V.size();
        // K >= n: the Krylov space spans the whole vector space, the Ritz pair is exact
        const bool exhausted = int64_t(K) >= n;
        if (K == kd || beta <= prm->tol || (prm->eager && K >= 1) || exhausted) {
            std::vector<double> A(size_t(K) * K);
            for (int i = 0; i < K; ++i)
                for (int j = 0; j < K; ++j) A[size_t(i) * K + j] = 0.5 * (Hat(i, j) + Hat(j, i));
            sym_eig(K, A, D, U);
            converged = 0;
            while (converged < K && std::fabs(beta * U[size_t(K - 1) * K + converged]) <= prm->tol)
                converged++;
            if (converged >= 1 || exhausted) break;
        }
        if (K < kd) {
            double* v = take();
            launch_scale_into(v, w, nullptr, 1.0 / beta, n, st);
            V.push_back(v);
            apply(v, w);
            out.matvecs++;
            gs2(K + 1, h, beta);
            for (int i = 0; i <= K; ++i) {
                Hat(i, K) = h[i];
                Hat(K, i) = h[i];
            }
        } else {
            if (numiter == prm->maxiter) break;
            const int keep = (3 * kd + 2 * converged) / 5;
            std::vector<double*> NV;
            for (int j = 0; j < keep; ++j) {
                double* q = take();
                std::vector<double> coef(K);
                for (int i = 0; i < K; ++i) coef[i] = U[size_t(i) * K + j];
                TN_CUDA(cudaMemcpyAsync(dv + 96, coef.data(), K * 8, cudaMemcpyHostToDevice, st));
                launch_lincomb(q, V.data(), K, dv + 96, n, st);
                sync(ctx);  // coef staging slot is reused
                NV.push_back(q);
            }
            for (double* q : V) pool.push_back(q);
            V = NV;
            std::fill(Hm.begin(), Hm.end(), 0.0);
            for (int j = 0; j < keep; ++j) Hat(j, j) = D[j];
            numiter++;
        }
    }
    // Ritz vector of the lowest value, normalised
    const int K = (int)V.size();
    std::vector<double> coef(K);
    for (int i = 0; i < K; ++i) coef[i] = U[size_t(i) * K + 0];
    TN_CUDA(cudaMemcpyAsync(dv + 96, coef.data(), K * 8, cudaMemcpyHostToDevice, st));
    launch_lincomb(result, V.data(), K, dv + 96, n, st);
    const double* rp = result;
    launch_multi_dot(&rp, 1, result, n, env->part.d(), dv + 64, st);
    launch_scale_into(result, result, dv + 64, 1.0, n, st);
    sync(ctx);
    out.energy = D[0];
    out.converged = converged;
    return out;
}

// -------------------------------------------------------------------------------------
// Krylov exponentiation exp(tau H_eff) x, tau = t + i ti (KrylovKit exponentiate semantics
// restated): eager Lanczos with full re-orthogonalisation; after each expansion
// y = exp(dt T) e1 and the step is accepted when |dt| * beta * |y[K-1]| <= tol (or
// beta <= tol, or the space is exhausted); a full Krylov space that misses the tolerance
// takes the largest dt = tau f / 2^j that meets it and restarts from the evolved vector for
// the remaining time.
//
// Complex vectors are planar (n = 2 nc reals: real parts, then imaginary parts).  For a
// Hermitian H_eff the Lanczos coefficients of the complex iteration are real and its basis
// vectors are those of the real iteration on the planar vectors (whose inner product is the
// real part of the complex one), so the same real kernels build T; only the final
// combination takes the complex y: x = sum_j Re(y_j) v_j + i sum_j Im(y_j) v_j.
// -------------------------------------------------------------------------------------
template <class MV>
int krylov_exp(tn_env* env, MV&& apply, int64_t n, double t, const double* x0, double* out,
               const tn_update_params* prm, double ti = 0.0, int64_t nc = 0) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    TN_REQUIRE(ti == 0.0 || 2 * nc == n, "internal: a complex time step needs complex vectors");
    const int kd = prm->krylovdim;
    const int nvec = kd + 2;  // basis + residual + current vector
    env->kry.alloc(size_t(nvec) * size_t(std::max<int64_t>(n, 1)) * 8, st);
    env->part.alloc(size_t(32) * blas_nparts() * 8, st);
    env->dots.alloc(256 * 8, st);
    if (!env->ticket.p) {
        env->ticket.alloc(sizeof(unsigned), st);
        TN_CUDA(cudaMemsetAsync(env->ticket.p, 0, sizeof(unsigned), st));
    }
    unsigned* tk = env->ticket.as<unsigned>();
    double* dv = env->dots.d();
    std::vector<double*> pool;
    for (int i = 0; i < nvec; ++i) pool.push_back(env->kry.d() + int64_t(i) * n);
    double* cur = pool.back();
    pool.pop_back();
    double* w = pool.back();
    pool.pop_back();
    TN_CUDA(cudaMemcpyAsync(cur, x0, size_t(n) * 8, cudaMemcpyDeviceToDevice, st));
    std::vector<double> hostd(65);
    int matvecs = 0;
    double rem = 1.0;  // fraction of tau still to go
    const double tabs = std::hypot(t, ti);
    if (ti != 0.0) {
        const double one = 1.0;
        TN_CUDA(cudaMemcpyAsync(dv + 224, &one, 8, cudaMemcpyHostToDevice, st));
    }
    auto norm2 = [&](double* v) {
        const double* vp = v;
        launch_gs_pass(&vp, 0, v, nullptr, 0.0, n, false, true, env->part.d(), dv + 64, tk, st);
        double r = 0;
        TN_CUDA(cudaMemcpyAsync(&r, dv + 64, 8, cudaMemcpyDeviceToHost, st));
        sync(ctx);
        return r;
    };
    for (int it = 0; it < prm->maxiter && rem != 0.0; ++it) {
        const double nrm = std::sqrt(std::max(norm2(cur), 0.0));
        if (nrm == 0.0) break;
        std::vector<double*> V;
        V.push_back(pool[0]);
        launch_scale_into(V[0], cur, nullptr, 1.0 / nrm, n, st);
        std::vector<double> Hm(size_t(kd + 1) * (kd + 1), 0.0);
        auto Hat = [&](int i, int j) -> double& { return Hm[size_t(i) * (kd + 1) + j]; };
        auto gs = [&](int K, std::vector<double>& h, double& beta) {
            const int e0 = ctx->timer.mark();
            launch_gs_pass(V.data(), K, w, nullptr, 0.0, n, true, false, env->part.d(), dv, tk, st);
            launch_gs_pass(V.data(), K, w, dv, -1.0, n, true, false, env->part.d(), dv + 32, tk, st);
            launch_gs_pass(V.data(), K, w, dv + 32, -1.0, n, false, true, env->part.d(), dv + 64, tk, st);
            ctx->timer.add(T_LANCZOS, e0, ctx->timer.mark());
            TN_CUDA(cudaMemcpyAsync(hostd.data(), dv, 65 * 8, cudaMemcpyDeviceToHost, st));
            sync(ctx);
            h.resize(K);
            for (int i = 0; i < K; ++i) h[i] = hostd[i] + hostd[32 + i];
            beta = std::sqrt(std::max(hostd[64], 0.0));
        };
        std::vector<double> h, D, U;
        double beta = 0.0;
        apply(V[0], w);
        matvecs++;
        gs(1, h, beta);
        Hat(0, 0) = h[0];
        double f = rem;  // this step: tau f
        while (true) {
            const int K = (int)V.size();
            std::vector<double> A(size_t(K) * K);
            for (int i = 0; i < K; ++i)
                for (int j = 0; j < K; ++j) A[size_t(i) * K + j] = 0.5 * (Hat(i, j) + Hat(j, i));
            sym_eig(K, A, D, U);
            // y = exp(tau f T) e1 = U exp(tau f D) U^T e1, real and imaginary parts
            auto expv = [&](double fr, std::vector<double>& yr, std::vector<double>& yi) {
                yr.assign(K, 0.0);
                yi.assign(K, 0.0);
                for (int j = 0; j < K; ++j) {
                    const double m = std::exp(fr * t * D[j]) * U[size_t(0) * K + j];
                    const double ph = fr * ti * D[j];
                    const double cr = ph == 0.0 ? m : m * std::cos(ph);
                    const double ci = ph == 0.0 ? 0.0 : m * std::sin(ph);
                    for (int i = 0; i < K; ++i) {
                        yr[i] += U[size_t(i) * K + j] * cr;
                        yi[i] += U[size_t(i) * K + j] * ci;
                    }
                }
            };
            std::vector<double> yr, yi;
            expv(f, yr, yi);
            double err = f * tabs * beta * std::hypot(yr[K - 1], yi[K - 1]);
            const bool exhausted = int64_t(K) >= (nc > 0 ? nc : n);  // the complex dimension
            bool accept = err <= prm->tol || beta <= prm->tol || exhausted;
            if (!accept && K == kd) {
                while (err > prm->tol && f * tabs > 1e-300) {
                    f *= 0.5;
                    expv(f, yr, yi);
                    err = f * tabs * beta * std::hypot(yr[K - 1], yi[K - 1]);
                }
                accept = true;
            }
            if (accept) {
                for (double& c : yr) c *= nrm;
                TN_CUDA(cudaMemcpyAsync(dv + 96, yr.data(), K * 8, cudaMemcpyHostToDevice, st));
                launch_lincomb(cur, V.data(), K, dv + 96, n, st);
                if (ti != 0.0) {
                    // cur += i (sum_j Im(y_j) v_j), through the residual buffer
                    for (double& c : yi) c *= nrm;
                    TN_CUDA(cudaMemcpyAsync(dv + 160, yi.data(), K * 8, cudaMemcpyHostToDevice, st));
                    launch_lincomb(w, V.data(), K, dv + 160, n, st);
                    const double* wim = w + nc;
                    const double* wre = w;
                    launch_multi_axpy(cur, &wim, 1, dv + 224, -1.0, nc, st);
                    launch_multi_axpy(cur + nc, &wre, 1, dv + 224, 1.0, nc, st);
                }
                sync(ctx);
                rem -= f;
                break;
            }
            double* v = pool[K];
            launch_scale_into(v, w, nullptr, 1.0 / beta, n, st);
            V.push_back(v);
            apply(v, w);
            matvecs++;
            gs(K + 1, h, beta);
            for (int i = 0; i <= K; ++i) {
                Hat(i, K) = h[i];
                Hat(K, i) = h[i];
            }
        }
    }
    TN_CUDA(cudaMemcpyAsync(out, cur, size_t(n) * 8, cudaMemcpyDeviceToDevice, st));
    return matvecs;
}

// normalise x in place (when asked) and return <x|H x> using y as scratch
template <class MV>
double normalize_and_energy(tn_env* env, MV&& apply, int64_t n, double* x, double* y,
                            bool normalize) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    unsigned* tk = env->ticket.as<unsigned>();
    double* dv = env->dots.d();
    const double* xp = x;
    if (normalize) {
        launch_gs_pass(&xp, 0, x, nullptr, 0.0, n, false, true, env->part.d(), dv + 64, tk, st);
        launch_scale_into(x, x, dv + 64, 1.0, n, st);
    }
    apply(x, y);
    launch_gs_pass(&xp, 1, y, nullptr, 0.0, n, true, false, env->part.d(), dv + 64, tk, st);
    double e = 0.0;
    TN_CUDA(cudaMemcpyAsync(&e, dv + 64, 8, cudaMemcpyDeviceToHost, st));
    sync(ctx);
    return e;
}

// -------------------------------------------------------------------------------------
// block SVD + truncation
// -------------------------------------------------------------------------------------
struct SvdResult {
    std::vector<SvdBlockDesc> desc;
    std::vector<double> S;  // sorted per block at desc.s_off
    int64_t total_n = 0;
};

// SVD of the listed blocks of src (device); results stay in the env work buffers.
// Thresholds the SVD tuner tries for a bond whose largest pipeline-eligible block falls in
// bucket k (32 (k - 1) < n <= 32 k, k <= 32): every block on the one-CTA kernel while n <= 256
// (beyond that its work matrices leave shared memory and it is known to lose), and the
// thresholds 64, 96, 128 and 176 below the bucket (the mid-size blocks ride along with the
// large ones in the cooperative launch).
std::vector<int> svd_candidates(int k) {
    const int lo = 32 * (k - 1) + 1, hi = 32 * k;
    std::vector<int> c;
    if (hi <= 256) c.push_back(INT_MAX);
    for (int t : {64, 96, 128, 176})
        if (t < lo) c.push_back(t);
    if (c.empty()) c.push_back(INT_MAX);
    return c;
}

void block_svd(tn_ctx* ctx, DevBuf& dX, DevBuf& dW, DevBuf& dV, DevBuf& dP, DevBuf& dS,
               DevBuf& dPerm, DevBuf& ddesc, const std::vector<int>& rows,
               const std::vector<int>& cols, const std::vector<int64_t>& offs, const double* src,
               SvdResult& R) {
    cudaStream_t st = ctx->stream;
    R.desc.clear();
    int64_t xo = 0, vo = 0, so = 0;
    int maxn = 1;
    for (size_t b = 0; b < rows.size(); ++b) {
        SvdBlockDesc d{};
        d.src_off = offs[b];
        d.rows = rows[b];
        d.cols = cols[b];
        d.trans = rows[b] < cols[b] ? 1 : 0;
        d.m = std::max(rows[b], cols[b]);
        d.n = std::min(rows[b], cols[b]);
        d.x_off = xo;
        d.v_off = vo;
        d.s_off = so;
        xo += int64_t(d.m) * d.n;
        vo += int64_t(d.n) * d.n;
        so += d.n;
        maxn = std::max(maxn, d.n);
        R.desc.push_back(d);
    }
    R.total_n = so;
    dX.alloc(size_t(std::max<int64_t>(xo, 1)) * 8, st);
    dW.alloc(size_t(std::max<int64_t>(xo, 1)) * 8, st);
    dV.alloc(size_t(std::max<int64_t>(vo, 1)) * 8, st);
    dP.alloc(size_t(std::max<int64_t>(vo, 1)) * 8, st);
    dS.alloc(size_t(std::max<int64_t>(so, 1)) * 8, st);
    dPerm.alloc(size_t(std::max<int64_t>(so, 1)) * 4, st);
    // blocks with more than `thr` columns (after orienting m >= n) go to the multi-SM
    // pipeline, the others to the one-CTA-per-block kernel; thr is the context's fixed
    // threshold, or the tuned one of this bond's block-size histogram
    auto eligible = [](const SvdBlockDesc& d) {
        return d.n <= bsvd_max_n() && bsvd_panel_width(d.m) > 0;
    };
    int thr = ctx->svd_big_n;
    SvdTuner::Entry* te = nullptr;
    int ci = -1;
    if (thr < 0) {
        int nmax_e = 0;
        for (const auto& d : R.desc)
            if (eligible(d)) nmax_e = std::max(nmax_e, d.n);
        SvdTuner::Entry& e = ctx->svd_tune.table[std::min((nmax_e + 31) / 32, 32)];
        if (e.cand.empty()) {
            e.cand = svd_candidates(std::min((nmax_e + 31) / 32, 32));
            e.ms.assign(e.cand.size(), -1.f);
            if (e.cand.size() == 1) e.best = 0;
        }
        ci = e.best >= 0 ? e.best : e.next;
        thr = e.cand[size_t(ci)];
        if (e.best < 0) te = &e;
    }
    std::vector<SvdBlockDesc> small, big;
    int maxn_small = 1;
    for (const auto& d : R.desc) {
        if (d.n > thr && eligible(d)) {
            big.push_back(d);
        } else {
            small.push_back(d);
            maxn_small = std::max(maxn_small, d.n);
        }
    }
    if (te) {
        if (!ctx->svd_tune.a) {
            TN_CUDA(cudaEventCreate(&ctx->svd_tune.a));
            TN_CUDA(cudaEventCreate(&ctx->svd_tune.b));
        }
        TN_CUDA(cudaEventRecord(ctx->svd_tune.a, st));
    }
    const int nsm_blocks = (int)small.size();
    ddesc.alloc(std::max<size_t>(size_t(nsm_blocks) * sizeof(SvdBlockDesc), 16), st);
    if (nsm_blocks)
        TN_CUDA(cudaMemcpyAsync(ddesc.p, small.data(), nsm_blocks * sizeof(SvdBlockDesc),
                                cudaMemcpyHostToDevice, st));
    static const bool dbg = std::getenv("TENNET_DEBUG_SVD") != nullptr;
    // sweep counts of the one-CTA blocks (work accounting) and their phase clocks
    DevBuf& dsw = ctx->svd_counts;
    const size_t clk_off = size_t((nsm_blocks + 1) & ~1) * 4;  // 8-byte aligned clock area
    dsw.alloc(clk_off + size_t(std::max(nsm_blocks, 1)) * 8 * 8, st);
    const int e0 = ctx->timer.mark();
    launch_svd_jacobi(ddesc.as<SvdBlockDesc>(), nsm_blocks, maxn_small, src, dX.d(), dW.d(),
                      dV.d(), dP.d(), dS.d(), dPerm.as<int>(), dsw.as<int>(), st);
    BsvdStats bst;
    big_block_svd(ctx, ctx->bsvd, big, src, dW.d(), dV.d(), dS.d(), dPerm.as<int>(), &bst);
    ctx->timer.add(T_SVD, e0, ctx->timer.mark());
    ctx->svd_stats.gemm_flops += bst.gemm_flops;
    ctx->svd_stats.jacobi_flops += bst.jacobi_flops;
    ctx->svd_stats.sweeps32 = std::max(ctx->svd_stats.sweeps32, bst.sweeps32);
    ctx->svd_stats.sweeps_df = std::max(ctx->svd_stats.sweeps_df, bst.sweeps_df);
    std::vector<int> sw(size_t(std::max(nsm_blocks, 1)));
    if (nsm_blocks)
        TN_CUDA(cudaMemcpyAsync(sw.data(), dsw.p, nsm_blocks * 4, cudaMemcpyDeviceToHost, st));
    if (dbg && nsm_blocks) {
        std::vector<long long> ck(size_t(nsm_blocks) * 8);
        TN_CUDA(cudaMemcpyAsync(ck.data(), static_cast<char*>(dsw.p) + clk_off, ck.size() * 8,
                                cudaMemcpyDeviceToHost, st));
        TN_CUDA(cudaStreamSynchronize(st));
        for (int b = 0; b < nsm_blocks; ++b) {
            const long long* c = &ck[size_t(b) * 8];
            std::fprintf(stderr,
                         "svd block %d: %dx%d sweeps fp32=%d fp64=%d kcycles qr=%lld fp32=%lld "
                         "gs=%lld y=%lld polish=%lld norms=%lld qv=%lld\n",
                         b, small[b].m, small[b].n, sw[b] >> 16, sw[b] & 0xffff, (c[1] - c[0]) / 1000,
                         (c[2] - c[1]) / 1000, (c[3] - c[2]) / 1000, (c[4] - c[3]) / 1000,
                         (c[5] - c[4]) / 1000, (c[6] - c[5]) / 1000, (c[7] - c[6]) / 1000);
        }
    }
    if (dbg && !big.empty()) {
        int mx = 0;
        for (const auto& d : big) mx = std::max(mx, d.n);
        std::fprintf(stderr, "svd big blocks: %d (largest n %d) sweeps fp32=%d df=%d\n",
                     (int)big.size(), mx, bst.sweeps32, bst.sweeps_df);
    }
    if (te) TN_CUDA(cudaEventRecord(ctx->svd_tune.b, st));
    R.S.resize(size_t(so));
    if (so)
        TN_CUDA(cudaMemcpyAsync(R.S.data(), dS.p, size_t(so) * 8, cudaMemcpyDeviceToHost, st));
    sync(ctx);
    // algorithmic flops of the one-CTA blocks: Householder QR 2mn^2 - 2n^3/3, per Jacobi
    // sweep 9 n^2 (n - 1) (18 n per rotated pair), Gram-Schmidt 2n^3, R^T V n^3, Q V
    // 4mn^2 - 2n^3
    for (int b = 0; b < nsm_blocks; ++b) {
        const double m = small[size_t(b)].m, n = small[size_t(b)].n;
        const double sweeps = double(sw[size_t(b)] >> 16) + double(sw[size_t(b)] & 0xffff);
        ctx->svd_stats.small_flops += 2 * m * n * n - 2 * n * n * n / 3 + sweeps * 9 * n * n * (n - 1) +
                                      3 * n * n * n + 4 * m * n * n - 2 * n * n * n;
    }
    if (!big.empty()) check_device_error(ctx);
    if (te) {
        float ms = 0.f;
        TN_CUDA(cudaEventElapsedTime(&ms, ctx->svd_tune.a, ctx->svd_tune.b));
        te->ms[size_t(ci)] = ms;
        if (++te->next == int(te->cand.size()))
            te->best = int(std::min_element(te->ms.begin(), te->ms.end()) - te->ms.begin());
    }
}

struct TruncDecision {
    std::vector<int> kept;
    double truncerr = 0, norm = 1;
    std::vector<double> eigs;
};

TruncDecision decide(const SvdResult& R, int maxdim, int mindim, double cutoff) {
    std::vector<double> P;
    P.reserve(R.S.size());
    for (double s : R.S) P.push_back(s * s);
    std::sort(P.begin(), P.end(), std::greater<double>());
    TruncOut t = truncation_rule(P, maxdim, mindim, cutoff);
    TruncDecision D;
    D.truncerr = t.truncerr;
    D.kept.assign(R.desc.size(), 0);
    int total = 0;
    for (size_t b = 0; b < R.desc.size(); ++b) {
        const auto& d = R.desc[b];
        int k = 0;
        while (k < d.n && R.S[d.s_off + k] * R.S[d.s_off + k] > t.docut) ++k;
        D.kept[b] = k;
        total += k;
    }
    if (total == 0 && !R.desc.empty()) {
        // every value fell under the cut (fully degenerate spectrum at maxdim): keep the
        // largest so that the link never becomes empty.
        size_t best = 0;
        double bv = -1;
        for (size_t b = 0; b < R.desc.size(); ++b)
            if (R.desc[b].n > 0 && R.S[R.desc[b].s_off] > bv) {
                bv = R.S[R.desc[b].s_off];
                best = b;
            }
        D.kept[best] = 1;
    }
    double nrm2 = 0;
    for (size_t b = 0; b < R.desc.size(); ++b)
        for (int k = 0; k < D.kept[b]; ++k) {
            const double s = R.S[R.desc[b].s_off + k];
            nrm2 += s * s;
            D.eigs.push_back(s * s);
        }
    std::sort(D.eigs.begin(), D.eigs.end(), std::greater<double>());
    D.norm = std::sqrt(nrm2);
    return D;
}

// replacebond!: SVD of phi (phi layout ph, device), truncation, new site tensors p, p+1.
void replace_bond(tn_env* env, int p, const PhiLayout& ph, const double* phi,
                  const tn_update_params* prm, int ortho, tn_update_result* res,
                  std::vector<double>& eigs) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    tn_mps* psi = env->psi.get();
    SvdResult R;
    block_svd(ctx, env->svdX, env->svdW, env->svdV, env->svdP, env->svdS, env->svdPerm,
              env->desc, ph.rows, ph.cols, ph.off, phi, R);
    TruncDecision D = decide(R, prm->maxdim, prm->mindim, prm->cutoff);
    Link nl;
    for (int b = 0; b < ph.nblk(); ++b)
        if (D.kept[b] > 0) {
            nl.q.push_back(ph.m[b]);
            nl.dim.push_back(D.kept[b]);
        }
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 2];
    tn_site left, right;
    left.lay = make_site_layout(LG, lk, nl, psi->pq);
    right.lay = make_site_layout(RG, nl, rk, psi->pq);
    left.buf.alloc(size_t(std::max<int64_t>(left.lay.size, 1)) * 8, st);
    right.buf.alloc(size_t(std::max<int64_t>(right.lay.size, 1)) * 8, st);
    std::vector<ExtractDesc> ed;
    for (int b = 0, j = 0; b < ph.nblk(); ++b) {
        if (D.kept[b] == 0) continue;
        TN_REQUIRE(left.lay.rows[j] == ph.rows[b] && right.lay.cols[j] == ph.cols[b],
                   "internal: SVD block layout mismatch");
        ExtractDesc e{};
        e.x_off = R.desc[b].x_off;
        e.v_off = R.desc[b].v_off;
        e.s_off = R.desc[b].s_off;
        e.left_off = left.lay.off[j];
        e.right_off = right.lay.off[j];
        e.rows = ph.rows[b];
        e.cols = ph.cols[b];
        e.n = R.desc[b].n;
        e.trans = R.desc[b].trans;
        e.k = D.kept[b];
        ed.push_back(e);
        ++j;
    }
    env->desc2.alloc(std::max<size_t>(ed.size() * sizeof(ExtractDesc), 16), st);
    if (!ed.empty())
        TN_CUDA(cudaMemcpyAsync(env->desc2.p, ed.data(), ed.size() * sizeof(ExtractDesc),
                                cudaMemcpyHostToDevice, st));
    const double inv = (prm->normalize && D.norm > 0) ? 1.0 / D.norm : 1.0;
    const int e0 = ctx->timer.mark();
    launch_svd_extract(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(),
                       env->svdV.d(), env->svdS.d(), env->svdPerm.as<int>(), left.buf.d(),
                       right.buf.d(), ortho, inv, st);
    ctx->timer.add(T_SVD, e0, ctx->timer.mark());
    psi->sites[p] = std::move(left);
    psi->sites[p + 1] = std::move(right);
    psi->links[p + 1] = nl;
    psi->center = (ortho == TN_ORTHO_LEFT) ? p + 1 : p;
    env->lpos = std::min(env->lpos, p);
    env->rpos = std::max(env->rpos, p + 1);
    env->hp_pos = -1;
    res->truncerr = D.truncerr;
    res->newdim = nl.total();
    eigs = D.eigs;
}

// Block SVD of complex blocks (planar source, imaginary plane at src + plane) with
// ITensors' truncation (complex svd + truncate!): each block A = Ar + i Ai (r x c) is
// factorised through the real SVD of [[Ar, -Ai], [Ai, Ar]] (2r x 2c), whose singular values
// are those of A, each twice; the columns of one pair span a complex singular vector
// [re; im] and i times it, so the first column of each pair is taken (by
// launch_svd_extract_complex).  Within a cluster of (nearly) equal complex values the taken
// columns are made complex-orthonormal on the host (the same combinations applied to the
// partner factor), which keeps A v = s u.  R holds the realified blocks' results, D the
// truncation of the complex values.
void complex_block_svd(tn_env* env, const std::vector<int>& rows, const std::vector<int>& cols,
                       const std::vector<int64_t>& offs, const double* src, int64_t plane,
                       const tn_update_params* prm, SvdResult& R, TruncDecision& D) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    const int nb = int(rows.size());
    std::vector<int> rows2(nb), cols2(nb);
    std::vector<int64_t> off2(nb);
    int64_t tot = 0;
    CombPlan rb;
    auto quad = [&](int64_t doff, int ldd, int r, int c, int sbuf, int64_t soff, double coef) {
        CombOut o{};
        o.doff = doff;
        o.dbuf = S_Y;
        o.ldd = ldd;
        o.rows = r;
        o.cols = c;
        o.t0 = int(rb.terms.size());
        o.nt = 1;
        rb.terms.push_back(CombTerm{soff, sbuf, r, coef});
        rb.outs.push_back(o);
    };
    for (int b = 0; b < nb; ++b) {
        const int r = rows[b], c = cols[b];
        rows2[b] = 2 * r;
        cols2[b] = 2 * c;
        off2[b] = tot;
        quad(tot, 2 * r, r, c, S_X, offs[b], 1.0);
        quad(tot + r, 2 * r, r, c, S_X + S_IM, offs[b], 1.0);
        quad(tot + int64_t(c) * 2 * r, 2 * r, r, c, S_X + S_IM, offs[b], -1.0);
        quad(tot + r + int64_t(c) * 2 * r, 2 * r, r, c, S_X, offs[b], 1.0);
        tot += int64_t(4) * r * c;
    }
    env->cx.alloc(size_t(std::max<int64_t>(tot, 1)) * 8, st);
    rb.finalize(st);
    {
        Bases bs{};
        bs.p[S_X] = const_cast<double*>(src);
        set_im(bs, S_X, plane);
        bs.p[S_Y] = env->cx.d();
        launch_combine(rb, bs, st);
    }
    block_svd(ctx, env->svdX, env->svdW, env->svdV, env->svdP, env->svdS, env->svdPerm,
              env->desc, rows2, cols2, off2, env->cx.d(), R);
    // the complex values: the first of each realified pair
    SvdResult C;
    C.desc = R.desc;
    for (int b = 0; b < nb; ++b) {
        C.desc[b].n = R.desc[b].n / 2;
        C.desc[b].s_off = int64_t(C.S.size());
        for (int j = 0; j < C.desc[b].n; ++j) C.S.push_back(R.S[size_t(R.desc[b].s_off + 2 * j)]);
    }
    C.total_n = int64_t(C.S.size());
    D = decide(C, prm->maxdim, prm->mindim, prm->cutoff);
    // clusters of kept values closer than 1e-8 of the block's largest: complex Gram-Schmidt
    std::vector<int> perm;
    for (int b = 0; b < nb; ++b) {
        const int k = D.kept[b];
        if (k < 2) continue;
        const double* sb = &C.S[size_t(C.desc[b].s_off)];
        for (int j0 = 0; j0 < k;) {
            int j1 = j0;
            while (j1 + 1 < k && sb[j1] - sb[j1 + 1] <= 1e-8 * sb[0]) ++j1;
            if (j1 > j0) {
                if (perm.empty()) {
                    perm.resize(size_t(R.total_n));
                    TN_CUDA(cudaMemcpyAsync(perm.data(), env->svdPerm.p, perm.size() * 4,
                                            cudaMemcpyDeviceToHost, st));
                    sync(ctx);
                }
                const SvdBlockDesc& d = R.desc[b];
                const int mq = d.m, np = d.n;  // lengths of the QV and PY columns
                const int hq = mq / 2, hp = np / 2;
                const int cnt = j1 - j0 + 1;
                std::vector<std::vector<double>> q, y;  // candidate columns
                for (int c = 2 * j0; c <= 2 * j1 + 1; ++c) {
                    const int pc = perm[size_t(d.s_off + c)];
                    std::vector<double> a(static_cast<size_t>(mq)), bcol(static_cast<size_t>(np));
                    TN_CUDA(cudaMemcpyAsync(a.data(), env->svdW.d() + d.x_off + int64_t(pc) * mq,
                                            size_t(mq) * 8, cudaMemcpyDeviceToHost, st));
                    TN_CUDA(cudaMemcpyAsync(bcol.data(), env->svdV.d() + d.v_off + int64_t(pc) * np,
                                            size_t(np) * 8, cudaMemcpyDeviceToHost, st));
                    q.push_back(std::move(a));
                    y.push_back(std::move(bcol));
                }
                sync(ctx);
                std::vector<std::vector<double>> qa, ya;  // accepted (complex-orthonormal)
                for (size_t c = 0; c < q.size() && int(qa.size()) < cnt; ++c) {
                    std::vector<double> x = q[c], z = y[c];
                    for (int pass = 0; pass < 2; ++pass)
                        for (size_t a = 0; a < qa.size(); ++a) {
                            // h = <qa, x> (complex), x -= h qa, z -= h ya
                            double hr = 0, hi = 0;
                            for (int i = 0; i < hq; ++i) {
                                hr += qa[a][i] * x[i] + qa[a][hq + i] * x[hq + i];
                                hi += qa[a][i] * x[hq + i] - qa[a][hq + i] * x[i];
                            }
                            for (int i = 0; i < hq; ++i) {
                                const double ar = qa[a][i], ai = qa[a][hq + i];
                                x[i] -= hr * ar - hi * ai;
                                x[hq + i] -= hr * ai + hi * ar;
                            }
                            for (int i = 0; i < hp; ++i) {
                                const double ar = ya[a][i], ai = ya[a][hp + i];
                                z[i] -= hr * ar - hi * ai;
                                z[hp + i] -= hr * ai + hi * ar;
                            }
                        }
                    double nx = 0;
                    for (double v : x) nx += v * v;
                    nx = std::sqrt(nx);
                    if (nx < 0.5) continue;  // (nearly) i times an accepted vector
                    for (double& v : x) v /= nx;
                    for (double& v : z) v /= nx;
                    qa.push_back(std::move(x));
                    ya.push_back(std::move(z));
                }
                TN_REQUIRE(int(qa.size()) == cnt, "complex SVD: degenerate cluster not resolved");
                for (int a = 0; a < cnt; ++a) {
                    const int pc = perm[size_t(d.s_off + 2 * (j0 + a))];
                    TN_CUDA(cudaMemcpyAsync(env->svdW.d() + d.x_off + int64_t(pc) * mq, qa[a].data(),
                                            size_t(mq) * 8, cudaMemcpyHostToDevice, st));
                    TN_CUDA(cudaMemcpyAsync(env->svdV.d() + d.v_off + int64_t(pc) * np, ya[a].data(),
                                            size_t(np) * 8, cudaMemcpyHostToDevice, st));
                }
                sync(ctx);  // host columns go out of scope
            }
            j0 = j1 + 1;
        }
    }
}

// replacebond! of a complex two-site tensor (planar phi): complex_block_svd of the phi
// blocks, U to the left tensor and S V^H to the right one (or U S and V^H), planar.
void replace_bond_complex(tn_env* env, int p, const PhiLayout& ph, const double* phi,
                          const tn_update_params* prm, int ortho, tn_update_result* res,
                          std::vector<double>& eigs) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    tn_mps* psi = env->psi.get();
    const int nb = ph.nblk();
    SvdResult R;
    TruncDecision D;
    complex_block_svd(env, ph.rows, ph.cols, ph.off, phi, ph.size, prm, R, D);
    Link nl;
    for (int b = 0; b < nb; ++b)
        if (D.kept[b] > 0) {
            nl.q.push_back(ph.m[b]);
            nl.dim.push_back(D.kept[b]);
        }
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 2];
    tn_site left, right;
    left.lay = make_site_layout(LG, lk, nl, psi->pq);
    right.lay = make_site_layout(RG, nl, rk, psi->pq);
    left.buf.alloc(size_t(std::max<int64_t>(left.lay.size, 1)) * 16, st);
    right.buf.alloc(size_t(std::max<int64_t>(right.lay.size, 1)) * 16, st);
    std::vector<ExtractDesc> ed;
    for (int b = 0, j = 0; b < nb; ++b) {
        if (D.kept[b] == 0) continue;
        TN_REQUIRE(left.lay.rows[j] == ph.rows[b] && right.lay.cols[j] == ph.cols[b],
                   "internal: SVD block layout mismatch");
        ExtractDesc e{};
        e.x_off = R.desc[b].x_off;
        e.v_off = R.desc[b].v_off;
        e.s_off = R.desc[b].s_off;
        e.left_off = left.lay.off[j];
        e.right_off = right.lay.off[j];
        e.rows = ph.rows[b];
        e.cols = ph.cols[b];
        e.n = R.desc[b].n;
        e.trans = R.desc[b].trans;
        e.k = D.kept[b];
        ed.push_back(e);
        ++j;
    }
    env->desc2.alloc(std::max<size_t>(ed.size() * sizeof(ExtractDesc), 16), st);
    if (!ed.empty())
        TN_CUDA(cudaMemcpyAsync(env->desc2.p, ed.data(), ed.size() * sizeof(ExtractDesc),
                                cudaMemcpyHostToDevice, st));
    const double inv = (prm->normalize && D.norm > 0) ? 1.0 / D.norm : 1.0;
    const int e0 = ctx->timer.mark();
    launch_svd_extract_complex(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(),
                               env->svdV.d(), env->svdS.d(), env->svdPerm.as<int>(), left.buf.d(),
                               left.lay.size, right.buf.d(), right.lay.size, ortho, inv, st);
    ctx->timer.add(T_SVD, e0, ctx->timer.mark());
    psi->sites[p] = std::move(left);
    psi->sites[p + 1] = std::move(right);
    psi->links[p + 1] = nl;
    psi->center = (ortho == TN_ORTHO_LEFT) ? p + 1 : p;
    env->lpos = std::min(env->lpos, p);
    env->rpos = std::max(env->rpos, p + 1);
    env->hp_pos = -1;
    res->truncerr = D.truncerr;
    res->newdim = nl.total();
    eigs = D.eigs;
}

// replacebond! with eigen_perturbation = noise * noiseterm(PH, phi, ortho) (called at
// TenNetLib src/mps/update_site.jl:59-76; ITensors factorize_eigen).  ortho "left": per charge
// m of the rows (l, s1) the density matrix rho = phi phi^T + noise N N^T with
// N[(l', s1'), (b, s2, r)] = sum L[l', a, l] W_p[a, b, s1', s1] phi[l, s1, s2, r] (the MPO
// link b between the two sites left open) is diagonalised; its eigenvectors are the left
// singular vectors of the augmented block [phi_m | sqrt(noise) N_m], its eigenvalues their
// S^2, so the block SVD of the augmented blocks gives both.  The kept vectors U form the
// left tensor, U^T phi the right one (normalised).  ortho "right" is the mirror image on the
// columns (s2', r') with N = phi W_{p+1} R and the row-augmented blocks [phi_m; sqrt(noise) N].
void replace_bond_noise(tn_env* env, int p, Heff2Plan& P, const double* phi,
                        const tn_update_params* prm, int ortho, tn_update_result* res,
                        std::vector<double>& eigs) {
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    tn_mps* psi = env->psi.get();
    const tn_mpo* H = env->H;
    const int d = psi->d;
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 2];
    const PhiLayout& ph = P.ph;
    const bool left = ortho == TN_ORTHO_LEFT;
    const double sq = std::sqrt(prm->noise);
    const int w0 = H->wd[p], w1 = H->wd[p + 1], w2 = H->wd[p + 2];
    const EnvLayout& Lin = env->L[p].lay;
    const EnvLayout& Rin = env->R[p + 1].lay;
    // every charge of the kept side, one sector each
    Link allm;
    {
        std::vector<int> cand;
        if (left)
            for (int l : lk.q)
                for (int s = 0; s < d; ++s) cand.push_back(l + psi->pq[s]);
        else
            for (int r : rk.q)
                for (int s = 0; s < d; ++s) cand.push_back(r - psi->pq[s]);
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        allm.q = cand;
        allm.dim.assign(cand.size(), 1);
    }
    const SiteLayout side = left ? make_site_layout(LG, lk, allm, psi->pq)
                                 : make_site_layout(RG, allm, rk, psi->pq);
    const int nm = allm.nsec();
    // pieces of each augmented block: the phi block itself, then (MPO state, phi block) pairs
    struct Piece { int b, mi; int64_t off; };  // off: column (left) / row (right) offset
    std::vector<std::vector<Piece>> pieces(nm);
    std::vector<int> phib(nm, -1);
    std::vector<int64_t> ext(nm, 0);  // augmented columns (left) / rows (right)
    for (int k = 0; k < nm; ++k) {
        phib[k] = ph.find(allm.q[k]);
        if (phib[k] >= 0) ext[k] = left ? ph.cols[phib[k]] : ph.rows[phib[k]];
    }
    const std::vector<int>& dmid = H->delta[p + 1];
    for (int mi = 0; mi < ph.nblk(); ++mi)
        for (int b = 0; b < w1; ++b) {
            const int k = allm.find(ph.m[mi] + dmid[b]);
            if (k < 0) continue;
            pieces[k].push_back(Piece{b, mi, ext[k]});
            ext[k] += left ? ph.cols[mi] : ph.rows[mi];
        }
    std::vector<int64_t> aoff(nm);
    std::vector<int> arows(nm), acols(nm);
    int64_t asize = 0;
    for (int k = 0; k < nm; ++k) {
        arows[k] = left ? side.rows[k] : int(ext[k]);
        acols[k] = left ? int(ext[k]) : side.cols[k];
        aoff[k] = asize;
        asize += int64_t(arows[k]) * acols[k];
    }
    DevBuf aug, tbuf;
    aug.alloc(size_t(std::max<int64_t>(asize, 1)) * 8, st);
    TN_CUDA(cudaMemsetAsync(aug.p, 0, size_t(std::max<int64_t>(asize, 1)) * 8, st));
    CombPlan cb;
    Bases bs{};
    bs.p[S_L] = env->L[p].buf.d();
    bs.p[S_R] = env->R[p + 1].buf.d();
    bs.p[S_X] = const_cast<double*>(phi);
    bs.p[S_Y] = aug.d();
    bs.p[S_T1] = env->t1.d();
    auto add_copy = [&](int k) {  // phi block into the augmented block
        const int pi = phib[k];
        if (pi < 0) return;
        CombOut o;
        o.doff = aoff[k];
        o.dbuf = S_Y;
        o.ldd = arows[k];
        o.rows = ph.rows[pi];
        o.cols = ph.cols[pi];
        o.t0 = (int)cb.terms.size();
        o.nt = 1;
        cb.terms.push_back(CombTerm{ph.off[pi], S_X, ph.rows[pi], 1.0});
        cb.outs.push_back(o);
    };
    if (left) {
        // Y(a, il, s1) = L(a, il) phi[slab (s1, l)]: stage 1 of the H_eff product
        if (ctx->prec == TN_PREC_SPLIT) {
            if (!P.s1) P.s1 = make_split(P.g1, ctx->slices, true, false, st);
            run_split(ctx, *P.s1, bs, nullptr, nullptr);
        } else {
            launch_gemm_f64(P.g1, bs, st);
        }
        for (int k = 0; k < nm; ++k) {
            add_copy(k);
            for (const Piece& pc : pieces[k])
                for (int s1p = 0; s1p < d; ++s1p) {
                    const int rs = side.sub[size_t(k) * d + s1p];
                    if (rs < 0) continue;
                    const int ilp = side.subsec[size_t(k) * d + s1p];
                    CombOut o;
                    o.doff = aoff[k] + rs + pc.off * arows[k];
                    o.dbuf = S_Y;
                    o.ldd = arows[k];
                    o.rows = lk.dim[ilp];
                    o.cols = ph.cols[pc.mi];
                    o.t0 = (int)cb.terms.size();
                    o.nt = 0;
                    for (int a = 0; a < w0; ++a) {
                        const int il = lk.find(lk.q[ilp] - H->delta[p][a]);
                        if (il < 0 || Lin.off[size_t(a) * Lin.nsec + il] < 0) continue;
                        if (Lin.bra[size_t(a) * Lin.nsec + il] != ilp) continue;
                        for (int s1 = 0; s1 < d; ++s1) {
                            const int64_t yo = P.yoff[(size_t(a) * lk.nsec() + il) * d + s1];
                            if (yo < 0 || ph.find(lk.q[il] + psi->pq[s1]) != pc.mi) continue;
                            const double w = H->at(p, a, pc.b, s1p, s1);
                            if (w == 0.0) continue;
                            cb.terms.push_back(CombTerm{yo, S_T1, lk.dim[ilp], sq * w});
                            o.nt++;
                        }
                    }
                    if (o.nt > 0) cb.outs.push_back(o);
                }
        }
    } else {
        // T(c, mi, s2) = phi_mi[:, slab (s2, r)] R(c, r)^T, then the combination over (c, s2)
        GemmPlan gt;
        std::vector<int64_t> toff(size_t(ph.nblk()) * d * w2, -1);
        int64_t t = 0;
        for (int mi = 0; mi < ph.nblk(); ++mi)
            for (int s2 = 0; s2 < d; ++s2) {
                const int cs = ph.csub[size_t(mi) * d + s2];
                if (cs < 0) continue;
                const int ir = ph.csec[size_t(mi) * d + s2];
                for (int c = 0; c < w2; ++c) {
                    const int64_t ro = Rin.off[size_t(c) * Rin.nsec + ir];
                    if (ro < 0 || !need_right(H, p + 1, c, s2)) continue;
                    const int Drp = rk.dim[Rin.bra[size_t(c) * Rin.nsec + ir]];
                    toff[(size_t(mi) * d + s2) * w2 + c] = t;
                    gt.add_task(S_T2, t, ph.rows[mi], Drp, ph.rows[mi]);
                    gt.add_seg(S_X, ph.off[mi] + int64_t(cs) * ph.rows[mi], ph.rows[mi], 0, S_R, ro,
                               Drp, 1, rk.dim[ir]);
                    t += int64_t(ph.rows[mi]) * Drp;
                }
            }
        tbuf.alloc(size_t(std::max<int64_t>(t, 1)) * 8, st);
        bs.p[S_T2] = tbuf.d();
        if (!gt.tasks.empty()) {
            if (ctx->prec != TN_PREC_SPLIT) gt.finalize(st);
            run_gemm(ctx, gt, bs);
        }
        for (int k = 0; k < nm; ++k) {
            add_copy(k);
            for (const Piece& pc : pieces[k])
                for (int s2p = 0; s2p < d; ++s2p) {
                    const int cs = side.sub[size_t(k) * d + s2p];
                    if (cs < 0) continue;
                    const int irp = side.subsec[size_t(k) * d + s2p];
                    CombOut o;
                    o.doff = aoff[k] + pc.off + int64_t(cs) * arows[k];
                    o.dbuf = S_Y;
                    o.ldd = arows[k];
                    o.rows = ph.rows[pc.mi];
                    o.cols = rk.dim[irp];
                    o.t0 = (int)cb.terms.size();
                    o.nt = 0;
                    for (int s2 = 0; s2 < d; ++s2) {
                        if (ph.csub[size_t(pc.mi) * d + s2] < 0) continue;
                        const int ir = ph.csec[size_t(pc.mi) * d + s2];
                        for (int c = 0; c < w2; ++c) {
                            const int64_t to = toff[(size_t(pc.mi) * d + s2) * w2 + c];
                            if (to < 0 || Rin.bra[size_t(c) * Rin.nsec + ir] != irp) continue;
                            const double w = H->at(p + 1, pc.b, c, s2p, s2);
                            if (w == 0.0) continue;
                            cb.terms.push_back(CombTerm{to, S_T2, ph.rows[pc.mi], sq * w});
                            o.nt++;
                        }
                    }
                    if (o.nt > 0) cb.outs.push_back(o);
                }
        }
    }
    cb.finalize(st);
    const int e0 = ctx->timer.mark();
    launch_combine(cb, bs, st);
    ctx->timer.add(T_SVD, e0, ctx->timer.mark());
    // block SVD of the nonempty augmented blocks
    std::vector<int> bidx, brow, bcol;
    std::vector<int64_t> boff;
    for (int k = 0; k < nm; ++k)
        if (arows[k] > 0 && acols[k] > 0) {
            bidx.push_back(k);
            brow.push_back(arows[k]);
            bcol.push_back(acols[k]);
            boff.push_back(aoff[k]);
        }
    SvdResult R;
    block_svd(ctx, env->svdX, env->svdW, env->svdV, env->svdP, env->svdS, env->svdPerm, env->desc,
              brow, bcol, boff, aug.d(), R);
    TruncDecision D = decide(R, prm->maxdim, prm->mindim, prm->cutoff);
    Link nl;
    std::vector<int> kb;  // block of the decision for each new sector
    for (size_t j = 0; j < bidx.size(); ++j)
        if (D.kept[j] > 0) {
            nl.q.push_back(allm.q[bidx[j]]);
            nl.dim.push_back(D.kept[j]);
            kb.push_back(int(j));
        }
    tn_site lsite, rsite;
    lsite.lay = make_site_layout(LG, lk, nl, psi->pq);
    rsite.lay = make_site_layout(RG, nl, rk, psi->pq);
    lsite.buf.alloc(size_t(std::max<int64_t>(lsite.lay.size, 1)) * 8, st);
    rsite.buf.alloc(size_t(std::max<int64_t>(rsite.lay.size, 1)) * 8, st);
    TN_CUDA(cudaMemsetAsync(lsite.buf.p, 0, size_t(std::max<int64_t>(lsite.lay.size, 1)) * 8, st));
    TN_CUDA(cudaMemsetAsync(rsite.buf.p, 0, size_t(std::max<int64_t>(rsite.lay.size, 1)) * 8, st));
    // the eigenvectors go to the kept side; the other factor of the SVD is not used
    std::vector<ExtractDesc> ed;
    int64_t dsize = 0;
    for (size_t j = 0; j < kb.size(); ++j) {
        const int b = kb[j];
        ExtractDesc e{};
        e.x_off = R.desc[b].x_off;
        e.v_off = R.desc[b].v_off;
        e.s_off = R.desc[b].s_off;
        e.rows = brow[b];
        e.cols = bcol[b];
        e.n = R.desc[b].n;
        e.trans = R.desc[b].trans;
        e.k = D.kept[b];
        if (left) {
            e.left_off = lsite.lay.off[j];
            e.right_off = dsize;
            dsize += int64_t(e.k) * e.cols;
        } else {
            e.left_off = dsize;
            e.right_off = rsite.lay.off[j];
            dsize += int64_t(e.rows) * e.k;
        }
        ed.push_back(e);
    }
    DevBuf dummy;
    dummy.alloc(size_t(std::max<int64_t>(dsize, 1)) * 8, st);
    env->desc2.alloc(std::max<size_t>(ed.size() * sizeof(ExtractDesc), 16), st);
    if (!ed.empty())
        TN_CUDA(cudaMemcpyAsync(env->desc2.p, ed.data(), ed.size() * sizeof(ExtractDesc),
                                cudaMemcpyHostToDevice, st));
    const int e1 = ctx->timer.mark();
    if (left)
        launch_svd_extract(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(), env->svdV.d(),
                           env->svdS.d(), env->svdPerm.as<int>(), lsite.buf.d(), dummy.d(),
                           TN_ORTHO_LEFT, 1.0, st);
    else
        launch_svd_extract(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(), env->svdV.d(),
                           env->svdS.d(), env->svdPerm.as<int>(), dummy.d(), rsite.buf.d(),
                           TN_ORTHO_RIGHT, 1.0, st);
    // the other tensor: U^T phi (left) or phi V (right), per sector with a phi block
    GemmPlan g;
    for (size_t j = 0; j < kb.size(); ++j) {
        const int pi = phib[bidx[kb[j]]];
        if (pi < 0) continue;
        const int k = nl.dim[j];
        if (left) {
            TN_REQUIRE(rsite.lay.cols[j] == ph.cols[pi], "internal: noise right layout");
            g.add_task(S_Y, rsite.lay.off[j], k, ph.cols[pi], k);
            g.add_seg(S_A, lsite.lay.off[j], lsite.lay.rows[j], 1, S_X, ph.off[pi], ph.rows[pi], 0,
                      ph.rows[pi]);
        } else {
            TN_REQUIRE(lsite.lay.rows[j] == ph.rows[pi], "internal: noise left layout");
            g.add_task(S_Y, lsite.lay.off[j], ph.rows[pi], k, ph.rows[pi]);
            g.add_seg(S_X, ph.off[pi], ph.rows[pi], 0, S_A, rsite.lay.off[j], k, 1, ph.cols[pi]);
        }
    }
    tn_site& kept_site = left ? lsite : rsite;
    tn_site& other = left ? rsite : lsite;
    if (!g.tasks.empty()) {
        g.finalize(st);
        Bases gb{};
        gb.p[S_X] = const_cast<double*>(phi);
        gb.p[S_A] = kept_site.buf.d();
        gb.p[S_Y] = other.buf.d();
        launch_gemm_f64(g, gb, st);
    }
    if (prm->normalize && other.lay.size > 0) {
        const double* op = other.buf.d();
        launch_multi_dot(&op, 1, op, other.lay.size, env->part.d(), env->dots.d() + 64, st);
        launch_scale_into(other.buf.d(), other.buf.d(), env->dots.d() + 64, 1.0, other.lay.size, st);
    }
    ctx->timer.add(T_SVD, e1, ctx->timer.mark());
    sync(ctx);  // the plans' buffers and the scratch are released after their launches
    psi->sites[p] = std::move(lsite);
    psi->sites[p + 1] = std::move(rsite);
    psi->links[p + 1] = nl;
    psi->center = left ? p + 1 : p;
    env->lpos = std::min(env->lpos, p);
    env->rpos = std::max(env->rpos, p + 1);
    env->hp_pos = -1;
    res->truncerr = D.truncerr;
    res->newdim = nl.total();
    eigs = D.eigs;
}

// halfsweep_done (TenNetLib src/mps/update_site.jl:13-23), 0-based, nsite = 2
bool halfsweep_done2(int N, int pos, int ortho) {
    return (pos == 0 && ortho == TN_ORTHO_RIGHT) || (pos == N - 2 && ortho == TN_ORTHO_LEFT);
}

// _update_two_site! (TenNetLib src/mps/update_site.jl:27-90).  time_step == nullptr: the
// eigensolver; otherwise the exponential solver with the reverse one-site step.
void update_two_site(tn_env* env, int p, int ortho, const tn_update_params* prm,
                     tn_update_result* res, std::vector<double>& eigs,
                     const double* time_step = nullptr, double time_im = 0.0) {
    check_params(prm);
    tn_mps* psi = env->psi.get();
    TN_REQUIRE(!psi->cplx || time_step,
               "complex states are evolved by tdvpsweep; the eigensolver takes real states");
    TN_REQUIRE(time_im == 0.0 || psi->cplx, "internal: a complex time step needs a complex state");
    TN_REQUIRE(p >= 0 && p < psi->N - 1, "bond position out of range");
    TN_REQUIRE((ortho == TN_ORTHO_LEFT && psi->center == p) ||
                   (ortho == TN_ORTHO_RIGHT && psi->center == p + 1),
               "orthogonality center must be at pos (ortho left) or pos+1 (ortho right)");
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    position(env, p, 2);
    Heff2Plan& P = heff_plan(env);
    const int64_t nph = P.ph.size;                 // complex dimension
    const int64_t n = nph * psi->planes();         // reals of one (planar) vector
    env->vecA.alloc(size_t(std::max<int64_t>(n, 1)) * 8, st);
    env->vecB.alloc(size_t(std::max<int64_t>(n, 1)) * 8, st);
    form_phi(env, p, P.ph, env->vecA.d());
    if (!env->proj.empty()) {
        TN_REQUIRE(!time_step, "excited-state projectors are built for the eigensolver only");
        proj_vectors2(env, p, P.ph);
    }
    auto apply2 = [&](const double* x, double* y) {
        heff_apply(env, P, x, y);
        proj_apply(env, x, y, n);
    };
    if (!time_step) {
        EigOut eo = lanczos_lowest(env, apply2, n, env->vecA.d(), env->vecB.d(), prm);
        if (prm->check_convergence && eo.converged < 1)
            throw Error(TN_E_NOTCONV, "`eig_solver()` not converged !!");
        res->energy = eo.energy;
        res->matvecs = eo.matvecs;
        res->converged = eo.converged;
    } else {
        const int64_t mv0 = env->matvecs;
        krylov_exp(env, apply2, n, *time_step, env->vecA.d(), env->vecB.d(), prm, time_im,
                   psi->cplx ? nph : 0);
        res->energy = normalize_and_energy(env, apply2, n, env->vecB.d(), env->vecA.d(),
                                           prm->normalize != 0);
        res->matvecs = int32_t(env->matvecs - mv0);
        res->converged = 1;
    }
    TN_REQUIRE(!(time_step && prm->noise > 1e-15),
               "`updatePosition()` :: `noise` cannot be greater than zero for `reverse_step=true` !!");
    if (std::fabs(prm->noise) > 1e-15)  // Float64_threshold(), src/mps/update_site.jl:60
        replace_bond_noise(env, p, P, env->vecB.d(), prm, ortho, res, eigs);
    else if (psi->cplx)
        replace_bond_complex(env, p, P.ph, env->vecB.d(), prm, ortho, res, eigs);
    else
        replace_bond(env, p, P.ph, env->vecB.d(), prm, ortho, res, eigs);
    res->neigs = (int)eigs.size();
    if (time_step && !halfsweep_done2(psi->N, p, ortho)) {
        // reverse step: evolve the new orthogonality center back by -time_step
        const int p1 = (ortho == TN_ORTHO_LEFT) ? p + 1 : p;
        position(env, p1, 1);
        Heff1Plan& P1 = heff1_plan(env);
        const int np = psi->planes();
        const int64_t n1c = P1.lay.size, n1 = n1c * np;
        env->vecC.alloc(size_t(std::max<int64_t>(n1, 1)) * 8, st);
        env->vecD.alloc(size_t(std::max<int64_t>(n1, 1)) * 8, st);
        tn_site& site = psi->sites[p1];
        const Link& lk = psi->links[p1];
        const Link& rk = psi->links[p1 + 1];
        if (site.lay.layout == RG)
            TN_CUDA(cudaMemcpyAsync(env->vecC.p, site.buf.p, size_t(n1) * 8,
                                    cudaMemcpyDeviceToDevice, st));
        else
            regroup(ctx, site.lay, site.buf.d(), P1.lay, env->vecC.d(), lk, rk, np);
        auto apply1 = [&](const double* x, double* y) { heff1_apply(env, P1, x, y); };
        const double back = -*time_step;
        const int64_t mv0 = env->matvecs;
        krylov_exp(env, apply1, n1, back, env->vecC.d(), env->vecD.d(), prm, -time_im,
                   psi->cplx ? n1c : 0);
        res->energy = normalize_and_energy(env, apply1, n1, env->vecD.d(), env->vecC.d(),
                                           prm->normalize != 0);
        res->matvecs += int32_t(env->matvecs - mv0);
        if (site.lay.layout == RG)
            TN_CUDA(cudaMemcpyAsync(site.buf.p, env->vecD.p, size_t(n1) * 8,
                                    cudaMemcpyDeviceToDevice, st));
        else
            regroup(ctx, P1.lay, env->vecD.d(), site.lay, site.buf.d(), lk, rk, np);
        env->lpos = std::min(env->lpos, p1);
        env->rpos = std::max(env->rpos, p1);
        env->hp_pos = -1;
    }
    if (ctx->prec == TN_PREC_SPLIT) check_device_error(ctx);
}

// halfsweep_done (TenNetLib src/mps/update_site.jl:13-23), 0-based, nsite = 1
bool halfsweep_done1(int N, int pos, int ortho) {
    return (pos == 0 && ortho == TN_ORTHO_RIGHT) || (pos == N - 1 && ortho == TN_ORTHO_LEFT);
}

// zero-site effective Hamiltonian (ProjMPO with nsite = 0, the reverse step of one-site
// TDVP) on a bond matrix C between the links Ll and Lr, one block C_j (Ll.dim[xs[j]] x
// Lr.dim[ys[j]], column-major at moff[j]) per charge: y = sum_a L(a) C R(a)^T with L the
// environment of the sites left of the bond and R that of the sites right of it.
struct Heff0Plan {
    GemmPlan g1, g2;
    int64_t tsize = 0;
};
void build_heff0(const tn_envt& EL, const tn_envt& ER, const Link& Ll, const Link& Lr,
                 const std::vector<int>& xs, const std::vector<int>& ys,
                 const std::vector<int64_t>& moff, Heff0Plan& P) {
    std::map<int, int> jof;  // charge -> block
    for (size_t j = 0; j < xs.size(); ++j) jof[Ll.q[xs[j]]] = int(j);
    const int w = EL.lay.w;
    TN_REQUIRE(w == ER.lay.w, "internal: zero-site environments on different MPO links");
    struct Pend {
        int64_t toff, roff;
        int Dy;
    };
    std::vector<std::vector<Pend>> per_out(xs.size());
    int64_t t = 0;
    for (size_t j = 0; j < xs.size(); ++j) {
        const int x = xs[j], y = ys[j];
        for (int a = 0; a < w; ++a) {
            const int64_t lo = EL.lay.off[size_t(a) * EL.lay.nsec + x];
            const int64_t ro = ER.lay.off[size_t(a) * ER.lay.nsec + y];
            if (lo < 0 || ro < 0) continue;
            const int xp = EL.lay.bra[size_t(a) * EL.lay.nsec + x];
            const int yp = ER.lay.bra[size_t(a) * ER.lay.nsec + y];
            auto it = jof.find(Ll.q[xp]);
            if (it == jof.end()) continue;
            const int jp = it->second;
            TN_REQUIRE(ys[size_t(jp)] == yp, "internal: zero-site charge mismatch");
            const int Dxp = Ll.dim[xp], Dx = Ll.dim[x], Dy = Lr.dim[y];
            // T = L(a, x) C_j  (Dxp x Dy)
            P.g1.add_task(S_T1, t, Dxp, Dy, Dxp);
            P.g1.add_seg(S_L, lo, Dxp, 0, S_X, moff[j], Dx, 0, Dx);
            per_out[size_t(jp)].push_back(Pend{t, ro, Dy});
            t += int64_t(Dxp) * Dy;
        }
    }
    for (size_t jp = 0; jp < xs.size(); ++jp) {
        const int Dxp = Ll.dim[xs[jp]], Dyp = Lr.dim[ys[jp]];
        // y_j' = sum T R(a, y)^T
        P.g2.add_task(S_Y, moff[jp], Dxp, Dyp, Dxp);
        for (const auto& e : per_out[jp]) P.g2.add_seg(S_T1, e.toff, Dxp, 0, S_R, e.roff, Dyp, 1, e.Dy);
    }
    P.tsize = t;
}

// _update_one_site! (TenNetLib src/mps/update_site.jl:94-190): solve the one-site problem
// at pos (time_step null: the eigensolver; else the exponential solver, exp(time_step H_eff),
// complex when time_im != 0); unless the half sweep is done, split the new tensor by the
// block SVD with ITensors truncation, keep U at pos (a left isometry for ortho "left", a
// right one for "right") and multiply S V (resp. U S) into the next site, after evolving
// that bond matrix back by -time_step with the zero-site H_eff (reverse_step).  With
// noise > 0 the new tensor times the next site goes through the two-site noise split.
void update_one_site(tn_env* env, int p, int ortho, const tn_update_params* prm,
                     tn_update_result* res, std::vector<double>& eigs,
                     const double* time_step = nullptr, double time_im = 0.0) {
    check_params(prm);
    tn_mps* psi = env->psi.get();
    const int N = psi->N;
    TN_REQUIRE(!psi->cplx || time_step,
               "complex states are evolved by tdvpsweep; the eigensolver takes real states");
    TN_REQUIRE(time_im == 0.0 || psi->cplx, "internal: a complex time step needs a complex state");
    TN_REQUIRE(!(time_step && prm->noise > 1e-15),
               "`updatePosition()` :: `noise` cannot be greater than zero for `reverse_step=true` !!");
    TN_REQUIRE(!time_step || env->proj.empty(),
               "excited-state projectors are built for the eigensolver only");
    TN_REQUIRE(p >= 0 && p < N, "site position out of range");
    TN_REQUIRE(psi->center == p, "one-site update: the orthogonality center must be at pos");
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    const int np = psi->planes();
    position(env, p, 1);
    Heff1Plan& P1 = heff1_plan(env);
    const int64_t n1c = P1.lay.size, n1 = n1c * np;
    env->vecC.alloc(size_t(std::max<int64_t>(n1, 1)) * 8, st);
    env->vecD.alloc(size_t(std::max<int64_t>(n1, 1)) * 8, st);
    tn_site& site = psi->sites[p];
    const Link lk = psi->links[p];
    const Link rk = psi->links[p + 1];
    if (site.lay.layout == RG)
        TN_CUDA(cudaMemcpyAsync(env->vecC.p, site.buf.p, size_t(n1) * 8, cudaMemcpyDeviceToDevice, st));
    else
        regroup(ctx, site.lay, site.buf.d(), P1.lay, env->vecC.d(), lk, rk, np);
    if (!env->proj.empty()) proj_vectors1(env, p, P1.lay);
    auto apply1 = [&](const double* x, double* y) {
        heff1_apply(env, P1, x, y);
        proj_apply(env, x, y, n1);
    };
    if (!time_step) {
        EigOut eo = lanczos_lowest(env, apply1, n1, env->vecC.d(), env->vecD.d(), prm);
        if (prm->check_convergence && eo.converged < 1)
            throw Error(TN_E_NOTCONV, "`eig_solver()` not converged !!");
        res->energy = eo.energy;
        res->matvecs = eo.matvecs;
        res->converged = eo.converged;
    } else {
        const int64_t mv0 = env->matvecs;
        krylov_exp(env, apply1, n1, *time_step, env->vecC.d(), env->vecD.d(), prm, time_im,
                   psi->cplx ? n1c : 0);
        res->energy = normalize_and_energy(env, apply1, n1, env->vecD.d(), env->vecC.d(),
                                           prm->normalize != 0);
        res->matvecs = int32_t(env->matvecs - mv0);
        res->converged = 1;
    }
    res->truncerr = 0.0;
    eigs.clear();
    // the solver's vector is normalised (normalize!(phi) is then the identity)
    if (halfsweep_done1(N, p, ortho)) {
        if (site.lay.layout == RG)
            TN_CUDA(cudaMemcpyAsync(site.buf.p, env->vecD.p, size_t(n1) * 8, cudaMemcpyDeviceToDevice, st));
        else
            regroup(ctx, P1.lay, env->vecD.d(), site.lay, site.buf.d(), lk, rk, np);
        env->lpos = std::min(env->lpos, p);
        env->rpos = std::max(env->rpos, p);
        env->h1p_pos = -1;
        env->hp_pos = -1;
        res->newdim = (ortho == TN_ORTHO_LEFT ? rk : lk).total();
        res->neigs = 0;
        if (ctx->prec == TN_PREC_SPLIT) check_device_error(ctx);
        return;
    }
    const bool left = ortho == TN_ORTHO_LEFT;
    if (prm->noise > 1e-15) {
        // src/mps/update_site.jl:135-152: the solved site times the next one is split as a
        // two-site tensor at pos0 with the density-matrix perturbation of that bond.  The
        // solved site is stored in a grouping the two-site former accepts next to its
        // neighbour (every pair but right-grouped left of left-grouped).
        const int p0 = left ? p : p - 1;
        const Layout nbr = psi->sites[left ? p + 1 : p - 1].lay.layout;
        const Layout want = left ? (nbr == LG ? LG : site.lay.layout)
                                 : (nbr == RG ? RG : site.lay.layout);
        if (want != site.lay.layout) {
            site.lay = make_site_layout(want, lk, rk, psi->pq);
            site.buf.alloc(size_t(std::max<int64_t>(site.lay.size, 1)) * 8, st);
        }
        if (site.lay.layout == RG)
            TN_CUDA(cudaMemcpyAsync(site.buf.p, env->vecD.p, size_t(n1) * 8, cudaMemcpyDeviceToDevice, st));
        else
            regroup(ctx, P1.lay, env->vecD.d(), site.lay, site.buf.d(), lk, rk);
        env->h1p_pos = -1;
        position(env, p0, 2);
        Heff2Plan& P = heff_plan(env);
        const int64_t n2 = P.ph.size;
        env->vecA.alloc(size_t(std::max<int64_t>(n2, 1)) * 8, st);
        form_phi(env, p0, P.ph, env->vecA.d());
        replace_bond_noise(env, p0, P, env->vecA.d(), prm, ortho, res, eigs);
        res->neigs = int(eigs.size());
        if (ctx->prec == TN_PREC_SPLIT) check_device_error(ctx);
        return;
    }
    // SVD blocks: per right sector (LG grouping) for "left", per left sector (RG) for "right"
    SiteLayout sv_lay = left ? make_site_layout(LG, lk, rk, psi->pq) : P1.lay;
    const double* phi = env->vecD.d();
    if (left) {
        regroup(ctx, P1.lay, env->vecD.d(), sv_lay, env->vecC.d(), lk, rk, np);
        phi = env->vecC.d();
    }
    SvdResult R;
    TruncDecision D;
    if (psi->cplx) {
        complex_block_svd(env, sv_lay.rows, sv_lay.cols, sv_lay.off, phi, sv_lay.size, prm, R, D);
    } else {
        block_svd(ctx, env->svdX, env->svdW, env->svdV, env->svdP, env->svdS, env->svdPerm,
                  env->desc, sv_lay.rows, sv_lay.cols, sv_lay.off, phi, R);
        D = decide(R, prm->maxdim, prm->mindim, prm->cutoff);
    }
    const Link& olink = left ? rk : lk;  // the link that is truncated
    Link nl;
    std::vector<int> osec;  // sector of the old link of each kept block
    for (int b = 0; b < sv_lay.nblk(); ++b)
        if (D.kept[b] > 0) {
            const int sec = b;  // LG blocks follow the right link's sectors, RG the left's
            nl.q.push_back(olink.q[sec]);
            nl.dim.push_back(D.kept[b]);
            osec.push_back(sec);
        }
    tn_site here;
    here.lay = left ? make_site_layout(LG, lk, nl, psi->pq) : make_site_layout(RG, nl, rk, psi->pq);
    here.buf.alloc(size_t(std::max<int64_t>(here.lay.size, 1)) * 8 * np, st);
    // bond matrix per kept sector: S V^T (k x D) for "left", U S (D x k) for "right"
    std::vector<int64_t> moff;
    int64_t msize = 0;
    for (size_t j = 0; j < osec.size(); ++j) {
        moff.push_back(msize);
        msize += int64_t(nl.dim[j]) * olink.dim[osec[j]];
    }
    env->t1.alloc(size_t(std::max<int64_t>(msize, 1)) * 8 * np, st);
    std::vector<ExtractDesc> ed;
    for (int b = 0, j = 0; b < sv_lay.nblk(); ++b) {
        if (D.kept[b] == 0) continue;
        ExtractDesc e{};
        e.x_off = R.desc[b].x_off;
        e.v_off = R.desc[b].v_off;
        e.s_off = R.desc[b].s_off;
        e.rows = sv_lay.rows[b];
        e.cols = sv_lay.cols[b];
        e.n = R.desc[b].n;
        e.trans = R.desc[b].trans;
        e.k = D.kept[b];
        if (left) {
            TN_REQUIRE(here.lay.rows[j] == sv_lay.rows[b], "internal: one-site SVD layout mismatch");
            e.left_off = here.lay.off[j];
            e.right_off = moff[j];
        } else {
            TN_REQUIRE(here.lay.cols[j] == sv_lay.cols[b], "internal: one-site SVD layout mismatch");
            e.left_off = moff[j];
            e.right_off = here.lay.off[j];
        }
        ed.push_back(e);
        ++j;
    }
    env->desc2.alloc(std::max<size_t>(ed.size() * sizeof(ExtractDesc), 16), st);
    TN_CUDA(cudaMemcpyAsync(env->desc2.p, ed.data(), ed.size() * sizeof(ExtractDesc),
                            cudaMemcpyHostToDevice, st));
    const double inv = (prm->normalize && D.norm > 0) ? 1.0 / D.norm : 1.0;
    const int e0 = ctx->timer.mark();
    // "left": U stays (ortho 0), S V^T to the bond matrix; "right": V^T stays (ortho 1)
    if (psi->cplx && left)
        launch_svd_extract_complex(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(),
                                   env->svdV.d(), env->svdS.d(), env->svdPerm.as<int>(),
                                   here.buf.d(), here.lay.size, env->t1.d(), msize, TN_ORTHO_LEFT,
                                   inv, st);
    else if (psi->cplx)
        launch_svd_extract_complex(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(),
                                   env->svdV.d(), env->svdS.d(), env->svdPerm.as<int>(),
                                   env->t1.d(), msize, here.buf.d(), here.lay.size,
                                   TN_ORTHO_RIGHT, inv, st);
    else if (left)
        launch_svd_extract(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(), env->svdV.d(),
                           env->svdS.d(), env->svdPerm.as<int>(), here.buf.d(), env->t1.d(),
                           TN_ORTHO_LEFT, inv, st);
    else
        launch_svd_extract(env->desc2.as<ExtractDesc>(), (int)ed.size(), env->svdW.d(), env->svdV.d(),
                           env->svdS.d(), env->svdPerm.as<int>(), env->t1.d(), here.buf.d(),
                           TN_ORTHO_RIGHT, inv, st);
    ctx->timer.add(T_SVD, e0, ctx->timer.mark());
    if (time_step) {
        // reverse step (update_site.jl:175-182): the bond matrix C between the new link and
        // the old one evolves by -time_step under the zero-site H_eff, whose left (right)
        // environment contains the new site for ortho "left" ("right")
        const int64_t n0 = msize * np;
        env->vecA.alloc(size_t(std::max<int64_t>(n0, 1)) * 8, st);
        env->vecB.alloc(size_t(std::max<int64_t>(n0, 1)) * 8, st);
        if (n0) TN_CUDA(cudaMemcpyAsync(env->vecA.p, env->t1.p, size_t(n0) * 8,
                                        cudaMemcpyDeviceToDevice, st));
        const int li = left ? p + 1 : p;
        std::swap(psi->sites[p], here);
        const Link saved = psi->links[li];
        psi->links[li] = nl;
        if (left) env_left_step(env, p);
        else env_right_step(env, p);
        const tn_envt& EL = left ? env->L[p + 1] : env->L[p];
        const tn_envt& ER = left ? env->R[p] : env->R[p - 1];
        std::vector<int> xs, ys;
        for (size_t j = 0; j < osec.size(); ++j) {
            xs.push_back(left ? int(j) : osec[j]);
            ys.push_back(left ? osec[j] : int(j));
        }
        Heff0Plan H0;
        build_heff0(EL, ER, left ? nl : olink, left ? olink : nl, xs, ys, moff, H0);
        GemmPlan c1, c2;
        if (psi->cplx) {
            c1 = complex_plan(H0.g1, 0);
            c2 = complex_plan(H0.g2, 0);
            c1.finalize(st);
            c2.finalize(st);
        } else {
            H0.g1.finalize(st);
            H0.g2.finalize(st);
        }
        env->cx.alloc(size_t(std::max<int64_t>(H0.tsize, 1)) * 8 * np, st);
        auto apply0 = [&](const double* x, double* y) {
            Bases bs{};
            bs.p[S_L] = EL.buf.d();
            bs.p[S_R] = ER.buf.d();
            bs.p[S_X] = const_cast<double*>(x);
            bs.p[S_Y] = y;
            bs.p[S_T1] = env->cx.d();
            const int h0 = ctx->timer.mark();
            if (psi->cplx) {
                set_im(bs, S_L, EL.lay.size);
                set_im(bs, S_R, ER.lay.size);
                set_im(bs, S_X, msize);
                set_im(bs, S_Y, msize);
                set_im(bs, S_T1, H0.tsize);
                launch_gemm_f64(c1, bs, st);
                launch_gemm_f64(c2, bs, st);
            } else {
                launch_gemm_f64(H0.g1, bs, st);
                launch_gemm_f64(H0.g2, bs, st);
            }
            ctx->timer.add(T_HEFF, h0, ctx->timer.mark());
            env->matvecs++;
        };
        const int64_t mv0 = env->matvecs;
        krylov_exp(env, apply0, n0, -*time_step, env->vecA.d(), env->vecB.d(), prm, -time_im,
                   psi->cplx ? msize : 0);
        res->energy = normalize_and_energy(env, apply0, n0, env->vecB.d(), env->vecA.d(),
                                           prm->normalize != 0);
        res->matvecs += int32_t(env->matvecs - mv0);
        env->t1.alloc(size_t(std::max<int64_t>(msize, 1)) * 8 * np, st);
        if (n0) TN_CUDA(cudaMemcpyAsync(env->t1.p, env->vecB.p, size_t(n0) * 8,
                                        cudaMemcpyDeviceToDevice, st));
        std::swap(psi->sites[p], here);
        psi->links[li] = saved;
        sync(ctx);  // the zero-site plans go out of scope
    }
    // next site: RG (blocks per left sector) for "left", LG (per right sector) for "right"
    const int q = left ? p + 1 : p - 1;
    tn_site& nxt = psi->sites[q];
    const Link& qa = psi->links[q];
    const Link& qb = psi->links[q + 1];
    SiteLayout nlay_old = make_site_layout(left ? RG : LG, qa, qb, psi->pq);
    DevBuf oldbuf;
    const double* oldp = nxt.buf.d();
    if (nxt.lay.layout != nlay_old.layout) {
        oldbuf.alloc(size_t(std::max<int64_t>(nlay_old.size, 1)) * 8 * np, st);
        regroup(ctx, nxt.lay, nxt.buf.d(), nlay_old, oldbuf.d(), qa, qb, np);
        oldp = oldbuf.d();
    }
    tn_site nnew;
    nnew.lay = left ? make_site_layout(RG, nl, qb, psi->pq) : make_site_layout(LG, qa, nl, psi->pq);
    nnew.buf.alloc(size_t(std::max<int64_t>(nnew.lay.size, 1)) * 8 * np, st);
    GemmPlan g;
    for (size_t j = 0; j < osec.size(); ++j) {
        const int sec = osec[j], k = nl.dim[j], D0 = olink.dim[sec];
        if (left) {
            // new (k x cols) = M (k x D0) * old (D0 x cols)
            const int cols = nlay_old.cols[sec];
            if (cols == 0) continue;
            g.add_task(S_Y, nnew.lay.off[j], k, cols, k);
            g.add_seg(S_X, moff[j], k, 0, S_A, nlay_old.off[sec], D0, 0, D0);
        } else {
            // new (rows x k) = old (rows x D0) * M (D0 x k)
            const int rows = nlay_old.rows[sec];
            if (rows == 0) continue;
            g.add_task(S_Y, nnew.lay.off[j], rows, k, rows);
            g.add_seg(S_A, nlay_old.off[sec], rows, 0, S_X, moff[j], D0, 0, D0);
        }
    }
    GemmPlan gc;
    if (!g.tasks.empty()) {
        Bases bs{};
        bs.p[S_X] = env->t1.d();
        bs.p[S_A] = const_cast<double*>(oldp);
        bs.p[S_Y] = nnew.buf.d();
        const int e1 = ctx->timer.mark();
        if (psi->cplx) {
            set_im(bs, S_X, msize);
            set_im(bs, S_A, nlay_old.size);
            set_im(bs, S_Y, nnew.lay.size);
            gc = complex_plan(g, 0);
            gc.finalize(st);
            launch_gemm_f64(gc, bs, st);
        } else {
            g.finalize(st);
            launch_gemm_f64(g, bs, st);  // the small bond matrix is multiplied in FP64
        }
        ctx->timer.add(T_SVD, e1, ctx->timer.mark());
    }
    psi->sites[p] = std::move(here);
    psi->sites[q] = std::move(nnew);
    if (left)
        psi->links[p + 1] = nl;
    else
        psi->links[p] = nl;
    psi->center = q;
    env->lpos = std::min(env->lpos, std::min(p, q));
    env->rpos = std::max(env->rpos, std::max(p, q));
    env->hp_pos = -1;
    env->h1p_pos = -1;
    sync(ctx);  // oldbuf and the plan's buffers are released after the launches
    res->truncerr = D.truncerr;
    res->newdim = nl.total();
    eigs = D.eigs;
    res->neigs = (int)eigs.size();
    if (ctx->prec == TN_PREC_SPLIT) check_device_error(ctx);
}

std::unique_ptr<tn_mps> copy_mps(const tn_mps* src) {
    auto m = std::make_unique<tn_mps>();
    m->ctx = src->ctx;
    m->N = src->N;
    m->d = src->d;
    m->pq = src->pq;
    m->links = src->links;
    m->center = src->center;
    m->cplx = src->cplx;
    m->sites.resize(src->N);
    for (int i = 0; i < src->N; ++i) {
        m->sites[i].lay = src->sites[i].lay;
        const size_t nb = size_t(std::max<int64_t>(src->sites[i].lay.size, 1)) * 8 * src->planes();
        m->sites[i].buf.alloc(nb, src->ctx->stream);
        TN_CUDA(cudaMemcpyAsync(m->sites[i].buf.p, src->sites[i].buf.p, nb,
                                cudaMemcpyDeviceToDevice, src->ctx->stream));
    }
    return m;
}

// a complex copy of every site tensor in place (imaginary planes zero)
void mps_to_complex(tn_mps* m) {
    if (m->cplx) return;
    cudaStream_t st = m->ctx->stream;
    for (auto& S : m->sites) {
        const int64_t n = S.lay.size;
        DevBuf b;
        b.alloc(size_t(std::max<int64_t>(n, 1)) * 16, st);
        if (n) TN_CUDA(cudaMemcpyAsync(b.p, S.buf.p, size_t(n) * 8, cudaMemcpyDeviceToDevice, st));
        TN_CUDA(cudaMemsetAsync(b.d() + n, 0, size_t(std::max<int64_t>(n, 1)) * 8, st));
        S.buf = std::move(b);
    }
    m->cplx = true;
}

// a real environment made complex: the state and every environment tensor it holds
void env_to_complex(tn_env* e) {
    if (e->psi->cplx) return;
    TN_REQUIRE(e->proj.empty(), "complex states with excited-state projectors are not built");
    cudaStream_t st = e->ctx->stream;
    mps_to_complex(e->psi.get());
    for (auto* side : {&e->L, &e->R})
        for (auto& E : *side) {
            if (!E.buf.p) continue;
            const int64_t n = E.lay.size;
            DevBuf b;
            b.alloc(size_t(std::max<int64_t>(n, 1)) * 24, st);  // re, im = 0, -im = 0
            if (n) TN_CUDA(cudaMemcpyAsync(b.p, E.buf.p, size_t(n) * 8, cudaMemcpyDeviceToDevice, st));
            TN_CUDA(cudaMemsetAsync(b.d() + n, 0, size_t(std::max<int64_t>(n, 1)) * 16, st));
            E.buf = std::move(b);
        }
    e->hp.reset();
    e->h1p.reset();
    e->hp_pos = e->h1p_pos = -1;
    TN_CUDA(cudaStreamSynchronize(st));
}

// dense (Dl, d, Dr) column-major <-> site blocks
void site_from_dense(const SiteLayout& lay, const Link& lk, const Link& rk, int d,
                     const double* dense, std::vector<double>& blocks) {
    blocks.assign(size_t(lay.size), 0.0);
    const int Dl = lk.total();
    auto lo = lk.offsets(), ro = rk.offsets();
    std::vector<char> used(size_t(Dl) * d * rk.total(), 0);
    for (int b = 0; b < lay.nblk(); ++b)
        for (int s = 0; s < d; ++s) {
            const int sub = lay.sub[size_t(b) * d + s];
            if (sub < 0) continue;
            const int oth = lay.subsec[size_t(b) * d + s];
            const int il = (lay.layout == LG) ? oth : b;
            const int ir = (lay.layout == LG) ? b : oth;
            for (int r = 0; r < rk.dim[ir]; ++r)
                for (int l = 0; l < lk.dim[il]; ++l) {
                    const size_t di = size_t(lo[il] + l) + size_t(Dl) * (s + size_t(d) * (ro[ir] + r));
                    used[di] = 1;
                    size_t bi;
                    if (lay.layout == LG) bi = lay.off[b] + (sub + l) + size_t(lay.rows[b]) * r;
                    else bi = lay.off[b] + l + size_t(lay.rows[b]) * (sub + r);
                    blocks[bi] = dense[di];
                }
        }
    for (size_t i = 0; i < used.size(); ++i)
        if (!used[i] && std::fabs(dense[i]) > 1e-12)
            throw Error(TN_E_INVALID, "site tensor has weight outside its charge sectors");
}

void site_to_dense(const SiteLayout& lay, const Link& lk, const Link& rk, int d,
                   const std::vector<double>& blocks, double* dense) {
    const int Dl = lk.total();
    auto lo = lk.offsets(), ro = rk.offsets();
    std::fill(dense, dense + size_t(Dl) * d * rk.total(), 0.0);
    for (int b = 0; b < lay.nblk(); ++b)
        for (int s = 0; s < d; ++s) {
            const int sub = lay.sub[size_t(b) * d + s];
            if (sub < 0) continue;
            const int oth = lay.subsec[size_t(b) * d + s];
            const int il = (lay.layout == LG) ? oth : b;
            const int ir = (lay.layout == LG) ? b : oth;
            for (int r = 0; r < rk.dim[ir]; ++r)
                for (int l = 0; l < lk.dim[il]; ++l) {
                    const size_t di = size_t(lo[il] + l) + size_t(Dl) * (s + size_t(d) * (ro[ir] + r));
                    size_t bi;
                    if (lay.layout == LG) bi = lay.off[b] + (sub + l) + size_t(lay.rows[b]) * r;
                    else bi = lay.off[b] + l + size_t(lay.rows[b]) * (sub + r);
                    dense[di] = blocks[bi];
                }
        }
}

// dense two-site (Dl, d, d, Dr) <-> phi layout
void phi_dense_map(const PhiLayout& ph, const Link& lk, const Link& rk, int d,
                   std::vector<int64_t>& map) {
    // map[block element] = dense index
    map.assign(size_t(ph.size), -1);
    const int Dl = lk.total();
    auto lo = lk.offsets(), ro = rk.offsets();
    for (int b = 0; b < ph.nblk(); ++b)
        for (int s1 = 0; s1 < d; ++s1) {
            const int rs = ph.rsub[size_t(b) * d + s1];
            if (rs < 0) continue;
            const int il = ph.rsec[size_t(b) * d + s1];
            for (int s2 = 0; s2 < d; ++s2) {
                const int cs = ph.csub[size_t(b) * d + s2];
                if (cs < 0) continue;
                const int ir = ph.csec[size_t(b) * d + s2];
                for (int r = 0; r < rk.dim[ir]; ++r)
                    for (int l = 0; l < lk.dim[il]; ++l) {
                        const int64_t bi = ph.off[b] + (rs + l) + int64_t(ph.rows[b]) * (cs + r);
                        const int64_t di = int64_t(lo[il] + l) +
                                           int64_t(Dl) * (s1 + int64_t(d) * (s2 + int64_t(d) * (ro[ir] + r)));
                        map[bi] = di;
                    }
            }
        }
}

}  // namespace

void tn::set_last_error(const char* msg) { g_err = msg; }

// helpers shared with the tree tensor network sweep (ttn.cpp)
void tn::sym_eig_host(int n, const std::vector<double>& A, std::vector<double>& D,
                      std::vector<double>& U) {
    sym_eig(n, A, D, U);
}
std::unique_ptr<SplitPlan> tn::make_split_plan(const GemmPlan& g, int slices, cudaStream_t st,
                                               bool own_packs) {
    return make_split(g, slices, false, false, st, own_packs);
}
void tn::run_split_plan(tn_ctx* ctx, SplitPlan& sp, const Bases& bs) {
    sp.a_packed = sp.b_packed = false;
    run_split(ctx, sp, bs, nullptr, nullptr);
}
void tn::check_device_error_public(tn_ctx* ctx) { check_device_error(ctx); }
tn::SvdTuner::~SvdTuner() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
}

// SVD with ITensors truncation of one dense m x n matrix A on the device (the block SVD of
// replacebond! on a single block): U (m x k, ld m) and S V^T (k x n, ld k); returns k.
int tn::svd_truncate_dense(tn_ctx* ctx, const double* A, int m, int n, int maxdim, int mindim,
                           double cutoff, double* U, double* SVt, double* truncerr) {
    cudaStream_t st = ctx->stream;
    DevBuf dX, dW, dV, dP, dS, dPerm, ddesc, ded;
    SvdResult R;
    block_svd(ctx, dX, dW, dV, dP, dS, dPerm, ddesc, {m}, {n}, {0}, A, R);
    TruncDecision D = decide(R, maxdim, mindim, cutoff);
    const int k = D.kept[0];
    ExtractDesc e{};
    e.x_off = R.desc[0].x_off;
    e.v_off = R.desc[0].v_off;
    e.s_off = R.desc[0].s_off;
    e.left_off = 0;
    e.right_off = 0;
    e.rows = m;
    e.cols = n;
    e.n = R.desc[0].n;
    e.trans = R.desc[0].trans;
    e.k = k;
    ded.alloc(sizeof(ExtractDesc), st);
    TN_CUDA(cudaMemcpyAsync(ded.p, &e, sizeof(ExtractDesc), cudaMemcpyHostToDevice, st));
    launch_svd_extract(ded.as<ExtractDesc>(), 1, dW.d(), dV.d(), dS.d(), dPerm.as<int>(), U, SVt,
                       TN_ORTHO_LEFT, 1.0, st);
    TN_CUDA(cudaStreamSynchronize(st));
    if (truncerr) *truncerr = D.truncerr;
    return k;
}

// -------------------------------------------------------------------------------------
// EventTimer
// -------------------------------------------------------------------------------------
namespace tn {
int EventTimer::mark() {
    if (used == pool.size()) {
        cudaEvent_t e;
        TN_CUDA(cudaEventCreate(&e));
        pool.push_back(e);
    }
    TN_CUDA(cudaEventRecord(pool[used], s));
    return int(used++);
}
void EventTimer::collect(double* acc) {
    for (const auto& iv : ivs) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, pool[iv.a], pool[iv.b]) == cudaSuccess) acc[iv.cat] += ms;
    }
    ivs.clear();
    used = 0;
}
EventTimer::~EventTimer() {
    for (auto e : pool) cudaEventDestroy(e);
}
}  // namespace tn

// -------------------------------------------------------------------------------------
// C ABI
// -------------------------------------------------------------------------------------
extern "C" {

const char* tn_last_error(void) { return g_err.c_str(); }
const char* tn_version(void) { return "tennet-gb300 0.1 (sm_103a)"; }
int64_t tn_kernel_launches(void) { return launch_count(); }

int tn_ctx_create(int device, tn_ctx** out) {
    return guarded([&] {
        TN_REQUIRE(out != nullptr, "null output handle");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0)
            throw Error(TN_E_NOGPU, "no CUDA device " + std::to_string(device));
        cudaDeviceProp pr;
        TN_CUDA(cudaGetDeviceProperties(&pr, device));
        if (!(pr.major == 10 && pr.minor == 3))
            throw Error(TN_E_NOGPU, std::string("device is not sm_103 (GB300): ") + pr.name);
        TN_CUDA(cudaSetDevice(device));
        auto c = std::make_unique<tn_ctx>();
        c->device = device;
        TN_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->timer.s = c->stream;
        c->nsm = pr.multiProcessorCount;
        c->err.alloc(4 * sizeof(int), c->stream);  // [0] error flag, [1] injected wait timeout
        TN_CUDA(cudaMemsetAsync(c->err.p, 0, 4 * sizeof(int), c->stream));
        TN_CUDA(cudaStreamSynchronize(c->stream));
        cudaMemPool_t mp;
        TN_CUDA(cudaDeviceGetDefaultMemPool(&mp, device));
        uint64_t thr = UINT64_MAX;
        TN_CUDA(cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &thr));
        *out = c.release();
    });
}

int tn_ctx_destroy(tn_ctx* ctx) {
    return guarded([&] {
        if (!ctx) return;
        cudaStreamSynchronize(ctx->stream);
        cudaStream_t s = ctx->stream;
        delete ctx;
        cudaStreamDestroy(s);
    });
}

int tn_ctx_set_precision(tn_ctx* ctx, int mode, int slices) {
    return guarded([&] {
        TN_REQUIRE(ctx, "null context");
        TN_REQUIRE(mode == TN_PREC_FP64 || mode == TN_PREC_SPLIT, "unknown precision mode");
        TN_REQUIRE(slices >= 2 && slices <= 7, "slices must be in [2, 7]");
        TN_REQUIRE(mode == TN_PREC_FP64 || (slices >= 4 && slices <= 7),
                   "split precision needs 4..7 slices");
        ctx->prec = mode;
        ctx->slices = slices;
    });
}

int tn_ctx_inject_wait_timeout(tn_ctx* ctx, int kernel) {
    return guarded([&] {
        TN_REQUIRE(ctx, "null context");
        TN_REQUIRE(kernel >= 1 && kernel <= 3, "kernel must be 1, 2 or 3");
        const int code = kernel;
        TN_CUDA(cudaMemcpyAsync(ctx->err.as<int>() + 1, &code, sizeof(int), cudaMemcpyHostToDevice,
                                ctx->stream));
        TN_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tn_ctx_set_svd_split(tn_ctx* ctx, int ncols) {
    return guarded([&] {
        TN_REQUIRE(ctx, "null context");
        TN_REQUIRE(ncols >= -1, "the column threshold must be >= 0, or -1 (tuned)");
        ctx->svd_big_n = ncols;
    });
}

int tn_ctx_svd_schedule(tn_ctx* ctx, int32_t* entries, float* ms, int cap, int* count) {
    return guarded([&] {
        TN_REQUIRE(ctx && count && (cap == 0 || (entries && ms)), "null argument");
        *count = int(ctx->svd_tune.table.size());
        int i = 0;
        for (const auto& kv : ctx->svd_tune.table) {
            if (i >= cap) break;
            const SvdTuner::Entry& e = kv.second;
            int32_t* o = entries + size_t(i) * 9;
            o[0] = kv.first;
            o[1] = int(e.cand.size());
            o[2] = e.best >= 0 ? e.cand[size_t(e.best)] : -1;
            o[3] = e.next;
            for (int j = 0; j < 5; ++j) {
                o[4 + j] = j < int(e.cand.size()) ? e.cand[size_t(j)] : 0;
                ms[size_t(i) * 5 + j] = j < int(e.ms.size()) ? e.ms[size_t(j)] : -1.f;
            }
            ++i;
        }
    });
}

int tn_mpo_create(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q, const int32_t* wdims,
                  const int32_t* wq, const double* W, tn_mpo** out) {
    return guarded([&] {
        TN_REQUIRE(ctx && out && phys_q && wdims && wq && W, "null argument");
        TN_REQUIRE(nsites >= 2 && d >= 1, "need at least two sites");
        auto m = std::make_unique<tn_mpo>();
        m->ctx = ctx;
        m->N = nsites;
        m->d = d;
        m->pq.assign(phys_q, phys_q + d);
        m->wd.assign(wdims, wdims + nsites + 1);
        TN_REQUIRE(m->wd[0] == 1 && m->wd[nsites] == 1, "boundary MPO links must have dimension 1");
        size_t qo = 0, wo = 0;
        for (int i = 0; i <= nsites; ++i) {
            TN_REQUIRE(m->wd[i] >= 1, "MPO link dimension must be >= 1");
            m->delta.emplace_back(wq + qo, wq + qo + m->wd[i]);
            qo += m->wd[i];
        }
        for (int i = 0; i < nsites; ++i) {
            const size_t n = size_t(m->wd[i]) * m->wd[i + 1] * d * d;
            m->W.emplace_back(W + wo, W + wo + n);
            wo += n;
            for (int a = 0; a < m->wd[i]; ++a)
                for (int b = 0; b < m->wd[i + 1]; ++b)
                    for (int sp = 0; sp < d; ++sp)
                        for (int s = 0; s < d; ++s)
                            if (m->at(i, a, b, sp, s) != 0.0 &&
                                m->pq[sp] - m->pq[s] != m->delta[i + 1][b] - m->delta[i][a])
                                throw Error(TN_E_INVALID, "MPO entry violates charge conservation at site " +
                                                              std::to_string(i));
        }
        *out = m.release();
    });
}

int tn_mpo_destroy(tn_mpo* mpo) {
    delete mpo;
    return TN_OK;
}

int tn_mps_create(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q, const int32_t* nsec,
                  const int32_t* sec_q, const int32_t* sec_dim, const double* site_data,
                  int center, tn_mps** out) {
    return guarded([&] {
        TN_REQUIRE(ctx && out && phys_q && nsec && sec_q && sec_dim && site_data, "null argument");
        TN_REQUIRE(nsites >= 2, "need at least two sites");
        TN_REQUIRE(center >= 0 && center < nsites, "center out of range");
        auto m = std::make_unique<tn_mps>();
        m->ctx = ctx;
        m->N = nsites;
        m->d = d;
        m->pq.assign(phys_q, phys_q + d);
        m->center = center;
        size_t so = 0;
        for (int i = 0; i <= nsites; ++i) {
            Link L;
            for (int k = 0; k < nsec[i]; ++k) {
                L.q.push_back(sec_q[so + k]);
                L.dim.push_back(sec_dim[so + k]);
                TN_REQUIRE(sec_dim[so + k] >= 1, "sector dimension must be >= 1");
                if (k) TN_REQUIRE(sec_q[so + k] > sec_q[so + k - 1], "sectors must be sorted by charge");
            }
            so += nsec[i];
            TN_REQUIRE(L.nsec() >= 1, "every link needs a sector");
            m->links.push_back(L);
        }
        TN_REQUIRE(m->links[0].total() == 1 && m->links[nsites].total() == 1,
                   "boundary links must have dimension 1");
        m->sites.resize(nsites);
        size_t off = 0;
        std::vector<double> blocks;
        for (int i = 0; i < nsites; ++i) {
            const Link& lk = m->links[i];
            const Link& rk = m->links[i + 1];
            m->sites[i].lay = make_site_layout(i < center ? LG : RG, lk, rk, m->pq);
            site_from_dense(m->sites[i].lay, lk, rk, d, site_data + off, blocks);
            off += size_t(lk.total()) * d * rk.total();
            m->sites[i].buf.alloc(std::max<size_t>(blocks.size(), 1) * 8, ctx->stream);
            if (!blocks.empty())
                TN_CUDA(cudaMemcpyAsync(m->sites[i].buf.p, blocks.data(), blocks.size() * 8,
                                        cudaMemcpyHostToDevice, ctx->stream));
            sync(ctx);
        }
        *out = m.release();
    });
}

int tn_mps_create_complex(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q,
                          const int32_t* nsec, const int32_t* sec_q, const int32_t* sec_dim,
                          const double* site_data, int center, tn_mps** out) {
    return guarded([&] {
        TN_REQUIRE(ctx && out && nsec && sec_dim && site_data, "null argument");
        // total dense length from the link dimensions
        std::vector<int64_t> tot(size_t(nsites) + 1, 0);
        size_t so = 0;
        for (int i = 0; i <= nsites; ++i) {
            for (int k = 0; k < nsec[i]; ++k) tot[size_t(i)] += sec_dim[so + k];
            so += nsec[i];
        }
        int64_t len = 0;
        for (int i = 0; i < nsites; ++i) len += tot[size_t(i)] * d * tot[size_t(i) + 1];
        std::vector<double> re(static_cast<size_t>(len)), im(static_cast<size_t>(len));
        for (int64_t e = 0; e < len; ++e) {
            re[size_t(e)] = site_data[2 * e];
            im[size_t(e)] = site_data[2 * e + 1];
        }
        tn_mps* m = nullptr;
        const int rc = tn_mps_create(ctx, nsites, d, phys_q, nsec, sec_q, sec_dim, re.data(),
                                     center, &m);
        if (rc != TN_OK) throw Error(rc, g_err);
        std::unique_ptr<tn_mps> hold(m);
        mps_to_complex(m);
        size_t off = 0;
        std::vector<double> blocks;
        for (int i = 0; i < nsites; ++i) {
            const Link& lk = m->links[i];
            const Link& rk = m->links[i + 1];
            site_from_dense(m->sites[i].lay, lk, rk, d, im.data() + off, blocks);
            off += size_t(lk.total()) * d * rk.total();
            if (!blocks.empty())
                TN_CUDA(cudaMemcpyAsync(m->sites[i].buf.d() + m->sites[i].lay.size, blocks.data(),
                                        blocks.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
            sync(ctx);
        }
        *out = hold.release();
    });
}

int tn_mps_create_blocks(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q,
                         const int32_t* nsec, const int32_t* sec_q, const int32_t* sec_dim,
                         const double* block_data, const int64_t* site_len, int center,
                         tn_mps** out) {
    return guarded([&] {
        TN_REQUIRE(ctx && out && phys_q && nsec && sec_q && sec_dim && block_data && site_len,
                   "null argument");
        TN_REQUIRE(nsites >= 2, "need at least two sites");
        TN_REQUIRE(center >= 0 && center < nsites, "center out of range");
        auto m = std::make_unique<tn_mps>();
        m->ctx = ctx;
        m->N = nsites;
        m->d = d;
        m->pq.assign(phys_q, phys_q + d);
        m->center = center;
        size_t so = 0;
        for (int i = 0; i <= nsites; ++i) {
            Link L;
            for (int k = 0; k < nsec[i]; ++k) {
                L.q.push_back(sec_q[so + k]);
                L.dim.push_back(sec_dim[so + k]);
                TN_REQUIRE(sec_dim[so + k] >= 1, "sector dimension must be >= 1");
                if (k) TN_REQUIRE(sec_q[so + k] > sec_q[so + k - 1], "sectors must be sorted by charge");
            }
            so += nsec[i];
            TN_REQUIRE(L.nsec() >= 1, "every link needs a sector");
            m->links.push_back(L);
        }
        TN_REQUIRE(m->links[0].total() == 1 && m->links[nsites].total() == 1,
                   "boundary links must have dimension 1");
        m->sites.resize(nsites);
        cudaStream_t st = ctx->stream;
        DevBuf tmp;
        int64_t off = 0;
        for (int i = 0; i < nsites; ++i) {
            const Link& lk = m->links[i];
            const Link& rk = m->links[i + 1];
            // the block order of the ABI is the right-grouped layout's memory order
            const SiteLayout rg = make_site_layout(RG, lk, rk, m->pq);
            TN_REQUIRE(site_len[i] == rg.size, "site block data has the wrong length");
            tn_site& S = m->sites[i];
            S.lay = i < center ? make_site_layout(LG, lk, rk, m->pq) : rg;
            S.buf.alloc(size_t(std::max<int64_t>(rg.size, 1)) * 8, st);
            if (rg.size == 0) continue;
            if (S.lay.layout == RG) {
                TN_CUDA(cudaMemcpyAsync(S.buf.p, block_data + off, size_t(rg.size) * 8,
                                        cudaMemcpyHostToDevice, st));
            } else {
                tmp.alloc(size_t(rg.size) * 8, st);
                TN_CUDA(cudaMemcpyAsync(tmp.p, block_data + off, size_t(rg.size) * 8,
                                        cudaMemcpyHostToDevice, st));
                regroup(ctx, rg, tmp.d(), S.lay, S.buf.d(), lk, rk);
            }
            off += rg.size;
        }
        sync(ctx);
        *out = m.release();
    });
}

int tn_mps_site_blocks(const tn_mps* mps, int site, double* out, int64_t cap, int64_t* len) {
    return guarded([&] {
        TN_REQUIRE(mps && len, "null argument");
        TN_REQUIRE(!mps->cplx, "block download of complex states is not built");
        TN_REQUIRE(site >= 0 && site < mps->N, "site out of range");
        const tn_site& S = mps->sites[site];
        *len = S.lay.size;
        if (!out) return;
        TN_REQUIRE(cap >= S.lay.size, "capacity too small");
        if (S.lay.size == 0) return;
        cudaStream_t st = mps->ctx->stream;
        if (S.lay.layout == RG) {
            TN_CUDA(cudaMemcpyAsync(out, S.buf.p, size_t(S.lay.size) * 8, cudaMemcpyDeviceToHost, st));
        } else {
            const Link& lk = mps->links[site];
            const Link& rk = mps->links[site + 1];
            const SiteLayout rg = make_site_layout(RG, lk, rk, mps->pq);
            DevBuf tmp;
            tmp.alloc(size_t(rg.size) * 8, st);
            regroup(mps->ctx, S.lay, S.buf.d(), rg, tmp.d(), lk, rk);
            TN_CUDA(cudaMemcpyAsync(out, tmp.p, size_t(rg.size) * 8, cudaMemcpyDeviceToHost, st));
        }
        TN_CUDA(cudaStreamSynchronize(st));
    });
}

int tn_mps_destroy(tn_mps* mps) {
    if (mps) cudaStreamSynchronize(mps->ctx->stream);
    delete mps;
    return TN_OK;
}

int tn_mps_link(const tn_mps* mps, int link, int32_t* nsec, int32_t* q, int32_t* dim, int cap) {
    return guarded([&] {
        TN_REQUIRE(mps && nsec, "null argument");
        TN_REQUIRE(link >= 0 && link <= mps->N, "link out of range");
        const Link& L = mps->links[link];
        *nsec = L.nsec();
        if (q || dim) {
            TN_REQUIRE(cap >= L.nsec(), "capacity too small");
            for (int k = 0; k < L.nsec(); ++k) {
                if (q) q[k] = L.q[k];
                if (dim) dim[k] = L.dim[k];
            }
        }
    });
}

int tn_mps_site(const tn_mps* mps, int site, double* out, int64_t cap) {
    return guarded([&] {
        TN_REQUIRE(mps && out, "null argument");
        TN_REQUIRE(!mps->cplx, "complex state: read its sites with tn_mps_site_complex");
        TN_REQUIRE(site >= 0 && site < mps->N, "site out of range");
        const Link& lk = mps->links[site];
        const Link& rk = mps->links[site + 1];
        TN_REQUIRE(cap >= int64_t(lk.total()) * mps->d * rk.total(), "capacity too small");
        const tn_site& S = mps->sites[site];
        std::vector<double> blocks(size_t(S.lay.size));
        if (!blocks.empty())
            TN_CUDA(cudaMemcpyAsync(blocks.data(), S.buf.p, blocks.size() * 8,
                                    cudaMemcpyDeviceToHost, mps->ctx->stream));
        TN_CUDA(cudaStreamSynchronize(mps->ctx->stream));
        site_to_dense(S.lay, lk, rk, mps->d, blocks, out);
    });
}

int tn_mps_is_complex(const tn_mps* mps) { return mps ? (mps->cplx ? 1 : 0) : TN_E_INVALID; }

int tn_mps_make_complex(tn_mps* mps) {
    return guarded([&] {
        TN_REQUIRE(mps, "null argument");
        mps_to_complex(mps);
        sync(mps->ctx);
    });
}

int tn_mps_site_complex(const tn_mps* mps, int site, double* out, int64_t cap) {
    return guarded([&] {
        TN_REQUIRE(mps && out, "null argument");
        TN_REQUIRE(site >= 0 && site < mps->N, "site out of range");
        const Link& lk = mps->links[site];
        const Link& rk = mps->links[site + 1];
        const int64_t nd = int64_t(lk.total()) * mps->d * rk.total();
        TN_REQUIRE(cap >= 2 * nd, "capacity too small");
        const tn_site& S = mps->sites[site];
        const int64_t n = S.lay.size;
        std::vector<double> blocks(size_t(n) * mps->planes());
        if (!blocks.empty())
            TN_CUDA(cudaMemcpyAsync(blocks.data(), S.buf.p, blocks.size() * 8,
                                    cudaMemcpyDeviceToHost, mps->ctx->stream));
        TN_CUDA(cudaStreamSynchronize(mps->ctx->stream));
        std::vector<double> re(static_cast<size_t>(nd)), im(static_cast<size_t>(nd), 0.0);
        std::vector<double> part(blocks.begin(), blocks.begin() + n);
        site_to_dense(S.lay, lk, rk, mps->d, part, re.data());
        if (mps->cplx) {
            part.assign(blocks.begin() + n, blocks.end());
            site_to_dense(S.lay, lk, rk, mps->d, part, im.data());
        }
        for (int64_t e = 0; e < nd; ++e) {
            out[2 * e] = re[size_t(e)];
            out[2 * e + 1] = im[size_t(e)];
        }
    });
}

int tn_mps_center(const tn_mps* mps) { return mps ? mps->center : TN_E_INVALID; }

int tn_env_create(tn_mps* psi, tn_mpo* H, tn_env** out) {
    return guarded([&] {
        TN_REQUIRE(psi && H && out, "null argument");
        TN_REQUIRE(psi->N == H->N && psi->d == H->d && psi->pq == H->pq,
                   "MPS and MPO site indices differ");
        auto e = std::make_unique<tn_env>();
        e->ctx = psi->ctx;
        e->psi = copy_mps(psi);
        e->H = H;
        const int N = psi->N;
        e->L.resize(N);
        e->R.resize(N);
        make_trivial_env(e->ctx, e->L[0], psi->links[0], H->delta[0], env_planes(psi));
        make_trivial_env(e->ctx, e->R[N - 1], psi->links[N], H->delta[N], env_planes(psi));
        e->lpos = 0;
        e->rpos = N - 1;
        e->pos = 0;
        e->nsite = 2;
        *out = e.release();
    });
}

int tn_env_update_mpo(tn_env* env, tn_mpo* H, int recalc_env) {
    return guarded([&] {
        TN_REQUIRE(env && H, "null argument");
        const tn_mps* psi = env->psi.get();
        TN_REQUIRE(H->ctx == env->ctx, "the MPO belongs to another context");
        TN_REQUIRE(psi->N == H->N && psi->d == H->d && psi->pq == H->pq,
                   "MPS and MPO site indices differ");
        const int N = psi->N;
        if (recalc_env) {
            // a new ProjMPO (src/mps/state_envs.jl:183-188): every environment is dropped and
            // rebuilt from the new MPO as positions are taken
            env->H = H;
            make_trivial_env(env->ctx, env->L[0], psi->links[0], H->delta[0], env_planes(psi));
            make_trivial_env(env->ctx, env->R[N - 1], psi->links[N], H->delta[N], env_planes(psi));
            env->lpos = 0;
            env->rpos = N - 1;
        } else {
            // the new MPO takes the old one's place and the environments built so far stay
            // (state_envs.jl:189-208): the next half sweep reads right environments of the
            // old MPO
            TN_REQUIRE(env->proj.empty(),
                       "`updateH!()` :: recalcEnv = false is defined for a single MPO only");
            TN_REQUIRE(env->lpos == 0, "`updateH!()` :: recalcEnv = false needs lpos == 0");
            TN_REQUIRE(psi->center == 0,
                       "`updateH!()` :: recalcEnv = false needs the orthogonality center at site 1");
            TN_REQUIRE(H->wd == env->H->wd && H->delta == env->H->delta,
                       "`updateH!()` :: recalcEnv = false needs the link indices of the old MPO");
            env->H = H;
        }
        env->hp_pos = -1;  // the H_eff plans carry the old MPO's tensors
        env->h1p_pos = -1;
    });
}

int tn_env_set_projectors(tn_env* env, const tn_mps* const* Ms, int count, double weight) {
    return guarded([&] {
        TN_REQUIRE(env, "null argument");
        TN_REQUIRE(count >= 0 && count <= 32, "between 0 and 32 projector states");
        const tn_mps* psi = env->psi.get();
        TN_REQUIRE(!psi->cplx || count == 0, "projectors on complex states are not built");
        if (count > 0) {
            TN_REQUIRE(Ms, "null argument");
            if (!(weight > 0.0)) {
                char msg[160];
                std::snprintf(msg, sizeof msg,
                              "`weight` parameter should be > 0.0 (value passed was `weight=%g`)",
                              weight);
                throw Error(TN_E_INVALID, msg);
            }
            for (int k = 0; k < count; ++k)
                TN_REQUIRE(Ms[k] && Ms[k]->ctx == env->ctx && Ms[k]->N == psi->N &&
                               Ms[k]->d == psi->d && Ms[k]->pq == psi->pq,
                           "projector states must share the context and the site indices of psi");
        }
        sync(env->ctx);
        env->proj.clear();
        for (int k = 0; k < count; ++k) {
            ProjState P;
            P.M = copy_mps(Ms[k]);
            env->proj.push_back(std::move(P));
        }
        env->proj_weight = count > 0 ? weight : 0.0;
        proj_init(env);
        sync(env->ctx);
        check_device_error(env->ctx);
        env->ctx->timer.collect(env->acc_ms);
    });
}

int tn_env_destroy(tn_env* env) {
    if (env) cudaStreamSynchronize(env->ctx->stream);
    delete env;
    return TN_OK;
}

int tn_env_getpsi(tn_env* env, tn_mps** out) {
    return guarded([&] {
        TN_REQUIRE(env && out, "null argument");
        auto m = copy_mps(env->psi.get());
        sync(env->ctx);
        *out = m.release();
    });
}

int tn_env_position(tn_env* env, int pos, int nsite) {
    return guarded([&] {
        TN_REQUIRE(env, "null argument");
        position(env, pos, nsite);
        sync(env->ctx);
        check_device_error(env->ctx);
        env->ctx->timer.collect(env->acc_ms);
    });
}

int tn_env_environment(tn_env* env, int side, int i, double* out, int64_t cap,
                       int32_t* dims) {
    return guarded([&] {
        TN_REQUIRE(env && dims, "null argument");
        const tn_mps* psi = env->psi.get();
        const int N = psi->N;
        TN_REQUIRE(!psi->cplx, "environment download of complex states is not built");
        TN_REQUIRE(i >= 0 && i < N, "environment index out of range");
        TN_REQUIRE(side == 0 ? i <= env->lpos : i >= env->rpos,
                   "environment is not built; call tn_env_position first");
        const tn_envt& E = side == 0 ? env->L[i] : env->R[i];
        const Link& lk = psi->links[side == 0 ? i : i + 1];
        const int w = env->H->wd[side == 0 ? i : i + 1];
        const int D = lk.total();
        dims[0] = D;
        dims[1] = w;
        dims[2] = D;
        if (!out) return;
        TN_REQUIRE(cap >= int64_t(D) * w * D, "capacity too small");
        std::vector<double> blocks(size_t(E.lay.size));
        if (!blocks.empty())
            TN_CUDA(cudaMemcpyAsync(blocks.data(), E.buf.p, blocks.size() * 8,
                                    cudaMemcpyDeviceToHost, env->ctx->stream));
        sync(env->ctx);
        std::fill(out, out + int64_t(D) * w * D, 0.0);
        const auto off = lk.offsets();
        for (int a = 0; a < w; ++a)
            for (int x = 0; x < lk.nsec(); ++x) {
                const int64_t bo = E.lay.off[size_t(a) * E.lay.nsec + x];
                if (bo < 0) continue;
                const int xb = E.lay.bra[size_t(a) * E.lay.nsec + x];
                for (int c = 0; c < lk.dim[x]; ++c)
                    for (int r = 0; r < lk.dim[xb]; ++r)
                        out[int64_t(off[xb] + r) + int64_t(D) * (a + int64_t(w) * (off[x] + c))] =
                            blocks[size_t(bo + r + int64_t(lk.dim[xb]) * c)];
            }
    });
}

int tn_env_product_flops(tn_env* env, double* flops) {
    return guarded([&] {
        TN_REQUIRE(env && flops, "null argument");
        Heff2Plan& P = heff_plan(env);
        *flops = P.flops;
    });
}

int tn_env_product_complex(tn_env* env, const double* v, double* out, int64_t n) {
    return guarded([&] {
        TN_REQUIRE(env && v && out, "null argument");
        TN_REQUIRE(env->psi->cplx, "a real state: use tn_env_product");
        TN_REQUIRE(env->nsite == 2, "only nsite = 2 products are built");
        const int p = env->pos;
        position(env, p, 2);
        Heff2Plan& P = heff_plan(env);
        const tn_mps* psi = env->psi.get();
        const Link& lk = psi->links[p];
        const Link& rk = psi->links[p + 2];
        const int64_t nd = int64_t(lk.total()) * psi->d * psi->d * rk.total();
        TN_REQUIRE(n == nd, "dense two-site tensor has the wrong size");
        std::vector<int64_t> map;
        phi_dense_map(P.ph, lk, rk, psi->d, map);
        const int64_t nb = P.ph.size;
        std::vector<double> hb(size_t(2 * nb));
        for (int64_t i = 0; i < nb; ++i) {
            hb[size_t(i)] = v[2 * map[size_t(i)]];
            hb[size_t(nb + i)] = v[2 * map[size_t(i)] + 1];
        }
        cudaStream_t st = env->ctx->stream;
        env->vecA.alloc(std::max<size_t>(hb.size(), 1) * 8, st);
        env->vecB.alloc(std::max<size_t>(hb.size(), 1) * 8, st);
        if (!hb.empty())
            TN_CUDA(cudaMemcpyAsync(env->vecA.p, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st));
        heff_apply(env, P, env->vecA.d(), env->vecB.d());
        if (!hb.empty())
            TN_CUDA(cudaMemcpyAsync(hb.data(), env->vecB.p, hb.size() * 8, cudaMemcpyDeviceToHost, st));
        sync(env->ctx);
        check_device_error(env->ctx);
        env->ctx->timer.collect(env->acc_ms);
        std::fill(out, out + 2 * nd, 0.0);
        for (int64_t i = 0; i < nb; ++i) {
            out[2 * map[size_t(i)]] = hb[size_t(i)];
            out[2 * map[size_t(i)] + 1] = hb[size_t(nb + i)];
        }
    });
}

int tn_env_product(tn_env* env, const double* v, double* out, int64_t n) {
    return guarded([&] {
        TN_REQUIRE(env && v && out, "null argument");
        TN_REQUIRE(!env->psi->cplx, "complex state: use tn_env_product_complex");
        TN_REQUIRE(env->nsite == 2, "only nsite = 2 products are built");
        const int p = env->pos;
        position(env, p, 2);
        Heff2Plan& P = heff_plan(env);
        const tn_mps* psi = env->psi.get();
        const Link& lk = psi->links[p];
        const Link& rk = psi->links[p + 2];
        const int64_t nd = int64_t(lk.total()) * psi->d * psi->d * rk.total();
        TN_REQUIRE(n == nd, "dense two-site tensor has the wrong size");
        std::vector<int64_t> map;
        phi_dense_map(P.ph, lk, rk, psi->d, map);
        std::vector<double> hb(size_t(P.ph.size));
        for (size_t i = 0; i < hb.size(); ++i) hb[i] = v[map[i]];
        cudaStream_t st = env->ctx->stream;
        env->vecA.alloc(std::max<size_t>(hb.size(), 1) * 8, st);
        env->vecB.alloc(std::max<size_t>(hb.size(), 1) * 8, st);
        if (!hb.empty())
            TN_CUDA(cudaMemcpyAsync(env->vecA.p, hb.data(), hb.size() * 8, cudaMemcpyHostToDevice, st));
        heff_apply(env, P, env->vecA.d(), env->vecB.d());
        if (!env->proj.empty()) {  // ProjMPO_MPS2 product (src/mps/projmpo_mps2.jl:94-101)
            env->part.alloc(size_t(32) * blas_nparts() * 8, st);
            proj_vectors2(env, p, P.ph);
            proj_apply(env, env->vecA.d(), env->vecB.d(), P.ph.size);
        }
        if (!hb.empty())
            TN_CUDA(cudaMemcpyAsync(hb.data(), env->vecB.p, hb.size() * 8, cudaMemcpyDeviceToHost, st));
        sync(env->ctx);
        check_device_error(env->ctx);
        env->ctx->timer.collect(env->acc_ms);
        std::fill(out, out + nd, 0.0);
        for (size_t i = 0; i < hb.size(); ++i) out[map[i]] = hb[i];
    });
}

int tn_env_update_position(tn_env* env, int pos, int ortho, const tn_update_params* p,
                           tn_update_result* res, double* eigs, int eigs_cap) {
    return tn_env_update_position_nsite(env, pos, 2, ortho, p, res, eigs, eigs_cap);
}

int tn_env_update_position_nsite(tn_env* env, int pos, int nsite, int ortho,
                                 const tn_update_params* p, tn_update_result* res, double* eigs,
                                 int eigs_cap) {
    return guarded([&] {
        TN_REQUIRE(env && res, "null argument");
        TN_REQUIRE(ortho == TN_ORTHO_LEFT || ortho == TN_ORTHO_RIGHT, "ortho must be left or right");
        TN_REQUIRE(nsite == 1 || nsite == 2, "nsite must be 1 or 2");
        std::vector<double> ev;
        *res = tn_update_result{};
        if (nsite == 2)
            update_two_site(env, pos, ortho, p, res, ev);
        else
            update_one_site(env, pos, ortho, p, res, ev);
        if (eigs) {
            const int k = std::min<int>(eigs_cap, (int)ev.size());
            std::copy(ev.begin(), ev.begin() + k, eigs);
        }
        sync(env->ctx);
        env->ctx->timer.collect(env->acc_ms);
    });
}

}  // extern "C"

namespace {
// per-bond choice of dynamic_fullsweep! (TenNetLib src/mps/sweep.jl:257-355): the smallest
// kept eigenvalue of each bond's last spectrum (SweepData.lasteigs[bond][end]), the threshold
// under which a bond takes a one-site update, and where the choices are reported (bond b of
// the left half at [b], of the right half at [N - 1 + b]; may be null)
struct DynamicSweep {
    const double* last_min;
    double eigthreshold;
    int32_t* choices;
};

// fullsweep! (TenNetLib src/mps/sweep.jl:94-196) with the eigensolver (time_step null) or
// the exponential solver at time_step with reverse steps (tdvpsweep!, src/mps/tdvp.jl:268);
// with dyn, dynamic_fullsweep!'s mixed one-/two-site sweep (sweep.jl:284-355)
void full_sweep(tn_env* env, const tn_update_params* p, tn_sweep_result* res, double* mid_eigs,
                int mid_cap, int32_t* n_mid_eigs, const double* time_step, int nsite = 2,
                double time_im = 0.0, const DynamicSweep* dyn = nullptr) {
    TN_REQUIRE(env && res, "null argument");
    check_params(p);
    tn_mps* psi = env->psi.get();
    TN_REQUIRE(psi->center == 0, "fullsweep! needs the orthogonality center at site 1");
    const int N = psi->N;
    tn_ctx* ctx = env->ctx;
    ctx->timer.collect(env->acc_ms);
    double acc0[T_NCAT];
    std::copy(env->acc_ms, env->acc_ms + T_NCAT, acc0);
    const int64_t mv0 = env->matvecs;
    const double fl0 = env->heff_flops;
    const double gf0 = env->gemm_flops;
    const int64_t gl0 = env->gemm_launches;
    const int64_t kl0 = launch_count();
    const int64_t kb0 = krylov_bytes();
    *res = tn_sweep_result{};
    ctx->svd_stats = BsvdStats{};
    const int es = ctx->timer.mark();
    double maxerr = 0.0, energy = NAN;
    std::vector<double> ev, mid;
    std::vector<std::vector<double>> last(size_t(N - 1));
    if (dyn) {
        // per bond (sweep.jl:302-304, 322-324): one site when the bond's last spectrum ends
        // below eigthreshold or its link is at maxdim, else two sites; the right half reads
        // the spectra the left half left (lasteigs is shared between the halves)
        auto pick = [&](int b, double lmin) {
            return (lmin < dyn->eigthreshold || psi->links[b + 1].total() >= p->maxdim) ? 1 : 2;
        };
        for (int b = 0; b < N - 1; ++b) {
            const int ns = pick(b, dyn->last_min[b]);
            if (dyn->choices) dyn->choices[b] = ns;
            tn_update_result r{};
            if (ns == 1)
                update_one_site(env, b, TN_ORTHO_LEFT, p, &r, ev, time_step, time_im);
            else
                update_two_site(env, b, TN_ORTHO_LEFT, p, &r, ev, time_step, time_im);
            energy = r.energy;
            maxerr = std::max(maxerr, r.truncerr);
            last[size_t(b)] = ev;
            if (ns == 1 && b == N - 2) {  // the last site (sweep.jl:314-316)
                tn_update_result r2{};
                update_one_site(env, N - 1, TN_ORTHO_LEFT, p, &r2, ev, time_step, time_im);
                energy = r2.energy;
            }
        }
        for (int b = N - 2; b >= 0; --b) {
            const auto& e = last[size_t(b)];
            const int ns = pick(b, e.empty() ? HUGE_VAL : e.back());
            if (dyn->choices) dyn->choices[N - 1 + b] = ns;
            tn_update_result r{};
            if (ns == 1)
                update_one_site(env, b + 1, TN_ORTHO_RIGHT, p, &r, ev, time_step, time_im);
            else
                update_two_site(env, b, TN_ORTHO_RIGHT, p, &r, ev, time_step, time_im);
            energy = r.energy;
            maxerr = std::max(maxerr, r.truncerr);
            last[size_t(b)] = ev;
            if (ns == 1 && b == 0) {  // the first site (sweep.jl:333-335)
                tn_update_result r2{};
                update_one_site(env, 0, TN_ORTHO_RIGHT, p, &r2, ev, time_step, time_im);
                energy = r2.energy;
            }
        }
        mid = last[size_t(N / 2 - 1)];
    } else if (nsite == 2) {
        for (int b = 0; b < N - 1; ++b) {
            tn_update_result r{};
            update_two_site(env, b, TN_ORTHO_LEFT, p, &r, ev, time_step, time_im);
            energy = r.energy;
            maxerr = std::max(maxerr, r.truncerr);
        }
        for (int b = N - 2; b >= 0; --b) {
            tn_update_result r{};
            update_two_site(env, b, TN_ORTHO_RIGHT, p, &r, ev, time_step, time_im);
            energy = r.energy;
            maxerr = std::max(maxerr, r.truncerr);
            last[size_t(b)] = ev;
            if (b == N / 2 - 1) mid = ev;
        }
    } else {
        // one-site sweep (src/mps/sweep.jl:118-152 with nsite = 1): sites 1..N left, then
        // N..1 right; lasteigs[bond] comes from the right-moving update at site bond + 1
        for (int q = 0; q < N; ++q) {
            tn_update_result r{};
            update_one_site(env, q, TN_ORTHO_LEFT, p, &r, ev, time_step, time_im);
            energy = r.energy;
            maxerr = std::max(maxerr, r.truncerr);
        }
        for (int q = N - 1; q >= 0; --q) {
            tn_update_result r{};
            update_one_site(env, q, TN_ORTHO_RIGHT, p, &r, ev, time_step, time_im);
            energy = r.energy;
            maxerr = std::max(maxerr, r.truncerr);
            if (q >= 1) last[size_t(q - 1)] = ev;
            if (q == N / 2) mid = ev;
        }
    }
    env->bond_eigs = std::move(last);
    ctx->timer.add(T_SWEEP, es, ctx->timer.mark());
    sync(ctx);
    ctx->timer.collect(env->acc_ms);
    int maxd = 0;
    for (const auto& L : psi->links) maxd = std::max(maxd, L.total());
    res->energy = energy;
    res->maxtruncerr = maxerr;
    res->maxlinkdim = maxd;
    res->matvecs = int32_t(env->matvecs - mv0);
    res->heff_flops = env->heff_flops - fl0;
    res->heff_ms = env->acc_ms[T_HEFF] - acc0[T_HEFF];
    res->env_ms = env->acc_ms[T_ENV] - acc0[T_ENV];
    res->svd_ms = env->acc_ms[T_SVD] - acc0[T_SVD];
    res->lanczos_ms = env->acc_ms[T_LANCZOS] - acc0[T_LANCZOS];
    res->sweep_ms = env->acc_ms[T_SWEEP] - acc0[T_SWEEP];
    res->gemm_ms = env->acc_ms[T_GEMM] - acc0[T_GEMM];
    res->pack_ms = env->acc_ms[T_PACK] - acc0[T_PACK];
    res->gemm_flops = env->gemm_flops - gf0;
    res->gemm_launches = env->gemm_launches - gl0;
    res->kernel_launches = launch_count() - kl0;
    res->krylov_bytes = double(krylov_bytes() - kb0);
    res->svd_gemm_flops = ctx->svd_stats.gemm_flops;
    res->svd_jacobi_flops = ctx->svd_stats.jacobi_flops;
    res->svd_sweeps32 = ctx->svd_stats.sweeps32;
    res->svd_sweeps_df = ctx->svd_stats.sweeps_df;
    res->svd_small_flops = ctx->svd_stats.small_flops;
    if (n_mid_eigs) *n_mid_eigs = (int32_t)mid.size();
    if (mid_eigs) {
        const int k = std::min<int>(mid_cap, (int)mid.size());
        std::copy(mid.begin(), mid.begin() + k, mid_eigs);
    }
}
}  // namespace

extern "C" {

int tn_env_fullsweep(tn_env* env, const tn_update_params* p, tn_sweep_result* res,
                     double* mid_eigs, int mid_cap, int32_t* n_mid_eigs) {
    return guarded([&] { full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, nullptr); });
}

int tn_env_fullsweep_nsite(tn_env* env, int nsite, const tn_update_params* p,
                           tn_sweep_result* res, double* mid_eigs, int mid_cap,
                           int32_t* n_mid_eigs) {
    return guarded([&] {
        TN_REQUIRE(nsite == 1 || nsite == 2, "nsite must be 1 or 2");
        full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, nullptr, nsite);
    });
}

int tn_env_tdvpsweep(tn_env* env, double tau, const tn_update_params* p, tn_sweep_result* res,
                     double* mid_eigs, int mid_cap, int32_t* n_mid_eigs) {
    return guarded([&] {
        TN_REQUIRE(std::isfinite(tau), "time step must be finite");
        const double half = 0.5 * tau;
        full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, &half);
    });
}

int tn_env_tdvpsweep_complex(tn_env* env, double tau_re, double tau_im, const tn_update_params* p,
                             tn_sweep_result* res, double* mid_eigs, int mid_cap,
                             int32_t* n_mid_eigs) {
    return guarded([&] {
        TN_REQUIRE(env, "null argument");
        TN_REQUIRE(std::isfinite(tau_re) && std::isfinite(tau_im), "time step must be finite");
        if (tau_im != 0.0) env_to_complex(env);
        const double half = 0.5 * tau_re;
        full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, &half, 2, 0.5 * tau_im);
    });
}

int tn_env_tdvpsweep_nsite(tn_env* env, int nsite, double tau_re, double tau_im,
                           const tn_update_params* p, tn_sweep_result* res, double* mid_eigs,
                           int mid_cap, int32_t* n_mid_eigs) {
    return guarded([&] {
        TN_REQUIRE(env, "null argument");
        TN_REQUIRE(nsite == 1 || nsite == 2, "nsite must be 1 or 2");
        TN_REQUIRE(std::isfinite(tau_re) && std::isfinite(tau_im), "time step must be finite");
        if (tau_im != 0.0) env_to_complex(env);
        const double half = 0.5 * tau_re;
        full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, &half, nsite, 0.5 * tau_im);
    });
}

int tn_env_fullsweep_dynamic(tn_env* env, double eigthreshold, const double* last_min,
                             int32_t* choices, const tn_update_params* p, tn_sweep_result* res,
                             double* mid_eigs, int mid_cap, int32_t* n_mid_eigs) {
    return guarded([&] {
        TN_REQUIRE(env && last_min, "null argument");
        TN_REQUIRE(!std::isnan(eigthreshold), "eigthreshold must be a number");
        const DynamicSweep dyn{last_min, eigthreshold, choices};
        full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, nullptr, 2, 0.0, &dyn);
    });
}

int tn_env_tdvpsweep_dynamic(tn_env* env, double tau_re, double tau_im, double eigthreshold,
                             const double* last_min, int32_t* choices, const tn_update_params* p,
                             tn_sweep_result* res, double* mid_eigs, int mid_cap,
                             int32_t* n_mid_eigs) {
    return guarded([&] {
        TN_REQUIRE(env && last_min, "null argument");
        TN_REQUIRE(std::isfinite(tau_re) && std::isfinite(tau_im), "time step must be finite");
        TN_REQUIRE(!std::isnan(eigthreshold), "eigthreshold must be a number");
        if (tau_im != 0.0) env_to_complex(env);
        const double half = 0.5 * tau_re;
        const DynamicSweep dyn{last_min, eigthreshold, choices};
        full_sweep(env, p, res, mid_eigs, mid_cap, n_mid_eigs, &half, 2, 0.5 * tau_im, &dyn);
    });
}

int tn_env_bond_spectra(const tn_env* env, double* out, int64_t cap, int32_t* counts,
                        int ncounts) {
    return guarded([&] {
        TN_REQUIRE(env && counts, "null argument");
        const int nb = env->psi->N - 1;
        TN_REQUIRE(ncounts >= nb, "counts must hold one entry per bond (N - 1)");
        int64_t total = 0;
        for (int b = 0; b < nb; ++b) {
            const bool have = b < int(env->bond_eigs.size());
            counts[b] = have ? int32_t(env->bond_eigs[size_t(b)].size()) : 0;
            total += counts[b];
        }
        if (!out) return;  // lengths only
        TN_REQUIRE(total <= cap, "output buffer too small for the spectra");
        int64_t o = 0;
        for (int b = 0; b < nb && b < int(env->bond_eigs.size()); ++b)
            for (double v : env->bond_eigs[size_t(b)]) out[o++] = v;
    });
}

int tn_env_make_complex(tn_env* env) {
    return guarded([&] {
        TN_REQUIRE(env, "null argument");
        env_to_complex(env);
    });
}

int tn_svd_truncate(tn_ctx* ctx, int nblocks, const int32_t* rows, const int32_t* cols,
                    const double* data, int32_t maxdim, int32_t mindim, double cutoff,
                    int32_t* kept, double* svals, double* truncerr) {
    return guarded([&] {
        TN_REQUIRE(ctx && rows && cols && data && kept, "null argument");
        TN_REQUIRE(nblocks >= 1, "need at least one block");
        TN_REQUIRE(maxdim >= 1 && mindim >= 1, "maxdim and mindim must be >= 1");
        std::vector<int> r(rows, rows + nblocks), c(cols, cols + nblocks);
        std::vector<int64_t> offs(nblocks);
        int64_t tot = 0;
        for (int b = 0; b < nblocks; ++b) {
            TN_REQUIRE(r[b] >= 1 && c[b] >= 1, "block dimensions must be >= 1");
            offs[b] = tot;
            tot += int64_t(r[b]) * c[b];
        }
        cudaStream_t st = ctx->stream;
        DevBuf src, X, W, V, P, S, Pm, desc;
        src.alloc(size_t(tot) * 8, st);
        TN_CUDA(cudaMemcpyAsync(src.p, data, size_t(tot) * 8, cudaMemcpyHostToDevice, st));
        SvdResult R;
        block_svd(ctx, X, W, V, P, S, Pm, desc, r, c, offs, src.d(), R);
        TruncDecision D = decide(R, maxdim, mindim, cutoff);
        for (int b = 0; b < nblocks; ++b) kept[b] = D.kept[b];
        if (svals) std::copy(R.S.begin(), R.S.end(), svals);
        if (truncerr) *truncerr = D.truncerr;
        sync(ctx);
        double scratch_ms[T_NCAT] = {0, 0, 0, 0, 0, 0, 0};
        ctx->timer.collect(scratch_ms);
    });
}

}  // extern "C"
