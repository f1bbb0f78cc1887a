// Local expectation values <psi|O_i|psi> / <psi|psi> of an MPS for every site i: the
// measure(T, psi, opstr) of TenNetLib (src/mps/measure.jl:150-219) on the GPU.
//
// The reference moves the orthogonality centre to each site in turn (orthogonalize!) and
// contracts the centre tensor with the operator.  Here the same numbers come from transfer
// matrices, which need no factorisation: E_i (contraction of sites < i with their copies)
// from the left, F_i (sites >= i) from the right, each block-diagonal in the link charge
// sectors, then <O_i> = sum_{s', s} O[s', s] <A_{s'}, E_i A_s F_{i+1}^T> / <psi|psi>.  Only
// O[s', s] with q_{s'} = q_s contribute (charge conservation); all arithmetic is FP64 grouped
// GEMMs plus one batched Frobenius-dot kernel.
#include <cstring>
#include <map>
#include <tuple>

#include "engine.h"

using namespace tn;

namespace {

struct SubBlock {  // A_s[l, r] of site i: D_l x D_r at off (concatenated sites), leading dim ld
    int64_t off;
    int ld, s, l, r;
};

template <class F>
int guarded_m(F&& f) {
    try {
        f();
        return TN_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return TN_E_INVALID;
    }
}

}  // namespace

extern "C" int tn_mps_expect_local(tn_mps* mps, const double* op, double* out) {
    return guarded_m([&] {
        TN_REQUIRE(mps && op && out, "null argument");
        tn_ctx* ctx = mps->ctx;
        cudaStream_t st = ctx->stream;
        const int N = mps->N, d = mps->d;
        const int np = mps->planes();  // complex: every buffer below holds two planes
        // concatenated site blocks and their sub-matrices A_s[l, r]
        std::vector<int64_t> soff(N + 1, 0);
        for (int i = 0; i < N; ++i) soff[i + 1] = soff[i] + mps->sites[i].lay.size;
        DevBuf S;
        S.alloc(size_t(std::max<int64_t>(soff[N], 1)) * 8 * np, st);
        for (int i = 0; i < N; ++i)
            for (int pl = 0; pl < np; ++pl)
                if (mps->sites[i].lay.size)
                    TN_CUDA(cudaMemcpyAsync(S.d() + pl * soff[N] + soff[i],
                                            mps->sites[i].buf.d() + pl * mps->sites[i].lay.size,
                                            size_t(mps->sites[i].lay.size) * 8,
                                            cudaMemcpyDeviceToDevice, st));
        std::vector<std::vector<SubBlock>> subs(N);
        for (int i = 0; i < N; ++i) {
            const SiteLayout& L = mps->sites[i].lay;
            const Link& lk = mps->links[i];
            const Link& rk = mps->links[i + 1];
            for (int b = 0; b < L.nblk(); ++b)
                for (int s = 0; s < d; ++s) {
                    const int sub = L.sub[size_t(b) * d + s];
                    if (sub < 0) continue;
                    const int oth = L.subsec[size_t(b) * d + s];
                    SubBlock x;
                    x.s = s;
                    x.ld = L.rows[b];
                    if (L.layout == LG) {
                        x.l = oth;
                        x.r = b;
                        x.off = soff[i] + L.off[b] + sub;
                    } else {
                        x.l = b;
                        x.r = oth;
                        x.off = soff[i] + L.off[b] + int64_t(sub) * L.rows[b];
                    }
                    if (lk.dim[x.l] > 0 && rk.dim[x.r] > 0) subs[i].push_back(x);
                }
        }
        // transfer matrices: one D_x x D_x block per sector x of every link
        std::vector<std::vector<int64_t>> eoff(N + 1);
        int64_t etot = 0;
        for (int i = 0; i <= N; ++i)
            for (int x = 0; x < mps->links[i].nsec(); ++x) {
                eoff[i].push_back(etot);
                etot += int64_t(mps->links[i].dim[x]) * mps->links[i].dim[x];
            }
        DevBuf E, F, T, X;
        E.alloc(size_t(etot) * 8 * np, st);
        F.alloc(size_t(etot) * 8 * np, st);
        TN_CUDA(cudaMemsetAsync(E.p, 0, size_t(etot) * 8 * np, st));
        TN_CUDA(cudaMemsetAsync(F.p, 0, size_t(etot) * 8 * np, st));
        const double one = 1.0;
        TN_CUDA(cudaMemcpyAsync(E.d() + eoff[0][0], &one, 8, cudaMemcpyHostToDevice, st));
        TN_CUDA(cudaMemcpyAsync(F.d() + eoff[N][0], &one, 8, cudaMemcpyHostToDevice, st));
        // temporaries: per sub-block D_l x D_r (largest site, and all sites for the local stage)
        std::vector<std::vector<int64_t>> toff(N);
        int64_t ttot = 0, tmax = 0;
        for (int i = 0; i < N; ++i) {
            int64_t t = 0;
            for (const auto& x : subs[i]) {
                toff[i].push_back(ttot + t);
                t += int64_t(mps->links[i].dim[x.l]) * mps->links[i + 1].dim[x.r];
            }
            ttot += t;
            tmax = std::max(tmax, t);
        }
        T.alloc(size_t(std::max<int64_t>(ttot, 1)) * 8 * np, st);
        X.alloc(size_t(std::max<int64_t>(ttot, 1)) * 8 * np, st);
        Bases bs{};
        bs.p[S_L] = E.d();
        bs.p[S_R] = F.d();
        bs.p[S_X] = S.d();
        bs.p[S_T1] = T.d();
        bs.p[S_T2] = X.d();
        if (np == 2) {
            bs.p[S_L + S_IM] = E.d() + etot;
            bs.p[S_R + S_IM] = F.d() + etot;
            bs.p[S_X + S_IM] = S.d() + soff[N];
            bs.p[S_T1 + S_IM] = T.d() + ttot;
            bs.p[S_T2 + S_IM] = X.d() + ttot;
        }
        // complex states: the bra factors (the conjugated site tensors) enter through
        // complex_plan's conjugation; F is Hermitian, so the local stage's F^T becomes F^H = F
        auto run = [&](GemmPlan& g, unsigned conj) {
            if (np == 2) {
                GemmPlan c = complex_plan(g, conj);
                c.finalize(st);
                launch_gemm_f64(c, bs, st);
                TN_CUDA(cudaStreamSynchronize(st));  // the plan goes out of scope
            } else {
                g.finalize(st);
                launch_gemm_f64(g, bs, st);
            }
        };
        const int e0 = ctx->timer.mark();
        // left pass: T = E_i[l] A_s ; E_{i+1}[r] = sum_s A_s^T T
        for (int i = 0; i < N; ++i) {
            const Link& lk = mps->links[i];
            const Link& rk = mps->links[i + 1];
            GemmPlan g1, g2;
            std::map<int, std::vector<size_t>> byr;
            for (size_t k = 0; k < subs[i].size(); ++k) {
                const auto& x = subs[i][k];
                const int Dl = lk.dim[x.l], Dr = rk.dim[x.r];
                g1.add_task(S_T1, toff[i][k], Dl, Dr, Dl);
                g1.add_seg(S_L, eoff[i][x.l], Dl, 0, S_X, x.off, x.ld, 0, Dl);
                byr[x.r].push_back(k);
            }
            for (auto& kv : byr) {
                const int Dr = rk.dim[kv.first];
                g2.add_task(S_L, eoff[i + 1][kv.first], Dr, Dr, Dr);
                for (size_t k : kv.second) {
                    const auto& x = subs[i][k];
                    g2.add_seg(S_X, x.off, x.ld, 1, S_T1, toff[i][k], lk.dim[x.l], 0, lk.dim[x.l]);
                }
            }
            run(g1, 0);
            run(g2, 1u << S_X);
            TN_CUDA(cudaStreamSynchronize(st));  // plans go out of scope
        }
        // right pass: U = A_s F_{i+1}[r] ; F_i[l] = sum_s U A_s^T
        for (int i = N - 1; i >= 0; --i) {
            const Link& lk = mps->links[i];
            const Link& rk = mps->links[i + 1];
            GemmPlan g1, g2;
            std::map<int, std::vector<size_t>> byl;
            for (size_t k = 0; k < subs[i].size(); ++k) {
                const auto& x = subs[i][k];
                const int Dl = lk.dim[x.l], Dr = rk.dim[x.r];
                g1.add_task(S_T1, toff[i][k], Dl, Dr, Dl);
                g1.add_seg(S_X, x.off, x.ld, 0, S_R, eoff[i + 1][x.r], Dr, 0, Dr);
                byl[x.l].push_back(k);
            }
            for (auto& kv : byl) {
                const int Dl = lk.dim[kv.first];
                g2.add_task(S_R, eoff[i][kv.first], Dl, Dl, Dl);
                for (size_t k : kv.second) {
                    const auto& x = subs[i][k];
                    g2.add_seg(S_T1, toff[i][k], Dl, 0, S_X, x.off, x.ld, 1, rk.dim[x.r]);
                }
            }
            run(g1, 0);
            run(g2, 1u << S_X);
            TN_CUDA(cudaStreamSynchronize(st));
        }
        // local stage, all sites at once: W = E_i[l] A_s ; X = W F_{i+1}[r]^T ; dots with A_{s'}
        GemmPlan ga, gb;
        std::vector<BlockDot> dots;
        struct Key { int i, sp, s; };
        std::vector<Key> keys;
        for (int i = 0; i < N; ++i) {
            const Link& lk = mps->links[i];
            const Link& rk = mps->links[i + 1];
            for (size_t k = 0; k < subs[i].size(); ++k) {
                const auto& x = subs[i][k];
                const int Dl = lk.dim[x.l], Dr = rk.dim[x.r];
                ga.add_task(S_T1, toff[i][k], Dl, Dr, Dl);
                ga.add_seg(S_L, eoff[i][x.l], Dl, 0, S_X, x.off, x.ld, 0, Dl);
                gb.add_task(S_T2, toff[i][k], Dl, Dr, Dl);
                gb.add_seg(S_T1, toff[i][k], Dl, 0, S_R, eoff[i + 1][x.r], Dr, 1, Dr);
                for (const auto& y : subs[i]) {
                    if (y.l != x.l || y.r != x.r) continue;
                    BlockDot bd;
                    bd.x = X.d() + toff[i][k];
                    bd.y = S.d() + y.off;
                    bd.ldx = Dl;
                    bd.ldy = y.ld;
                    bd.rows = Dl;
                    bd.cols = Dr;
                    dots.push_back(bd);
                    keys.push_back(Key{i, y.s, x.s});
                    if (np == 2) {  // Re sum conj(a) x = a_re . x_re + a_im . x_im
                        bd.x = X.d() + ttot + toff[i][k];
                        bd.y = S.d() + soff[N] + y.off;
                        dots.push_back(bd);
                        keys.push_back(Key{i, y.s, x.s});
                    }
                }
            }
        }
        run(ga, 0);
        run(gb, 1u << S_R);
        DevBuf dd, dout;
        dd.alloc(std::max<size_t>(dots.size(), 1) * sizeof(BlockDot), st);
        dout.alloc(std::max<size_t>(dots.size(), 1) * 8, st);
        if (!dots.empty()) {
            TN_CUDA(cudaMemcpyAsync(dd.p, dots.data(), dots.size() * sizeof(BlockDot),
                                    cudaMemcpyHostToDevice, st));
            launch_block_dots(dd.as<BlockDot>(), int(dots.size()), dout.d(), st);
        }
        std::vector<double> part(dots.size());
        double norm = 0.0;
        TN_CUDA(cudaMemcpyAsync(&norm, E.d() + eoff[N][0], 8, cudaMemcpyDeviceToHost, st));
        if (!dots.empty())
            TN_CUDA(cudaMemcpyAsync(part.data(), dout.p, dots.size() * 8, cudaMemcpyDeviceToHost, st));
        ctx->timer.add(T_ENV, e0, ctx->timer.mark());
        TN_CUDA(cudaStreamSynchronize(st));
        TN_REQUIRE(norm > 0.0, "the state has zero norm");
        for (int i = 0; i < N; ++i) out[i] = 0.0;
        for (size_t k = 0; k < dots.size(); ++k) {
            const Key& q = keys[k];
            out[q.i] += op[q.sp + size_t(d) * q.s] * part[k];  // O[s', s], column-major
        }
        for (int i = 0; i < N; ++i) out[i] /= norm;
    });
}

// <a|b> of two MPS on the same sites (ITensorMPS inner(psi, phi) on the sweep's states):
// mixed transfer matrices E_{i+1}[q] (Da_q x Db_q) = sum_s A_s[l, q]^T E_i[l] B_s[l, q] over
// the charge sectors present in both states, FP64 grouped GEMMs; the result is E_N.
namespace {
void overlap_impl(const tn_mps* a, const tn_mps* b, double* out, bool cx) {
    {
        TN_REQUIRE(a && b && out, "null argument");
        TN_REQUIRE(a->ctx == b->ctx && a->N == b->N && a->d == b->d && a->pq == b->pq,
                   "overlap needs two states of one context on the same sites");
        tn_ctx* ctx = a->ctx;
        cudaStream_t st = ctx->stream;
        const int N = a->N, d = a->d;
        // sub-blocks keyed by (s, left charge, right charge)
        auto subs_of = [&](const tn_mps* m, int i) {
            std::map<std::tuple<int, int, int>, SubBlock> out_map;
            const SiteLayout& L = m->sites[i].lay;
            for (int bk = 0; bk < L.nblk(); ++bk)
                for (int s = 0; s < d; ++s) {
                    const int sub = L.sub[size_t(bk) * d + s];
                    if (sub < 0) continue;
                    const int oth = L.subsec[size_t(bk) * d + s];
                    SubBlock x;
                    x.s = s;
                    x.ld = L.rows[bk];
                    if (L.layout == LG) {
                        x.l = oth;
                        x.r = bk;
                        x.off = L.off[bk] + sub;
                    } else {
                        x.l = bk;
                        x.r = oth;
                        x.off = L.off[bk] + int64_t(sub) * L.rows[bk];
                    }
                    out_map[{s, m->links[i].q[x.l], m->links[i + 1].q[x.r]}] = x;
                }
            return out_map;
        };
        // E_i blocks for the charges present in both links
        std::vector<std::map<int, int64_t>> eoff(N + 1);
        int64_t etot = 0;
        for (int i = 0; i <= N; ++i) {
            const Link& la = a->links[i];
            const Link& lb = b->links[i];
            for (int x = 0; x < la.nsec(); ++x) {
                const int y = lb.find(la.q[x]);
                if (y < 0) continue;
                eoff[i][la.q[x]] = etot;
                etot += int64_t(la.dim[x]) * lb.dim[y];
            }
        }
        TN_REQUIRE(!eoff[0].empty() && !eoff[N].empty(), "the states have different total charges");
        const int np = cx ? 2 : 1;
        DevBuf E, T, Za, Zb;  // Za / Zb: zero imaginary planes of a real state in a complex overlap
        E.alloc(size_t(std::max<int64_t>(etot, 1)) * 8 * np, st);
        TN_CUDA(cudaMemsetAsync(E.p, 0, E.bytes, st));
        const double one = 1.0;
        TN_CUDA(cudaMemcpyAsync(E.d() + eoff[0].begin()->second, &one, 8, cudaMemcpyHostToDevice, st));
        for (int i = 0; i < N; ++i) {
            const auto sa = subs_of(a, i), sb = subs_of(b, i);
            const Link &lka = a->links[i], &lkb = b->links[i], &rka = a->links[i + 1],
                       &rkb = b->links[i + 1];
            struct Job { SubBlock xa, xb; int64_t toff, eo, en; int Dla, Dlb, Dra, Drb; int qr; };
            std::vector<Job> jobs;
            int64_t t = 0;
            for (const auto& kv : sa) {
                auto it = sb.find(kv.first);
                if (it == sb.end()) continue;
                const int ql = std::get<1>(kv.first), qr = std::get<2>(kv.first);
                if (!eoff[i].count(ql) || !eoff[i + 1].count(qr)) continue;
                Job j;
                j.xa = kv.second;
                j.xb = it->second;
                j.Dla = lka.dim[j.xa.l];
                j.Dlb = lkb.dim[j.xb.l];
                j.Dra = rka.dim[j.xa.r];
                j.Drb = rkb.dim[j.xb.r];
                j.eo = eoff[i][ql];
                j.en = eoff[i + 1][qr];
                j.qr = qr;
                j.toff = t;
                t += int64_t(j.Dla) * j.Drb;
                jobs.push_back(j);
            }
            T.alloc(size_t(std::max<int64_t>(t, 1)) * 8 * np, st);
            Bases bs{};
            bs.p[S_L] = E.d();
            bs.p[S_X] = a->sites[i].buf.d();
            bs.p[S_A] = b->sites[i].buf.d();
            bs.p[S_T1] = T.d();
            if (cx) {
                auto im_of = [&](const tn_mps* m, DevBuf& Z) {
                    const int64_t n = m->sites[i].lay.size;
                    if (m->cplx) return m->sites[i].buf.d() + n;
                    Z.alloc(size_t(std::max<int64_t>(n, 1)) * 8, st);
                    TN_CUDA(cudaMemsetAsync(Z.p, 0, Z.bytes, st));
                    return Z.d();
                };
                bs.p[S_L + S_IM] = E.d() + etot;
                bs.p[S_X + S_IM] = im_of(a, Za);
                bs.p[S_A + S_IM] = im_of(b, Zb);
                bs.p[S_T1 + S_IM] = T.d() + t;
            }
            GemmPlan g1, g2;
            std::map<int, std::vector<size_t>> byr;
            for (size_t k = 0; k < jobs.size(); ++k) {
                const Job& j = jobs[k];
                // T = E_i[ql] (Da_l x Db_l) * B_s (Db_l x Db_r)
                g1.add_task(S_T1, j.toff, j.Dla, j.Drb, j.Dla);
                g1.add_seg(S_L, j.eo, j.Dla, 0, S_A, j.xb.off, j.xb.ld, 0, j.Dlb);
                byr[j.qr].push_back(k);
            }
            for (auto& kv : byr) {
                const Job& j0 = jobs[kv.second[0]];
                g2.add_task(S_L, j0.en, j0.Dra, j0.Drb, j0.Dra);
                for (size_t k : kv.second) {
                    const Job& j = jobs[k];
                    g2.add_seg(S_X, j.xa.off, j.xa.ld, 1, S_T1, j.toff, j.Dla, 0, j.Dla);
                }
            }
            if (cx) {  // <a|b>: a conjugated
                GemmPlan c1 = complex_plan(g1, 0), c2 = complex_plan(g2, 1u << S_X);
                c1.finalize(st);
                c2.finalize(st);
                launch_gemm_f64(c1, bs, st);
                launch_gemm_f64(c2, bs, st);
            } else {
                g1.finalize(st);
                g2.finalize(st);
                launch_gemm_f64(g1, bs, st);
                launch_gemm_f64(g2, bs, st);
            }
            TN_CUDA(cudaStreamSynchronize(st));
        }
        const int64_t eN = eoff[N].begin()->second;
        TN_CUDA(cudaMemcpyAsync(&out[0], E.d() + eN, 8, cudaMemcpyDeviceToHost, st));
        if (cx) TN_CUDA(cudaMemcpyAsync(&out[1], E.d() + etot + eN, 8, cudaMemcpyDeviceToHost, st));
        TN_CUDA(cudaStreamSynchronize(st));
    }
}
}  // namespace

extern "C" int tn_mps_overlap(const tn_mps* a, const tn_mps* b, double* out) {
    return guarded_m([&] {
        TN_REQUIRE(a && b, "null argument");
        TN_REQUIRE(!a->cplx && !b->cplx, "complex states: use tn_mps_overlap_complex");
        overlap_impl(a, b, out, false);
    });
}

extern "C" int tn_mps_overlap_complex(const tn_mps* a, const tn_mps* b, double* out) {
    return guarded_m([&] { overlap_impl(a, b, out, true); });
}
