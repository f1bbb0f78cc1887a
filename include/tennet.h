/*
 * tennet.h -- C ABI of libtennet_cuda.so, the GB300 (sm_103a) sweep engine for the
 * DMRG hot path of TenNetLib.jl.
 *
 * Every call returns 0 on success or a negative TN_E_* code; tn_last_error() returns the
 * message of the last failure on the calling thread.  No call aborts or throws across
 * the ABI.  Host arrays are copied on entry and never retained; all device memory is
 * owned by the library and released by the matching *_destroy call.
 *
 * Conventions shared by all calls:
 *  - sites are 0-based (site i of the ABI is site i+1 of the Julia API);
 *  - a link (virtual bond) is a list of charge sectors (q, dim) sorted by q ascending;
 *    link i sits left of site i (links 0..N);
 *  - a physical site has d basis states with charges phys_q[0..d-1];
 *  - dense tensors cross the ABI column-major (first index fastest, Julia order): a site
 *    tensor is (Dl, d, Dr), a two-site tensor (Dl, d, d, Dr), a one-site tensor
 *    (Dl, d, Dr); basis states of a link are ordered sector by sector;
 *  - an MPO is given per site as a dense (w_left, w_right, d, d) array [a, b, s', s]
 *    column-major with one charge per MPO link state; W[a,b,s',s] may be nonzero only when
 *    q_{s'} - q_s = delta_b - delta_a.
 */
#ifndef TENNET_H
#define TENNET_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TN_OK 0
#define TN_E_INVALID (-1)      /* bad argument, layout or charge mismatch */
#define TN_E_CUDA (-2)         /* CUDA runtime error */
#define TN_E_NOMEM (-3)        /* device allocation failed */
#define TN_E_NOTCONV (-4)      /* solver did not converge and check_convergence was set */
#define TN_E_NOGPU (-5)        /* no usable sm_103 device */
#define TN_E_TIMEOUT (-6)      /* a bounded device wait gave up */

/* arithmetic of the contraction GEMMs */
#define TN_PREC_FP64 0         /* FP64 on CUDA cores: the FP64 GPU oracle */
#define TN_PREC_SPLIT 1        /* bf16 slices on tcgen05 tensor cores, FP64-recovered */

#define TN_ORTHO_LEFT 0        /* ortho = "left": sweep moves right, U stays left */
#define TN_ORTHO_RIGHT 1       /* ortho = "right": sweep moves left, V stays right */

typedef struct tn_ctx tn_ctx;
typedef struct tn_mpo tn_mpo;
typedef struct tn_mps tn_mps;
typedef struct tn_env tn_env;

/* keyword arguments of update_position! / fullsweep! / eig_solver
 * (TenNetLib src/mps/update_site.jl:235-245, src/base/solver.jl:26-35) */
typedef struct tn_update_params {
    int32_t maxdim;            /* typemax(Int) in Julia: pass INT32_MAX */
    int32_t mindim;            /* default 1 */
    double cutoff;             /* default Float64_threshold() = 1e-15 */
    int32_t normalize;         /* default 1 */
    int32_t krylovdim;         /* default 5 */
    int32_t maxiter;           /* default 2 */
    double tol;                /* default 1e-14 */
    int32_t eager;             /* default 0 */
    int32_t check_convergence; /* default 0 */
    double noise;              /* density-matrix perturbation (two-site updates; 0 = off) */
} tn_update_params;

typedef struct tn_update_result {
    double energy;             /* Ritz value of the last solve */
    double truncerr;           /* relative discarded weight of replacebond! */
    int32_t newdim;            /* bond dimension after truncation */
    int32_t matvecs;           /* H_eff applications of the solve */
    int32_t converged;         /* converged Ritz pairs */
    int32_t neigs;             /* number of kept S^2 values written to eigs (if given) */
} tn_update_result;

typedef struct tn_sweep_result {
    double energy;             /* energy of the last update (bond 1 of the right pass) */
    double maxtruncerr;
    int32_t maxlinkdim;
    int32_t matvecs;           /* total H_eff applications in the sweep */
    double heff_flops;         /* algorithmic flops of all H_eff applications */
    double heff_ms;            /* device time of the H_eff applications (CUDA events) */
    double env_ms;             /* device time of environment updates */
    double svd_ms;             /* device time of the block SVDs */
    double lanczos_ms;         /* device time of the Krylov vector kernels */
    double sweep_ms;           /* device time of the whole sweep */
    double gemm_ms;            /* device time of the grouped-GEMM launches of H_eff */
    double gemm_flops;         /* algorithmic flops of those launches */
    double pack_ms;            /* device time of the bf16 slice packing (split precision) */
    int64_t gemm_launches;     /* number of those launches */
    int64_t kernel_launches;   /* all kernels this library launched during the sweep */
    double qr_panel_ms;        /* TTN: device time of the Householder column/panel kernels */
    double qr_gemm_ms;         /* TTN: device time of the QR's grouped GEMMs (with packing) */
    double krylov_bytes;       /* algorithmic HBM bytes of the Krylov vector kernels */
    double svd_gemm_flops;     /* algorithmic flops of the multi-SM block SVD's grouped GEMMs */
    double svd_jacobi_flops;   /* flops of its Jacobi rotations (dots and column updates) */
    int32_t svd_sweeps32;      /* largest FP32 presolve sweep count of a block */
    int32_t svd_sweeps_df;     /* largest double-float polish sweep count of a block */
    double svd_small_flops;    /* algorithmic flops of the one-CTA block SVDs (QR, Jacobi
                                * sweeps as run, Gram-Schmidt, R^T V, Q V) */
} tn_sweep_result;

/* ---- context ------------------------------------------------------------------- */
/* Replaces nothing in the reference (ITensors runs on the host); owns stream + pool. */
int tn_ctx_create(int device, tn_ctx** out);
int tn_ctx_destroy(tn_ctx* ctx);
/* TN_PREC_FP64 or TN_PREC_SPLIT; slices = bf16 slices per FP64 operand (2..7). */
int tn_ctx_set_precision(tn_ctx* ctx, int mode, int slices);
/* Block SVD of replacebond!: charge blocks with more than ncols columns (of the m >= n
 * orientation) are factored by the multi-SM pipeline (blocked QR + cooperative Jacobi), the
 * others by one CTA each; 0 sends every block to the multi-SM pipeline.  Default -1: the
 * threshold is tuned per block-size histogram (keyed on the bond's largest block in
 * 32-column buckets; each candidate threshold is timed once on the first bonds of a key,
 * then the fastest is kept). */
int tn_ctx_set_svd_split(tn_ctx* ctx, int ncols);
/* The tuned SVD schedule so far: *count keys; for the first cap of them entries[9 i ..] =
 * (bucket, candidates, chosen threshold or -1 while still timing, candidates timed,
 * threshold of candidate 0..4 (2147483647: every block on one CTA)) and ms[5 i ..] = the
 * measured milliseconds of each candidate (-1: not yet timed). */
int tn_ctx_svd_schedule(tn_ctx* ctx, int32_t* entries, float* ms, int cap, int* count);
/* Test hook of the failure path (no counterpart in the reference, whose solver only raises
 * on non-convergence, src/base/solver.jl:38-41): the next launch on this context of the
 * named kernel makes one of its bounded device waits run out, without any fault:
 * 1 = split-precision tensor-core GEMM (one CTA withholds one stage's bulk copies),
 * 2 = cooperative Jacobi of the multi-SM block SVD, 3 = cooperative Householder panel of the
 * TTN QR (one CTA leaves before its first barrier).  The call that ran the kernel returns
 * TN_E_TIMEOUT after about a second; the context stays usable. */
int tn_ctx_inject_wait_timeout(tn_ctx* ctx, int kernel);
const char* tn_last_error(void);
const char* tn_version(void);
/* number of CUDA kernels this library has launched since it was loaded (diagnostics) */
int64_t tn_kernel_launches(void);

/* ---- MPO --------------------------------------------------------------------------
 * Replaces the ITensorMPS MPO handed to StateEnvs(psi, H::MPO)
 * (TenNetLib src/mps/state_envs.jl:54-60).
 * wdims[N+1]: MPO link dimensions (wdims[0] = wdims[N] = 1); wq: concatenated MPO link
 * charges (sum wdims); W: concatenated dense site tensors. */
int tn_mpo_create(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q,
                  const int32_t* wdims, const int32_t* wq, const double* W, tn_mpo** out);
int tn_mpo_destroy(tn_mpo* mpo);

/* ---- MPS --------------------------------------------------------------------------
 * Replaces the ITensorMPS MPS (psi) of StateEnvs.  nsec[N+1], sec_q/sec_dim concatenated
 * sectors of links 0..N; site_data concatenated dense site tensors.  center = site of the
 * orthogonality center: sites < center must be left isometries, sites > center right
 * isometries (fullsweep! needs center = 0, TenNetLib src/mps/sweep.jl:100-104). */
int tn_mps_create(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q,
                  const int32_t* nsec, const int32_t* sec_q, const int32_t* sec_dim,
                  const double* site_data, int center, tn_mps** out);
/* The same from charge blocks only (the block-sparse storage of an ITensors QN MPS, no
 * zeros crossing the boundary).  Site i's data is the concatenation, over its left sectors a
 * (ascending charge) and physical states s (ascending), of the Dl(a) x Dr(b) block with
 * q_b = q_a + phys_q[s] (column-major), for every such b present in link i + 1;
 * site_len[i] is its length and block_data holds all sites back to back. */
int tn_mps_create_blocks(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q,
                         const int32_t* nsec, const int32_t* sec_q, const int32_t* sec_dim,
                         const double* block_data, const int64_t* site_len, int center,
                         tn_mps** out);
int tn_mps_destroy(tn_mps* mps);
/* number of sectors of link i, and (when q/dim are non-null) their charges and dims */
int tn_mps_link(const tn_mps* mps, int link, int32_t* nsec, int32_t* q, int32_t* dim, int cap);
/* dense site tensor (Dl, d, Dr) column-major */
int tn_mps_site(const tn_mps* mps, int site, double* out, int64_t cap);
/* site tensor as charge blocks in the order of tn_mps_create_blocks; *len receives the
 * length (out == NULL: only the length) */
int tn_mps_site_blocks(const tn_mps* mps, int site, double* out, int64_t cap, int64_t* len);
int tn_mps_center(const tn_mps* mps);
/* Complex states (the ComplexF64 MPS of a real-time evolution).  A complex MPS keeps real
 * and imaginary parts of every charge block on the device; tn_mps_make_complex turns a real
 * state into one (imaginary parts zero), tn_mps_is_complex answers 1 or 0, and
 * tn_mps_site_complex writes the dense site tensor (Dl, d, Dr) column-major as interleaved
 * (re, im) pairs, Julia's ComplexF64 memory layout (cap in doubles, >= 2 Dl d Dr; a real
 * state reads with zero imaginary parts).  tn_mps_site and tn_mps_site_blocks take real
 * states only. */
int tn_mps_make_complex(tn_mps* mps);
/* tn_mps_create for a complex state: site_data interleaved (re, im) pairs (ComplexF64) */
int tn_mps_create_complex(tn_ctx* ctx, int nsites, int d, const int32_t* phys_q,
                          const int32_t* nsec, const int32_t* sec_q, const int32_t* sec_dim,
                          const double* site_data, int center, tn_mps** out);
int tn_mps_is_complex(const tn_mps* mps);
int tn_mps_site_complex(const tn_mps* mps, int site, double* out, int64_t cap);
/* measure(T, psi, opstr) for every site (TenNetLib src/mps/measure.jl:150-219): out[i] =
 * <psi|O_i|psi> / <psi|psi> with the single-site operator op (d x d column-major [s', s]),
 * from GPU transfer matrices instead of moving the orthogonality centre (equal for the
 * normalised states the sweeps produce).  Entries with q_{s'} != q_s do not contribute
 * (charge conservation). */
int tn_mps_expect_local(tn_mps* mps, const double* op, double* out);
/* inner(a, b) = <a|b> of two states on the same sites (the ITensorMPS inner that users of
 * TenNetLib call on the states it returns; TenNetLib's own sweep calls no overlap), from GPU
 * transfer matrices over the charge sectors both states carry. */
int tn_mps_overlap(const tn_mps* a, const tn_mps* b, double* out);
/* inner(a, b) when either state is complex: out[0] + i out[1] = <a|b> (a conjugated).
 * tn_mps_expect_local also takes complex states (the real part of <O_i>, O Hermitian). */
int tn_mps_overlap_complex(const tn_mps* a, const tn_mps* b, double* out);

/* ---- StateEnvs --------------------------------------------------------------------
 * StateEnvs(psi, H) (TenNetLib src/mps/state_envs.jl:54-60): copies psi, builds ProjMPO
 * environments lazily. */
int tn_env_create(tn_mps* psi, tn_mpo* H, tn_env** out);
/* updateH!(sysenv, H; recalcEnv) (TenNetLib src/mps/state_envs.jl:181-212, through
 * updateH!(engine, H; recalcEnv) of src/mps/tdvp.jl:182-196): H replaces the MPO of env (same
 * site indices; env keeps a pointer, H must outlive env or the next update).  recalc_env != 0
 * drops every environment (rebuilt from H as positions are taken); recalc_env == 0 keeps the
 * environments built so far -- allowed with no excited-state projectors, the left
 * environments unset (after a full sweep) and the MPO link indices unchanged -- so the next
 * half sweep reads right environments of the old MPO, as the reference does.  Projector
 * environments do not depend on H and stay. */
int tn_env_update_mpo(tn_env* env, tn_mpo* H, int recalc_env);
/* StateEnvs(psi, H, Ms; weight) (src/mps/state_envs.jl:88-105): excited-state projectors.
 * The effective Hamiltonian of every later update and product becomes ProjMPO_MPS2's
 * (src/mps/projmpo_mps2.jl:94-101), H_eff + weight sum_k |m_k><m_k| with m_k the projection
 * of Ms[k] onto the sites being optimised (ProjMPS2, src/mps/projmps2.jl:26-224).  The
 * states are copied; count 0 removes the projectors.  weight <= 0 with count > 0 is
 * TN_E_INVALID with the reference's message; at most 32 states. */
int tn_env_set_projectors(tn_env* env, const tn_mps* const* Ms, int count, double weight);
int tn_env_destroy(tn_env* env);
/* getpsi(sysenv) (state_envs.jl:36): a copy of the current state */
int tn_env_getpsi(tn_env* env, tn_mps** out);
/* position!(sysenv, pos) + set_nsite!(sysenv, nsite) (state_envs.jl:352-367) */
int tn_env_position(tn_env* env, int pos, int nsite);
/* product(sysenv, v) = H_eff * v at the current position (state_envs.jl:376-378).
 * v/out dense (Dl, d, Dr) for nsite = 1 or (Dl, d, d, Dr) for nsite = 2. */
int tn_env_product(tn_env* env, const double* v, double* out, int64_t n);
/* the same for a complex state: v and out interleaved (re, im), n complex entries */
int tn_env_product_complex(tn_env* env, const double* v, double* out, int64_t n);
/* the state of env and its environments made complex (imaginary parts zero) */
int tn_env_make_complex(tn_env* env);
/* dense copy of environment L[i] (side 0: contracts sites < i) or R[i] (side 1: contracts
 * sites > i) as (D, w, D) [bra, MPO state, ket] column-major; dims[3] receives (D, w, D).
 * With out == NULL only dims are written.  The environment must have been built by a
 * position call (ProjMPO's cached LR[i], used via src/mps/state_envs.jl:364-367). */
int tn_env_environment(tn_env* env, int side, int i, double* out, int64_t cap, int32_t* dims);
/* algorithmic flops of one product at the current position */
int tn_env_product_flops(tn_env* env, double* flops);
/* update_position!(sysenv, eig_solver, pos, 2, ortho; kwargs...)
 * (TenNetLib src/mps/update_site.jl:231-277, two-site path :27-90).
 * eigs (optional, capacity eigs_cap) receives the kept S^2 sorted descending. */
int tn_env_update_position(tn_env* env, int pos, int ortho, const tn_update_params* p,
                           tn_update_result* res, double* eigs, int eigs_cap);
/* update_position!(sysenv, eig_solver, pos, nsite, ortho; kwargs...) for nsite 1 or 2:
 * nsite = 1 is _update_one_site! (TenNetLib src/mps/update_site.jl:94-190, noise = 0): the
 * one-site solve at pos (the orthogonality center), then unless the half sweep is done the
 * block SVD with ITensors truncation of the link toward the next site, whose factor S V
 * (ortho left) or U S (ortho right) is multiplied into that site. */
int tn_env_update_position_nsite(tn_env* env, int pos, int nsite, int ortho,
                                 const tn_update_params* p, tn_update_result* res, double* eigs,
                                 int eigs_cap);
/* fullsweep!(sysenv, eig_solver, nsite, swdata; kwargs...) (src/mps/sweep.jl:94-196) for
 * nsite 1 (one-site DMRG, dmrg1 of src/mps/dmrg.jl:314-320) or 2. */
int tn_env_fullsweep_nsite(tn_env* env, int nsite, const tn_update_params* p,
                           tn_sweep_result* res, double* mid_eigs, int mid_cap,
                           int32_t* n_mid_eigs);
/* fullsweep!(sysenv, eig_solver, 2, swdata; kwargs...) (TenNetLib src/mps/sweep.jl:94-196).
 * mid_eigs (optional) receives lasteigs[N/2] (1-based bond N/2), n_mid_eigs its length. */
int tn_env_fullsweep(tn_env* env, const tn_update_params* p, tn_sweep_result* res,
                     double* mid_eigs, int mid_cap, int32_t* n_mid_eigs);

/* tdvpsweep!(engine, tau; nsite = 2, kwargs...) (TenNetLib src/mps/tdvp.jl:247-277): a full
 * sweep with exp_solver (src/base/solver.jl:66-88) at time step tau/2 and the reverse
 * one-site step (src/mps/update_site.jl:78-87).  tau is real in this library (imaginary-time
 * evolution exp(tau H)); p->krylovdim / maxiter / tol are the exp_solver settings
 * (reference defaults 30 / 100 / 1e-12).  Fields of res as for tn_env_fullsweep. */
int tn_env_tdvpsweep(tn_env* env, double tau, const tn_update_params* p, tn_sweep_result* res,
                     double* mid_eigs, int mid_cap, int32_t* n_mid_eigs);
/* tdvpsweep! with a complex time step tau = tau_re + i tau_im (real-time evolution
 * exp(-i dt H) is tau = -i dt).  A real state is made complex first (ITensors promotes the
 * MPS to ComplexF64 the same way); the Krylov exponential, the contractions and the block
 * SVD then run on complex tensors (H_eff products in the context's precision, environment
 * updates, the realified block SVD and the Krylov exponential in FP64). */
int tn_env_tdvpsweep_complex(tn_env* env, double tau_re, double tau_im, const tn_update_params* p,
                             tn_sweep_result* res, double* mid_eigs, int mid_cap,
                             int32_t* n_mid_eigs);
/* tdvpsweep!(engine, tau; nsite) with nsite 1 or 2 and tau = tau_re + i tau_im.  nsite = 1
 * is the one-site sweep of fullsweep! (src/mps/sweep.jl:118-152) with _update_one_site!'s
 * exponential solver and reverse step (src/mps/update_site.jl:94-190): each site evolves by
 * tau/2, is split by the block SVD (ITensors truncation), and the bond matrix evolves back
 * by -tau/2 under the zero-site effective Hamiltonian before it enters the next site. */
int tn_env_tdvpsweep_nsite(tn_env* env, int nsite, double tau_re, double tau_im,
                           const tn_update_params* p, tn_sweep_result* res, double* mid_eigs,
                           int mid_cap, int32_t* n_mid_eigs);
/* The sweep of dynamic_fullsweep! after its first sweep (TenNetLib src/mps/sweep.jl:284-355):
 * left to right, then right to left, bond b (between sites b and b + 1, 0-based) takes a
 * one-site update when last_min[b] (the smallest kept eigenvalue of the bond's spectrum from
 * the previous sweep, SweepData.lasteigs[b][end]) is below eigthreshold or its link dimension
 * is at p->maxdim, else a two-site update; the right half decides on the spectra of the left
 * half, and a one-site update at the end bond adds the update of the end site.  last_min
 * holds N - 1 values; choices (optional, 2 (N - 1) entries) receives the nsite of bond b in
 * the left half at [b] and in the right half at [N - 1 + b].  Global subspace expansion
 * (krylov_extend!, the first sweep and every extendat-th sweep of the reference) is not
 * part of this call. */
int tn_env_fullsweep_dynamic(tn_env* env, double eigthreshold, const double* last_min,
                             int32_t* choices, const tn_update_params* p, tn_sweep_result* res,
                             double* mid_eigs, int mid_cap, int32_t* n_mid_eigs);
/* The same sweep with the exponential solver and reverse steps (tdvpsweep! with
 * nsite = "dynamic", src/mps/tdvp.jl:256-260): each update evolves by tau/2, tau = tau_re +
 * i tau_im (a complex step makes the state complex first, as tn_env_tdvpsweep_complex). */
int tn_env_tdvpsweep_dynamic(tn_env* env, double tau_re, double tau_im, double eigthreshold,
                             const double* last_min, int32_t* choices, const tn_update_params* p,
                             tn_sweep_result* res, double* mid_eigs, int mid_cap,
                             int32_t* n_mid_eigs);
/* SweepData.lasteigs of the last full sweep of any kind: counts[b] (N - 1 entries) receives
 * the length of bond b's kept spectrum (descending squared singular values, 0 before the
 * first sweep), out (cap doubles) the spectra one after another; with out null only the
 * lengths are written. */
int tn_env_bond_spectra(const tn_env* env, double* out, int64_t cap, int32_t* counts,
                        int ncounts);

/* ---- block SVD + truncation -------------------------------------------------------
 * The SVD/truncation of replacebond! (called at TenNetLib src/mps/update_site.jl:64-76)
 * on explicit dense blocks (column-major, concatenated).  kept[nblocks] receives the
 * kept dimension per block; svals (capacity sum min(rows,cols)) the singular values per
 * block sorted descending (all of them, before truncation); truncerr the relative
 * discarded weight. */
int tn_svd_truncate(tn_ctx* ctx, int nblocks, const int32_t* rows, const int32_t* cols,
                    const double* data, int32_t maxdim, int32_t mindim, double cutoff,
                    int32_t* kept, double* svals, double* truncerr);

/* ---- tree tensor networks (TTN) ----------------------------------------------------
 * A tree of nnodes nodes numbered 0..nnodes-1, given by nedges edges (node pairs), with
 * nsites physical sites of dimension d attached (site_node[nsites]).  The legs of a node
 * tensor are its sites in ascending order, then its neighbours in ascending node number;
 * node tensors cross the ABI dense and column-major in that leg order.  TenNetLib labels
 * nodes (layer, index) (src/ttn/ttn.jl:1-30, src/ttn/ttn_generators.jl:69-96): the caller
 * numbers the sorted labels.  No charge conservation (dense node tensors). */
typedef struct tn_ttn tn_ttn;
typedef struct tn_ttn_model tn_ttn_model;
typedef struct tn_ttn_env tn_ttn_env;

/* TTN(sites, graph, tensors, orthocenter) (src/ttn/ttn.jl:21-26).  link_dims[nedges]: bond
 * dimension of each edge in the order given; data: node tensors concatenated in node
 * order; center: the orthogonality centre (every other node an isometry toward it), or -1
 * for arbitrary tensors. */
int tn_ttn_create(tn_ctx* ctx, int nsites, int d, int nnodes, int nedges, const int32_t* edges,
                  const int32_t* site_node, const int32_t* link_dims, const double* data,
                  int center, tn_ttn** out);
int tn_ttn_destroy(tn_ttn* psi);
int tn_ttn_center(const tn_ttn* psi);
/* number of legs of `node` and (dims != NULL, capacity 64) their dimensions in leg order */
int tn_ttn_node_dims(const tn_ttn* psi, int node, int32_t* nlegs, int32_t* dims);
/* dense node tensor, column-major in leg order */
int tn_ttn_node(const tn_ttn* psi, int node, double* out, int64_t cap);
/* maxlinkdim(ttn) (src/ttn/ttn.jl:199-209) */
int tn_ttn_maxlinkdim(const tn_ttn* psi);
/* isometrize!(ttn, node; normalize) (src/ttn/ttn.jl:326-382) with QR moves on the GPU: from
 * scratch (isometrize_full!) when the TTN has no centre, else along the path from it. */
int tn_ttn_isometrize(tn_ttn* psi, int node, int normalize);

/* CouplingModel (src/base/couplingmodel.jl:153-230) from product terms, unmerged: term t is
 * coef[t] * prod_j op_{t,j}, term_nops[t] operators on distinct sites (term_sites, all terms
 * concatenated); ops: d x d column-major matrices [s', s] in the same order. */
int tn_ttn_model_create(int nsites, int d, int nterms, const int32_t* term_nops,
                        const int32_t* term_sites, const double* ops, const double* coef,
                        tn_ttn_model** out);
int tn_ttn_model_destroy(tn_ttn_model* model);

/* StateEnvsTTN(psi, H) (src/ttn/state_envs_ttn.jl:27-31, link tensors built as in
 * LinkTensorsTTN(psi, M), src/ttn/linktensors.jl:233-261) for `count` states at once: the
 * environments share one device arena and are swept together by tn_ttn_envs_fullsweep.
 * All states share one tree and one orthogonality centre; each has its own model. */
int tn_ttn_envs_create(int count, tn_ttn* const* psis, tn_ttn_model* const* models,
                       tn_ttn_env** out);
int tn_ttn_env_destroy(tn_ttn_env* env);
/* getpsi(sysenv) (state_envs_ttn.jl:87): a copy of the current state */
int tn_ttn_env_getpsi(tn_ttn_env* env, tn_ttn** out);
int tn_ttn_env_center(const tn_ttn_env* env);
/* position!(sysenv, node) (state_envs_ttn.jl:120-141): QR moves, normalisation, link
 * tensors moved along the same path (move_linktensors!, src/ttn/linktensors.jl:130-156) */
int tn_ttn_env_position(tn_ttn_env* env, int node);
/* product(sysenv, v) at the orthogonality centre (src/ttn/linktensors.jl:183-221); v and
 * out are dense node tensors of the centre */
int tn_ttn_env_product(tn_ttn_env* env, const double* v, double* out, int64_t n);
/* algorithmic flops of one product at the centre */
int tn_ttn_env_product_flops(tn_ttn_env* env, double* flops);
/* StateEnvsTTN(psi, H, Ms; weight) (src/ttn/state_envs_ttn.jl:36-52): excited-state
 * projectors.  Every later product and update uses EnvCouplingModelProjTTN's effective
 * Hamiltonian (src/ttn/environment.jl:104-110), H_eff + weight sum_k |m_k><m_k|, with m_k
 * the centre tensor of Ms[k] contracted with its overlaps with psi on every link of the
 * centre (LinkProjTTN, src/ttn/linkproj.jl:56-78, 143-224).  The states are copied and need
 * psi's tree and sites; count 0 removes the projectors; weight <= 0 with count > 0 is
 * TN_E_INVALID with the reference's message; at most 32 states. */
int tn_ttn_env_set_projectors(tn_ttn_env* env, const tn_ttn* const* Ms, int count,
                              double weight);
/* update_position!(sysenv, eig_solver, node; kwargs...) (src/ttn/update_site_ttn.jl:42-63);
 * a link larger than p->maxdim on the path is truncated by an SVD move
 * (moveisometry_to_next!, src/ttn/ttn.jl:292-300); p->noise must be 0 */
int tn_ttn_env_update_position(tn_ttn_env* env, int node, const tn_update_params* p,
                               tn_update_result* res);
/* fullsweep!(sysenv, sweeppath, eig_solver, swdata; kwargs...), noise = 0 branch
 * (src/ttn/sweep_ttn.jl:117-274): update_position! along path, then along the reversed
 * path, for the `count` environments created together (envs in creation order), in
 * lockstep: each contraction stage of all of them is one grouped launch.  res[count]
 * receives each environment's energy and maxlinkdim; the timings are of the whole group. */
int tn_ttn_envs_fullsweep(int count, tn_ttn_env* const* envs, int npath, const int32_t* path,
                          const tn_update_params* p, tn_sweep_result* res);
/* fullsweep! with noise = p->noise > 0 (src/ttn/sweep_ttn.jl:180-243): every node of path and
 * of the reversed path but `central` (find_eccentric_central_node) is first made the centre
 * (QR moves, the link move out of its next node toward `central` left out), the link to
 * that next node is widened by subspace_expand! (src/ttn/update_site_ttn.jl:75-109; at most
 * max_expand_dim, padding scaled to noise * |tensor|), and expand_numiter updates alternate
 * between the two nodes with maxdims maxdim + max_expand_dim, maxdim + expand_dim, ...,
 * maxdim and cutoff p->cutoff (truncating SVD moves).  The padding is a counter-based stream
 * keyed by `seed`, the instance and the expansion count (the reference draws it from Julia's
 * RNG).  The group's arena grows when the widened tensors need room. */
int tn_ttn_envs_fullsweep_expand(int count, tn_ttn_env* const* envs, int npath,
                                 const int32_t* path, int central, const tn_update_params* p,
                                 int expand_dim, int max_expand_dim, int expand_numiter,
                                 uint64_t seed, tn_sweep_result* res);

/* ---- allocation-free block singular values ----------------------------------------
 * No counterpart in the reference.  For callers that cannot let the library allocate
 * device memory (a host framework that owns all device memory through its own pool, a
 * process with a fixed memory budget): singular values of nblocks dense column-major
 * blocks that already live on the device (concatenated at `blocks`, dimensions in the
 * host arrays rows/cols), sorted descending per block into the device buffer `svals`
 * (sum of min(rows, cols) doubles), computed on `stream` (a cudaStream_t, NULL = legacy
 * default stream) with the same one-CTA-per-block kernel as the small blocks of
 * tn_svd_truncate.  Allocates nothing: its work space is a file-scope device array of
 * about 16.3 MiB that every GPU on which the library is loaded holds until the process
 * exits.  Limits: sum rows*cols <= 524288, sum min(rows, cols) <= 65536, nblocks <= 1024,
 * min(rows, cols) <= 3000 per block; larger requests return TN_E_INVALID.  Set-up: the
 * first call on a device looks up the work array's address with that device current and
 * keeps it, so make that first call before any stream capture; after a cudaDeviceReset of
 * the device the kept address is stale and the entry point must not be used on it again.
 * The caller's current device is unchanged on return.  All calls share the work array:
 * calls that overlap on the GPU race and must be serialised by the caller.  The call is
 * asynchronous; synchronise `stream` before reading svals. */
int tn_block_svals_noalloc(int device, const double* blocks, int nblocks, const int32_t* rows,
                           const int32_t* cols, double* svals, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TENNET_H */
