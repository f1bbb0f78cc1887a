// Internal declarations of libtennet_cuda.so: block layouts of U(1) tensors, contraction
// plans, device buffers and kernel launchers.  Host code is C++17; kernels are CUDA for
// sm_103a.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace tn {

// ------------------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void set_last_error(const char* msg);  // message returned by tn_last_error() on this thread
#define TN_CUDA(x)                                                          \
    do {                                                                    \
        cudaError_t _e = (x);                                               \
        if (_e != cudaSuccess) ::tn::cuda_fail(_e, #x, __FILE__, __LINE__); \
    } while (0)
#define TN_REQUIRE(cond, msg)                                     \
    do {                                                          \
        if (!(cond)) throw ::tn::Error(-1, std::string(msg));     \
    } while (0)

// ------------------------------------------------------------------------------------
// device buffers (stream-ordered pool allocation)
// ------------------------------------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p; bytes = o.bytes; stream = o.stream;
            o.p = nullptr; o.bytes = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t nbytes, cudaStream_t s);     // reallocates only when growing
    void release();
    double* d() const { return static_cast<double*>(p); }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// ------------------------------------------------------------------------------------
// links and block layouts
// ------------------------------------------------------------------------------------
struct Link {
    std::vector<int> q, dim;  // sectors sorted by q ascending
    int nsec() const { return (int)q.size(); }
    int find(int charge) const;  // sector index or -1
    int total() const;
    int maxdim() const;
    std::vector<int> offsets() const;  // basis offset of each sector
};

enum Layout { LG = 0, RG = 1 };

// Site tensor A[l, s, r] (charge rule q_r = q_l + q_s).
//  LG (left-grouped): one block per right sector r; rows = (s, l) slabs, s-major,
//      l = r - q_s; cols = D_r.  A left isometry is an LG tensor with orthonormal columns.
//  RG (right-grouped): one block per left sector l; rows = D_l; cols = (s, r) slabs,
//      r = l + q_s.  A right isometry is an RG tensor with orthonormal rows.
// Blocks are column-major and packed back to back.
struct SiteLayout {
    Layout layout = RG;
    int d = 0;
    std::vector<int> rows, cols;
    std::vector<int64_t> off;
    std::vector<int> sub;     // [nblk*d] slab offset (row for LG, column for RG), -1 absent
    std::vector<int> subsec;  // [nblk*d] sector of the other link, -1 absent
    int64_t size = 0;
    int nblk() const { return (int)rows.size(); }
};
SiteLayout make_site_layout(Layout lay, const Link& left, const Link& right,
                            const std::vector<int>& pq);

// Two-site tensor phi[l, s1, s2, r] grouped by the middle charge m = q_l + q_s1 = q_r - q_s2:
// block m has rows (s1, l) slabs (s1-major) and cols (s2, r) slabs (s2-major).  The rows of
// block m are the LG rows of a left tensor with right sector m; the columns are the RG
// columns of a right tensor with left sector m.  The same layout with one physical leg
// (nsite = 1, the one-site tensor (l, s, r) grouped by m = q_r) is not used by the engine.
struct PhiLayout {
    int d = 0;
    std::vector<int> m, rows, cols;
    std::vector<int64_t> off;
    std::vector<int> rsub, rsec;  // [nblk*d] row offset / left sector of slab s1
    std::vector<int> csub, csec;  // [nblk*d] col offset / right sector of slab s2
    int64_t size = 0;
    int nblk() const { return (int)m.size(); }
    int find(int charge) const;
};
PhiLayout make_phi_layout(const Link& left, const Link& right, const std::vector<int>& pq);

// Environment E[x', a, x] on one link: block (a, ket sector x) of size D_{x'} x D_x with
// the bra sector x' = x + delta_a.
struct EnvLayout {
    int w = 0, nsec = 0;
    std::vector<int64_t> off;  // [w*nsec], -1 absent
    std::vector<int> bra;      // [w*nsec]
    int64_t size = 0;
};
EnvLayout make_env_layout(const Link& link, const std::vector<int>& delta);

// ------------------------------------------------------------------------------------
// contraction plans (device-visible PODs)
// ------------------------------------------------------------------------------------
enum BufSlot {
    S_L = 0,   // left environment
    S_R = 1,   // right environment
    S_X = 2,   // input vector / site tensor
    S_Y = 3,   // output
    S_T1 = 4,  // intermediates
    S_T2 = 5,
    S_A = 6,   // second site tensor
    S_B = 7,
    S_IM = 8,  // slot s + S_IM: the imaginary plane of slot s's complex buffer
    NSLOT = 16
};
struct Bases {
    double* p[NSLOT];
};

// C[task] = sum over its segments of sgn * op(A) * op(B); op = transpose when t* = 1.
struct Seg {
    int64_t aoff, boff;
    int32_t abuf, bbuf, lda, ldb, k, ta, tb, sgn;
};
struct Task {
    int64_t coff;
    int32_t cbuf, m, n, ldc, seg0, nseg;
    int32_t accum;  // 1: C += result (tasks of one launch must not overlap), 0: C = result
};
struct Tile {
    int32_t task, m0, n0;
};
// dst sub-block = sum_t coef_t * src_t (all rows x cols, column-major)
struct CombOut {
    int64_t doff;
    int32_t dbuf, ldd, rows, cols, t0, nt;
};
struct CombTerm {
    int64_t soff;
    int32_t sbuf, lds;
    double coef;
};
struct CombTile {
    int32_t out, r0, c0;
};

struct GemmPlan {
    std::vector<Seg> segs;
    std::vector<Task> tasks;
    std::vector<Tile> tiles;
    double flops = 0;
    DevBuf dsegs, dtasks, dtiles;
    void add_task(int cbuf, int64_t coff, int m, int n, int ldc, int accum = 0);
    void add_seg(int abuf, int64_t aoff, int lda, int ta, int bbuf, int64_t boff, int ldb,
                 int tb, int k, int sgn = 1);
    void finalize(cudaStream_t s);  // builds tiles, uploads
};
struct CombPlan {
    std::vector<CombOut> outs;
    std::vector<CombTerm> terms;
    std::vector<CombTile> tiles;
    double flops = 0;
    DevBuf douts, dterms, dtiles;
    void finalize(cudaStream_t s);
};

// Complex forms of real plans over planar complex buffers (real plane in slot s, imaginary
// plane in slot s + S_IM).  Every task C = sum op(A) op(B) becomes two, C_re and C_im, of
// two segments per original one; operands read from a slot in conj_mask (bit s) enter
// conjugated.  A combine plan (real coefficients) is applied to both planes.  Unfinalized.
GemmPlan complex_plan(const GemmPlan& g, unsigned conj_mask);
CombPlan complex_comb(const CombPlan& c);

// split-precision (bf16 slice) GEMM descriptors.  A packed operand is a list of tiles
// (row tile, k tile, slice) of the canonical K-major SWIZZLE_128B layout.
struct KTileSrc {        // one k tile of one task's operand: element (r, k) at
    int64_t off;         // p[buf][off + r * sr + k * sk]
    int32_t buf, sr, sk, kvalid;
};
struct PackJob {         // one row tile of one task's operand
    int64_t out_off;     // byte offset of (this row tile, k tile 0, slice 0)
    int32_t kt0, nkt, rows, row0, eoff, pad;
};
struct SplitTask {
    int64_t coff, a_off, b_off;
    int32_t cbuf, m, n, ldc, nkt, ea_off, eb_off, accum;
};
struct SplitItem {
    int32_t task, mt, nt, pad;
};
struct SplitPlan {
    std::vector<SplitTask> tasks;
    std::vector<SplitItem> items;
    std::vector<PackJob> ajobs, bjobs;
    std::vector<KTileSrc> aks, bks;
    int64_t abytes = 0, bbytes = 0, ea_n = 0, eb_n = 0;
    int slices = 0;
    bool a_static = false, b_static = false, a_packed = false, b_packed = false;
    DevBuf dtasks, ditems, dajobs, dbjobs, daks, dbks, apack, bpack, ea, eb;
    // pack buffers used by the launches: the owned buffers above, or caller-provided
    // scratch (make_split with own_packs = false) of abytes / bbytes / 4 ea_n / 4 eb_n bytes
    uint8_t *ap = nullptr, *bp = nullptr;
    int *eap = nullptr, *ebp = nullptr;
    int a_maxnkt = 0, b_maxnkt = 0;   // longest k (in tiles) of a pack job
    DevBuf amax, bmax;                // row maxima scratch of the k-split pack
};
int split_tile_bytes_a();
int split_tile_bytes_b();
int split_tile_rows_a();
int split_tile_rows_b();
int split_ktile();
// max_nkt: the largest k-tile count of a job; operands with long k are packed by the k-split
// kernels, which need gmax (nrows 64-bit words of scratch, the exponent count of the operand)
void launch_split_pack(const PackJob* jobs, int njobs, const KTileSrc* ksrc, const Bases& b,
                       uint8_t* out, int* expo, int slices, int tile_rows, cudaStream_t s,
                       int max_nkt = 0, unsigned long long* gmax = nullptr, int64_t nrows = 0);
void launch_split_gemm(const SplitItem* items, int nitems, const SplitTask* tasks,
                       const uint8_t* apack, const uint8_t* bpack, const int* ea, const int* eb,
                       const Bases& b, int slices, int* err, int nsm, cudaStream_t s);

constexpr int GEMM_BM = 64, GEMM_BN = 64;
constexpr int COMB_TR = 32, COMB_TC = 32;

// ------------------------------------------------------------------------------------
// kernel launchers (kernels_*.cu)
// ------------------------------------------------------------------------------------
void launch_gemm_f64(const GemmPlan& p, const Bases& b, cudaStream_t s);
// number of kernel launches issued by this library since load (all kernels)
int64_t launch_count();
void count_launch(int n = 1);
// algorithmic HBM bytes moved by the Krylov vector kernels since load (each vector element
// read or written once per launch)
int64_t krylov_bytes();
void count_krylov_bytes(int64_t b);
void launch_combine(const CombPlan& p, const Bases& b, cudaStream_t s);

// Krylov vector kernels.  Partial sums go to `part` (>= K * nparts doubles) and the
// finalized results to `out` (K doubles), all on the device.
int blas_nparts();
void launch_multi_dot(const double* const* V, int K, const double* w, int64_t n,
                      double* part, double* out, cudaStream_t s);
void launch_multi_axpy(double* w, const double* const* V, int K, const double* h,
                       double sign, int64_t n, cudaStream_t s);
// Fused Gram-Schmidt pass (see kernels_f64.cu): optional w += sign * V hin, optional dots
// V^T w into out[0..K), optional |w|^2 into out[K or 0]; one launch, deterministic.
void launch_gs_pass(const double* const* V, int K, double* w, const double* hin, double sign,
                    int64_t n, bool dots, bool norm, double* part, double* out, unsigned* ticket,
                    cudaStream_t s);
void launch_scale_into(double* dst, const double* src, const double* denom_sq_or_null,
                       double host_scale, int64_t n, cudaStream_t s);
void launch_lincomb(double* dst, const double* const* V, int K, const double* coef,
                    int64_t n, cudaStream_t s);

// sum of x (.) y over one rows x cols block pair (x, y column-major with their leading
// dimensions), one result per pair, deterministic
struct BlockDot {
    const double* x;
    const double* y;
    int32_t ldx, ldy, rows, cols;
};
void launch_block_dots(const BlockDot* d, int n, double* out, cudaStream_t s);

// Block SVD: for each block b with rows x cols matrix at src + off[b], compute its SVD by
// one-sided Jacobi on the m x n work matrix (m >= n; the transpose when rows < cols).
struct SvdBlockDesc {
    int64_t src_off;   // offset of the block in the source buffer
    int64_t x_off;     // offset of the work matrix X (m x n, m >= n)
    int64_t v_off;     // offset of V (n x n)
    int64_t s_off;     // offset of the singular values (n) and permutation
    int32_t rows, cols, m, n, trans, pad;
};
void launch_svd_jacobi(const SvdBlockDesc* d, int nb, int max_n, const double* src, double* X,
                       double* W, double* V, double* P, double* S, int* perm, int* sweeps_out,
                       cudaStream_t s);

// ------------------------------------------------------------------------------------
// multi-SM SVD of large charge blocks (kernels_bsvd.cu, host driver bsvd.cpp):
// blocked Householder QR (one-CTA panels, grouped-GEMM trailing updates), one-sided Jacobi
// on R^T by rounds of column-block pairs spread over many CTAs (FP32 presolve, Newton-Schulz
// re-orthonormalisation, double-float polish), Q applied by grouped GEMMs.  All offsets are
// in doubles from the start of one work arena.
// ------------------------------------------------------------------------------------
struct BsvdBlk {
    int64_t src_off;          // block in the source buffer
    int64_t xq;               // QR work matrix, m x n (ld m)
    int64_t vp;               // explicit reflectors of panel p at vp + p * m * pw, (m - p0) x w
    int64_t tm;               // panel p: -T^T at tm + p * 2 pw^2, -T after it (w x w, ld w)
    int64_t rt64, v64, g64, v64b, y64;  // n x n FP64
    int64_t r32, v32;         // n x n FP32 (float arrays)
    int64_t ydf, vdf;         // n x n double-float
    int64_t scl;              // one double: the block is worked on scaled by 2^-e, e stored here
    int64_t cn;               // n doubles: norms of the work matrix's columns
    int64_t piv;              // n doubles holding 2 n ints: the column order (work column k is
                              // source column piv[k]) and its inverse at piv + n
    int64_t x_off, v_off, s_off;  // outputs: QV (m x n) in the QV buffer, PY (n x n), S / perm
    int32_t rows, cols, trans, m, n, pad;
};
struct BjDesc {               // one matrix of the cooperative one-sided Jacobi
    void* X;                  // n x n, column-major (float or double-float)
    void* V;                  // n x n rotations
    int32_t n, nb, cta0, ncta;
    unsigned* bar;            // barrier counter of the CTA group
    int* flags;               // [0..3) rotated flags, [3..6) largest rotated cosine (float bits)
    int* sweeps;              // sweeps run
};
// panel width for a largest row count m (the panel lives in shared memory)
int bsvd_panel_width(int mmax);
// largest n the Jacobi kernels accept
int bsvd_max_n();
// scales each block by a power of two to a largest entry in [1/2, 1) while copying it (or
// its transpose) into the QR work matrix, its columns ordered by decreasing norm
void launch_bsvd_gather(const BsvdBlk* d, int nb, int64_t mnmax, const double* src, double* ar,
                        cudaStream_t s);
void launch_bsvd_panel(const BsvdBlk* d, int nb, int p0, int pw, int rmax, double* ar,
                       cudaStream_t s);
// op 0: R^T (FP32 and FP64) and V32 = I; 1: V64 = V32; 2: G <- 1.5 I - 0.5 G (g64);
// 3: Ydf, Vdf from y64, v64
void launch_bsvd_elem(const BsvdBlk* d, int nb, int64_t nnmax, int op, double* ar, cudaStream_t s);
// cooperative Jacobi sweeps (precision 0: FP32 presolve, 1: double-float polish); returns
// the CTAs used per matrix in descs (cta0 / ncta filled by the caller)
void launch_bsvd_jacobi(const BjDesc* d, int nd, int nctas, int maxn, int precision, int* err,
                        cudaStream_t s);
int bsvd_jacobi_capacity(int maxn, int precision);
// columns per block of the Jacobi kernel for the largest n (precision 0 FP32, 1 double-float)
int bsvd_jacobi_block(int maxn, int precision);
// singular values (sorted, with the permutation), PY = P Y (rows back in the source column
// order) and QV = [V; 0]
void launch_bsvd_finish(const BsvdBlk* d, int nb, double* ar, double* qv, double* py, double* S,
                        int* perm, cudaStream_t s);

// extraction of truncated factors into site tensors
struct ExtractDesc {
    int64_t x_off, v_off, s_off;
    int64_t left_off, right_off;  // destination block offsets
    int32_t rows, cols, n, trans, k, pad;
};
void launch_svd_extract(const ExtractDesc* d, int nb, const double* QV, const double* PY,
                        const double* S, const int* perm, double* left, double* right, int ortho,
                        double inv_norm, cudaStream_t s);
// The same for complex blocks A (rows x cols) whose SVD was taken of the realified
// [[Re A, -Im A], [Im A, Re A]]: kept complex value c is the realified pair (2c, 2c + 1), its
// vectors the realified column of the first of them read as [re; im]; left and right are
// planar (imaginary planes at left + lplane, right + rplane), the right tensor gets V^H.
void launch_svd_extract_complex(const ExtractDesc* d, int nb, const double* QV, const double* PY,
                                const double* S, const int* perm, double* left, int64_t lplane,
                                double* right, int64_t rplane, int ortho, double inv_norm,
                                cudaStream_t s);

}  // namespace tn
