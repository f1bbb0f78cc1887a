// Allocation-free block singular values.
//
// Some callers cannot let this library allocate device memory: a host framework that owns
// the whole device memory through its own pool, or a solver embedded in a process whose
// memory budget is fixed up front.  For them tn_block_svals_noalloc computes the singular
// values of a list of dense blocks that already live on the device, using work space held
// in a file-scope __device__ array instead of cudaMalloc.  The array is part of the loaded
// module, so every GPU on which the library is loaded keeps it until the process exits.
//
// Limits (checked on entry, a larger request is rejected with TN_E_INVALID):
//   sum over blocks of rows*cols <= 524288 doubles;
//   sum over blocks of min(rows, cols) <= 65536;
//   number of blocks <= 1024; min(rows, cols) <= 3000 per block.
// Footprint: 4 x 4 MiB work matrices + 256 KiB permutation + descriptors, about 16.3 MiB.
//
// All calls share the one array and it keeps the previous call's contents; nothing in it
// has to start at zero (every word the kernel reads it has written earlier in the same
// call).  Two calls whose work overlaps on the GPU (different streams, or different host
// threads without ordering) race on the array: the caller must serialise them.
// The first call on a device looks up the array's device address (cudaGetSymbolAddress)
// with that device current and caches it; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/tennet.h"
#include "tn_internal.h"

namespace tn {
namespace {

constexpr int64_t MAX_ELEMS = 524288;
constexpr int MAX_SVALS = 65536;
constexpr int MAX_BLOCKS = 1024;
constexpr int MAX_N = 3000;

struct NoAllocScratch {
    double X[MAX_ELEMS];   // QR / reflector work matrix (m x n per block)
    double W[MAX_ELEMS];   // Q V
    double V[MAX_ELEMS];   // n x n rotations / P Y   (sum n^2 <= sum m n)
    double P[MAX_ELEMS];   // n x n Jacobi scratch
    int perm[MAX_SVALS];
    SvdBlockDesc desc[MAX_BLOCKS];
};

static __device__ __align__(256) NoAllocScratch g_scratch;

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
NoAllocScratch* g_addr[MAX_DEVICES] = {nullptr};

NoAllocScratch* scratch_for(int device) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        TN_CUDA(cudaGetSymbolAddress(&p, g_scratch));
        g_addr[device] = static_cast<NoAllocScratch*>(p);
    }
    return g_addr[device];
}

thread_local SvdBlockDesc t_desc[MAX_BLOCKS];
thread_local std::string t_err;

}  // namespace
}  // namespace tn

extern "C" int tn_block_svals_noalloc(int device, const double* blocks, int nblocks,
                                      const int32_t* rows, const int32_t* cols, double* svals,
                                      void* stream) {
    using namespace tn;
    try {
        if (!blocks || !rows || !cols || !svals) throw Error(TN_E_INVALID, "null argument");
        if (nblocks < 1 || nblocks > MAX_BLOCKS)
            throw Error(TN_E_INVALID, "tn_block_svals_noalloc: number of blocks must be in [1, 1024]");
        if (device < 0 || device >= MAX_DEVICES) throw Error(TN_E_INVALID, "device out of range");
        int64_t elems = 0, nsv = 0;
        int maxn = 1;
        for (int b = 0; b < nblocks; ++b) {
            if (rows[b] < 1 || cols[b] < 1) throw Error(TN_E_INVALID, "block dimensions must be >= 1");
            SvdBlockDesc& d = t_desc[b];
            d = SvdBlockDesc{};
            d.src_off = elems;
            d.rows = rows[b];
            d.cols = cols[b];
            d.trans = rows[b] < cols[b] ? 1 : 0;
            d.m = rows[b] > cols[b] ? rows[b] : cols[b];
            d.n = rows[b] < cols[b] ? rows[b] : cols[b];
            if (d.n > MAX_N)
                throw Error(TN_E_INVALID, "tn_block_svals_noalloc: min(rows, cols) above 3000");
            d.x_off = elems;   // m n per block, packed like the input
            d.v_off = 0;       // set below
            d.s_off = nsv;
            elems += int64_t(rows[b]) * cols[b];
            nsv += d.n;
            if (d.n > maxn) maxn = d.n;
        }
        if (elems > MAX_ELEMS)
            throw Error(TN_E_INVALID, "tn_block_svals_noalloc: sum of rows*cols above 524288");
        if (nsv > MAX_SVALS)
            throw Error(TN_E_INVALID, "tn_block_svals_noalloc: sum of min(rows, cols) above 65536");
        int64_t vo = 0;
        for (int b = 0; b < nblocks; ++b) {
            t_desc[b].v_off = vo;
            vo += int64_t(t_desc[b].n) * t_desc[b].n;  // <= sum m n
        }
        TN_CUDA(cudaSetDevice(device));
        NoAllocScratch* sc = scratch_for(device);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        TN_CUDA(cudaMemcpyAsync(sc->desc, t_desc, size_t(nblocks) * sizeof(SvdBlockDesc),
                                cudaMemcpyHostToDevice, st));
        // the kernel writes the sorted singular values straight into the caller's buffer
        launch_svd_jacobi(sc->desc, nblocks, maxn, blocks, sc->X, sc->W, sc->V, sc->P, svals,
                          sc->perm, nullptr, st);
        return TN_OK;
    } catch (const Error& e) {
        t_err = e.what();
        set_last_error(t_err.c_str());
        return e.code;
    } catch (const std::exception& e) {
        t_err = e.what();
        set_last_error(t_err.c_str());
        return TN_E_INVALID;
    }
}
