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
// has to start at zero (every word the kernels read they have written earlier in the same
// call).  Two calls whose work overlaps on the GPU (different streams, or different host
// threads without ordering) race on the array: the caller must serialise them.
// Set-up: the first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current and keeps it for the process; make that
// first call before any stream capture.  A cudaDeviceReset of the device discards the
// module and with it the address: the entry point must not be called on that device again.
// The block dimensions reach the device as kernel arguments (no host staging buffer is
// read after the call returns), and the caller's current device is restored on return.
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

// Block dimensions passed by value (8 KiB of kernel arguments).
struct BlockDims {
    int32_t rows[MAX_BLOCKS];
    int32_t cols[MAX_BLOCKS];
    int32_t nblocks;
};

// Writes the SVD descriptors of the blocks into the scratch array: inputs packed back to
// back, work matrices packed like the inputs, n x n matrices packed back to back.
__global__ void noalloc_desc_kernel(const BlockDims dims, NoAllocScratch* sc) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t elems = 0, vo = 0, so = 0;
    for (int b = 0; b < dims.nblocks; ++b) {
        const int r = dims.rows[b], c = dims.cols[b];
        SvdBlockDesc d{};
        d.src_off = elems;
        d.x_off = elems;
        d.v_off = vo;
        d.s_off = so;
        d.rows = r;
        d.cols = c;
        d.trans = r < c ? 1 : 0;
        d.m = r > c ? r : c;
        d.n = r < c ? r : c;
        sc->desc[b] = d;
        elems += int64_t(r) * c;
        vo += int64_t(d.n) * d.n;
        so += d.n;
    }
}

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
NoAllocScratch* g_addr[MAX_DEVICES] = {nullptr};

// set-up, once per device, with that device current
NoAllocScratch* scratch_for(int device) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        TN_CUDA(cudaGetSymbolAddress(&p, g_scratch));
        g_addr[device] = static_cast<NoAllocScratch*>(p);
    }
    return g_addr[device];
}

// makes `device` current for the lifetime of the guard and restores the caller's device
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int device) {
        TN_CUDA(cudaGetDevice(&prev));
        if (prev != device) TN_CUDA(cudaSetDevice(device));
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

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
        int ndev = 0;
        TN_CUDA(cudaGetDeviceCount(&ndev));
        if (device >= ndev) throw Error(TN_E_INVALID, "device out of range");
        BlockDims dims;
        dims.nblocks = nblocks;
        int64_t elems = 0, nsv = 0;
        int maxn = 1;
        for (int b = 0; b < nblocks; ++b) {
            if (rows[b] < 1 || cols[b] < 1) throw Error(TN_E_INVALID, "block dimensions must be >= 1");
            const int n = rows[b] < cols[b] ? rows[b] : cols[b];
            if (n > MAX_N)
                throw Error(TN_E_INVALID, "tn_block_svals_noalloc: min(rows, cols) above 3000");
            dims.rows[b] = rows[b];
            dims.cols[b] = cols[b];
            elems += int64_t(rows[b]) * cols[b];
            nsv += n;
            if (n > maxn) maxn = n;
        }
        if (elems > MAX_ELEMS)
            throw Error(TN_E_INVALID, "tn_block_svals_noalloc: sum of rows*cols above 524288");
        if (nsv > MAX_SVALS)
            throw Error(TN_E_INVALID, "tn_block_svals_noalloc: sum of min(rows, cols) above 65536");
        DeviceGuard guard(device);
        NoAllocScratch* sc = scratch_for(device);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        noalloc_desc_kernel<<<1, 32, 0, st>>>(dims, sc);
        TN_CUDA(cudaGetLastError());
        count_launch();
        // the SVD kernel writes the sorted singular values straight into the caller's buffer
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
