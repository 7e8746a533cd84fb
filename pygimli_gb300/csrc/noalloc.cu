// Allocation-free variant of the multi-right-hand-side CSR product with
// column dot products (ertgb_csr_spmm_dot).
//
// Who needs it: callers that cannot allocate device memory at call time --
// a host framework that owns the whole device-memory budget through its own
// pooling allocator and forbids other allocations, or a time-critical loop
// that must not allocate after start-up because cudaMalloc/cudaFree can
// synchronise the device and can fail once memory is fragmented.  Such a
// caller allocates its inputs and outputs once and then calls this entry
// point, which uses only the fixed scratch array below.
//
// Scratch: the block partials of the column dots, a file-scope device array
// of kRows x kMaxLd doubles (2 MiB).  Every GPU that loads the library holds
// it until the process exits.  All calls share it and it keeps the last
// call's contents; the kernel writes every partial before it reads any, so
// nothing has to be cleared.  Calls that overlap on the GPU (on different
// streams, or from several threads) race on this array and must be ordered
// by the caller.
//
// Set-up: host code cannot use the array's name as a device address (in
// host code it is a host-side stand-in), so the first call on each device
// looks up the array's device address with cudaGetSymbolAddress, with that
// device current, and caches it.  That first call per device should come
// before any stream capture.  The cached address is that of the device's
// primary context: a device reset (cudaDeviceReset) or a torn-down primary
// context would leave it stale, so neither may happen while the library is
// loaded.
#include <mutex>
#include <vector>

#include "ertgb_internal.cuh"

namespace {

constexpr int kRows = 256;       // block partial rows (row blocks of the kernel)
constexpr int64_t kMaxLd = 1024; // maximum columns (right-hand sides, padded to 32)

static __device__ __align__(256) double g_spmm_partials[kRows * kMaxLd];

std::mutex g_mutex;
std::vector<double *> g_address;  // per device: device address of g_spmm_partials

double *scratch_on_current_device() {
    int dev = 0;
    ERTGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_mutex);
    if ((int)g_address.size() <= dev) g_address.resize(dev + 1, nullptr);
    if (!g_address[dev]) {
        double *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_spmm_partials);
        if (e != cudaSuccess || !p)
            throw ertgb::Error(ERTGB_CUDA_ERROR,
                               std::string("cudaGetSymbolAddress of the fixed scratch: ") + cudaGetErrorString(e));
        g_address[dev] = p;
    }
    return g_address[dev];
}

}  // namespace

extern "C" int ertgb_csr_spmm_dot_noalloc(int64_t n, int64_t nnz, const int32_t *rowptr, const int32_t *colidx,
                                          const double *vals, int n_k, int n_per_k, int64_t ld, const double *X,
                                          double *Y, double *dots, void *stream) {
    try {
        ertgb::check_spmm_args(n, nnz, rowptr, colidx, vals, n_k, n_per_k, ld, X, Y, dots);
        if (ld > kMaxLd)
            throw ertgb::Error(ERTGB_BAD_INPUT, "ld = " + std::to_string(ld) +
                                                    " exceeds the fixed scratch of the allocation-free entry point "
                                                    "(at most 1024 columns)");
        double *part = scratch_on_current_device();
        const int NB = ertgb::spmm_partial_rows(n, kRows);
        ertgb::spmm_dot_launch(n, nnz, rowptr, colidx, vals, n_k, n_per_k, ld, X, Y, dots, part, NB,
                               (cudaStream_t)stream);
        ertgb::set_free_error("");
        return ERTGB_OK;
    } catch (ertgb::Error &e) {
        ertgb::set_free_error(e.what());
        return e.code;
    } catch (std::exception &e) {
        ertgb::set_free_error(e.what());
        return ERTGB_BAD_INPUT;
    }
}
