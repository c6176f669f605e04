// k_noalloc.cu — ftx_scan_noalloc: the prefix scan of ft_array_scan /
// ft_array_prescan without any device allocation.
//
// Who needs it: callers that cannot call cudaMalloc — for example a host
// framework whose caching allocator already holds the GPU's memory and hands
// out only its own buffers, or a latency-bound caller that must not trigger
// the implicit synchronisation cudaMalloc / cudaFree can cause.  They pass
// the points (their own device buffer, in this library's plane layout) and a
// stream; the scan's scratch (per-thread and per-chunk partial sums) comes
// from a fixed array compiled into this library instead of the allocator.
//
// Limits and sharing:
//  * at most FT_NOALLOC_SCAN_MAX_POINTS points per call (FT_ERR_BAD_SIZE
//    beyond it); the array is FT_NOALLOC_SCAN_SCRATCH_BYTES (about 11 MB) and
//    is resident on every GPU that loads the library until the process exits;
//  * every call uses the same array and leaves its partial sums there; each
//    launch writes all scratch it later reads, so nothing must start at zero;
//  * calls whose work overlaps on the GPU (different streams, or different
//    host threads) race on the array and give wrong results: serialise them.
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.  The address is kept for the life of the
//    process: after a cudaDeviceReset the module is loaded again and the
//    array may lie elsewhere, so calling this entry point on a device that
//    was reset is not supported.
#include <mutex>

#include "internal.h"
#include "../../include/ftcrypto.h"
#include "../../include/ftcrypto_gb300.h"

// the scan's scratch at the maximum size (ft::scan_scratch_points)
static constexpr size_t FT_NOALLOC_SCAN_SCRATCH_BYTES =
    ((ft::scan_scratch_points(FT_NOALLOC_SCAN_MAX_POINTS) * 128 + 256 + 255) / 256) * 256;

static __device__ __align__(256) unsigned char g_noalloc_scan_scratch[FT_NOALLOC_SCAN_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices];

// device address of the scratch array on the current device, looked up once
// per device and kept (a cudaDeviceReset afterwards is not supported)
cudaError_t scratch_address(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

} // namespace

extern "C" ft_error ftx_scan_noalloc(void *d_planes, size_t stride, size_t n, int exclusive, void *stream)
{
    if (n > FT_NOALLOC_SCAN_MAX_POINTS) return FT_ERR_BAD_SIZE;
    if (n > stride) return FT_ERR_SIZE_MISMATCH;
    if (n == 0) return FT_ERR_NO_ERROR;
    if (ft::scan_scratch_bytes(n) > FT_NOALLOC_SCAN_SCRATCH_BYTES) return FT_ERR_INTERNAL_LIBRARY_ERROR;
    void *scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e == cudaSuccess)
        e = ft::scan(ft::View{(uint4 *)d_planes, stride}, n, exclusive ? 1 : 0, scratch, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return FT_ERR_INTERNAL_LIBRARY_ERROR;
    }
    return FT_ERR_NO_ERROR;
}
