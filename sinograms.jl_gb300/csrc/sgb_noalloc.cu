// sgb_noalloc.cu -- project_bdd for callers that cannot allocate device memory.
//
// sgb_bdd_project allocates its per-view tables (and staging buffers) with cudaMalloc.
// Some callers cannot allow that: reconstruction services that forbid device
// allocation after start-up so every request has the same latency and memory
// footprint, and host programs or plugin hosts whose device memory is entirely owned by
// another allocator (a framework's caching pool with a fixed budget), where a
// cudaMalloc from a library would fail or fragment that pool.  sgb_bdd_project_noalloc
// takes device pointers for its input and output and keeps its scratch in the
// file-scope array below, which every GPU that loads this library holds until the
// process exits.
//
// The first call on a device resolves the array's device address (cudaGetSymbolAddress
// with that device current); make that first call before any stream capture begins.  The
// address is kept for the life of the process, so the entry point must not be used on a
// device after cudaDeviceReset (which reloads the module).  All calls on a device share
// the one array and it keeps the last call's contents, so calls whose GPU work overlaps
// (different streams, or different host threads) race on it: serialise them on one
// stream.
#include <mutex>

#include "sgb_common.cuh"
#include "sgb_kernels.cuh"

namespace sgb {

namespace {

// Scratch of the no-allocation entry point: the view angles plus the per-view tables of
// the distance-driven projector (see bdd_project_scratch).  16 MiB per device.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  In host code the array's
// name is only a host-side stand-in, so the address is resolved once per device with
// cudaGetSymbolAddress while that device is current.
int scratch_on_current_device(void **out) {
    int dev = -1;
    SGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("bdd_project_noalloc: device index %d is out of range", dev);
        return SGB_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("bdd_project_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return SGB_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return SGB_OK;
}

}  // namespace

}  // namespace sgb

using namespace sgb;

extern "C" int sgb_bdd_project_noalloc(const float *phantom, int nPix, int nDet, int na, const double *angle,
                                       double DSD, double DS0, double pSize, double dSize, float *sino,
                                       void *stream) {
    SGB_REQUIRE(phantom && sino && angle, "bdd_project_noalloc: null argument");
    SGB_REQUIRE(nPix > 0 && nDet > 0 && na > 0, "bdd_project_noalloc: sizes must be positive");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    BddArgs G{nPix, nDet, na, nullptr, DSD, DS0, pSize, dSize};
    const size_t angle_bytes = ((size_t)na * sizeof(double) + 255) / 256 * 256;
    const size_t need = angle_bytes + bdd_project_scratch(G);
    if (need > kNoAllocScratchBytes) {
        set_error("bdd_project_noalloc: na=%d nDet=%d needs %zu bytes of scratch, more than the %zu bytes this "
                  "entry point keeps per device; use sgb_bdd_project",
                  na, nDet, need, kNoAllocScratchBytes);
        return SGB_ERR_ARG;
    }
    void *base = nullptr;
    SGB_TRY(scratch_on_current_device(&base));
    double *angle_dev = static_cast<double *>(base);
    // Copy of the host angle vector into the scratch, ordered on `stream`.  From pageable
    // memory the copy is staged before the call returns, so the host array may be reused
    // then; a page-locked array must stay unchanged until the stream has reached this copy.
    // Every other scratch byte is written by the set-up kernel before it is read, and the
    // output is cleared by the launch itself.
    SGB_CUDA(cudaMemcpyAsync(angle_dev, angle, (size_t)na * sizeof(double), cudaMemcpyHostToDevice, st));
    G.angle = angle_dev;
    return launch_bdd_project(G, phantom, sino, static_cast<char *>(base) + angle_bytes, st);
}
