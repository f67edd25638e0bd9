// fg_energy_noalloc: the energy reduction of fg_energy for callers that cannot allocate
// device memory at the time of the call.
//
// Who needs it: code that runs where a cudaMalloc is not allowed or not wanted, e.g. a
// host framework that hands out all device memory from its own pool and forbids driver
// allocations after start-up, or a loop that must not trigger the implicit device
// synchronisation an allocation can cause. Such a caller creates its context once (that
// allocates) and afterwards reads energies through this entry point, which performs no
// cudaMalloc, cudaFree or allocating library call.
//
// The per-block partial sums of the reduction live in the file-scope array below instead
// of in the context: FG_NOALLOC_PARTIALS doubles (64 KiB), enough for 7 sums over up to
// 1170 reduction blocks (a context uses at most 4 blocks per SM). A context that would
// need more is rejected with FG_EINVAL and a message; nothing is launched then.
//
// The array is shared by every call in the process and keeps the last call's contents.
// Every slot a call reads was written by the same call first, so nothing has to be cleared
// beforehand. Calls whose GPU work overlaps (two host threads, or two contexts on different
// streams) race on the array: issue them one after the other.
//
// In host code the array's name is only a host-side stand-in, not a device address. Its
// device address is looked up once per device with cudaGetSymbolAddress, by the first call
// for a context on that device (the call makes the context's device current while it runs
// and restores the caller's current device afterwards); make that first call before any
// stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "fg_internal.h"

#define FG_NOALLOC_PARTIALS 8192

namespace fg {
cudaError_t launch_energy_into(Ctx &c, const double Hext[3], double *partial);
}

static __device__ __align__(256) double g_noalloc_partials[FG_NOALLOC_PARTIALS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_lock;
double *g_dev_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the context's device (looked up once per device,
// with that device current: the caller's current device may be another one).
int scratch_address(fg::Ctx &c, double **out) {
    if (c.device < 0 || c.device >= kMaxDevices) {
        c.err = "fg_energy_noalloc: device ordinal out of range";
        return FG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(g_lock);
    if (!g_dev_ptr[c.device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || !p) {
            c.err = std::string("fg_energy_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return FG_ECUDA;
        }
        g_dev_ptr[c.device] = static_cast<double *>(p);
    }
    *out = g_dev_ptr[c.device];
    return FG_OK;
}

// Makes the context's device current for the duration of a call and restores the caller's.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
        else if (err == cudaSuccess) prev = -1;  // already current: nothing to restore
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};
}  // namespace

extern "C" int fg_energy_noalloc(fg_ctx *h, const double Hext[3], double energies[4]) {
    if (!h || !Hext || !energies) return FG_EINVAL;
    fg::Ctx &c = h->c;
    const int need = 7 * c.epart_blocks;
    if (need > FG_NOALLOC_PARTIALS) {
        c.err = "fg_energy_noalloc: the reduction needs " + std::to_string(need) + " partial sums, more than the " +
                std::to_string(FG_NOALLOC_PARTIALS) + " of the static scratch array";
        return FG_EINVAL;
    }
    DeviceScope scope(c.device);
    if (scope.err != cudaSuccess) {
        c.err = std::string("fg_energy_noalloc: cannot make the context's device current: ") +
                cudaGetErrorString(scope.err);
        return FG_ECUDA;
    }
    double *scratch = nullptr;
    int s = scratch_address(c, &scratch);
    if (s != FG_OK) return s;
    cudaError_t e = fg::launch_energy_into(c, Hext, scratch);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c.hepart, scratch, sizeof(double) * need, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) {
        c.err = std::string("fg_energy_noalloc: ") + cudaGetErrorString(e);
        return FG_ECUDA;
    }
    double sum[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; k++)
        for (int b = 0; b < c.epart_blocks; b++) sum[k] += c.hepart[k * c.epart_blocks + b];
    for (int k = 0; k < 4; k++) energies[k] = sum[k];
    return FG_OK;
}
