// noalloc.cu -- shark_gpu_totals_noalloc: the conserved totals of a state the caller already holds
// on the device, computed without allocating any memory.
//
// Who needs it: callers that may not call cudaMalloc -- a host application whose own allocator
// or memory pool owns every device allocation (for example a Fortran driver that allocates its
// device arrays once at start-up), or a time loop that cannot afford cudaMalloc's implicit device
// synchronisation or a change of its device memory footprint mid-run.  shark_gpu_totals needs a
// context, and the context allocates its partial-sum buffer; this entry point takes the caller's
// state and output pointers and keeps its partial sums in a fixed device array compiled into the
// library.
//
// Scratch: g_totals_scratch, a file-scope __device__ array of kScratchDoubles doubles
// (256 blocks x 260 sums x 2 = 133,120 doubles = 1,064,960 bytes, about 1 MiB).  It becomes
// resident on a device when the CUDA module that holds it is loaded there: with CUDA's default
// lazy module loading that is the first call of this entry point on the device (which therefore
// allocates the module's memory and may synchronise), with CUDA_MODULE_LOADING=EAGER it is the
// creation of the device's context.  From then on the device holds it until the process exits or
// its context is reset.  Every call shares it: the first kernel writes every slot the second
// kernel reads, so nothing needs clearing, but two calls that overlap on the GPU (different
// streams, no ordering) race on it and give wrong results.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/shark_gpu.h"
#include "launch.h"

namespace {

constexpr int kMaxBlocks = 256;                       // stage-1 blocks (fixed)
constexpr int kMaxSums = 4 * (SHARK_MAX_DUST + 1);    // 4 sums per species, gas + 64 dust
constexpr size_t kScratchDoubles = (size_t)kMaxBlocks * kMaxSums * 2;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_totals_scratch[kScratchDoubles];

// Per-device address of g_totals_scratch, looked up with the device current.  The host-side
// symbol g_totals_scratch is only a stand-in for the runtime and must never reach a kernel.
// The address is looked up again on every call whose stream is not capturing (cheap once the
// module is loaded), so a cudaDeviceReset between calls, which unloads the module, cannot leave a
// stale address behind; a call on a capturing stream uses the address of the previous call.
std::mutex g_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// errors are reported through shark_gpu_last_error like every other entry point
int32_t fail(int32_t code, const std::string& msg) { return shark::set_error(code, msg.c_str()); }

// Stage 1: block b Kahan-sums the active cells [b*per, (b+1)*per) of the 4*(N+1) quantities
// (rho, rho*vx, rho*vy, rho*vz of the gas, then of each dust species) of a Fortran-order FP64
// state, and writes (sum, compensation) pairs to the scratch array.
__global__ void k_noalloc_stage1(const double* __restrict__ u, int nx, int ny, int ng, int ndust, long long per,
                                 double* __restrict__ part) {
    const int nq = 4 * (ndust + 1);
    const int nx_max = nx + 2 * ng;
    const int ny_max = (ny == 1) ? 1 : ny + 2 * ng;
    const long long ncells = (long long)nx_max * ny_max;
    const long long nact = (long long)nx * ny;
    const long long a0 = blockIdx.x * per;
    const long long a1 = (a0 + per < nact) ? a0 + per : nact;
    for (int qi = threadIdx.x; qi < nq; qi += blockDim.x) {
        const int s = qi / 4, c = qi % 4;
        const int v = (s == 0) ? c : 5 + c * ndust + (s - 1);
        double sum = 0.0, comp = 0.0;
        for (long long a = a0; a < a1; ++a) {
            const long long iy = (ny == 1) ? 0 : a / nx + ng;
            const long long ix = a % nx + ng;
            const double y = u[(long long)v * ncells + iy * nx_max + ix] - comp;
            const double t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
        part[((long long)blockIdx.x * nq + qi) * 2 + 0] = sum;
        part[((long long)blockIdx.x * nq + qi) * 2 + 1] = comp;
    }
}

// Stage 2: one block combines the per-block pairs in block order (deterministic).
__global__ void k_noalloc_stage2(const double* __restrict__ part, int nblocks, int nq, double* __restrict__ out) {
    for (int qi = threadIdx.x; qi < nq; qi += blockDim.x) {
        double sum = 0.0, comp = 0.0;
        for (int b = 0; b < nblocks; ++b) {
            const double y = (part[((long long)b * nq + qi) * 2 + 0] - part[((long long)b * nq + qi) * 2 + 1]) - comp;
            const double t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
        out[qi] = sum;
    }
}

}  // namespace

extern "C" int32_t shark_gpu_totals_noalloc(const double* u_dev, int32_t nx, int32_t ny, int32_t nghost,
                                            int32_t ndust, double* out_dev, void* stream) {
    if (!u_dev || !out_dev) return fail(SHARK_ERR_INVALID_ARG, "NULL device pointer");
    if (nx < 1 || ny < 1 || nghost < 0) return fail(SHARK_ERR_INVALID_ARG, "nx, ny >= 1 and nghost >= 0 required");
    if (ndust < 0 || ndust > SHARK_MAX_DUST)
        return fail(SHARK_ERR_INVALID_ARG, "ndust must be 0..64: the fixed scratch array holds 4*(64+1) sums per block");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SHARK_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(SHARK_ERR_NO_DEVICE, "device ordinal beyond the supported 64");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* part = nullptr;
    {
        // set-up with the device current: resolve the device address of the scratch array.  The
        // first call on a device must do this outside any capture (it may load the module), so it
        // must come before any stream capture; later calls refresh it unless `stream` is capturing
        std::lock_guard<std::mutex> lock(g_mutex);
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        const bool capturing = cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone;
        if (!capturing) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_totals_scratch);
            if (e != cudaSuccess)
                return fail(SHARK_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<double*>(ptr);
        } else if (!g_scratch_addr[dev]) {
            return fail(SHARK_ERR_INVALID_ARG,
                        "first call on this device made on a capturing stream: make one call before capture");
        }
        part = g_scratch_addr[dev];
    }
    const long long nact = (long long)nx * ny;
    const int nblocks = (int)((nact + 1023) / 1024 < kMaxBlocks ? (nact + 1023) / 1024 : kMaxBlocks);
    const long long per = (nact + nblocks - 1) / nblocks;
    k_noalloc_stage1<<<nblocks, 128, 0, st>>>(u_dev, nx, ny, nghost, ndust, per, part);
    k_noalloc_stage2<<<1, 128, 0, st>>>(part, nblocks, 4 * (ndust + 1), out_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SHARK_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return SHARK_OK;
}
