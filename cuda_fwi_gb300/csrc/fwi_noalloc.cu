// fwi_noalloc.cu -- residual and L2 misfit of device-resident traces with no
// memory allocation at all.
//
// Who needs it: callers that must not call cudaMalloc/cudaFree from the code
// that computes the misfit.  Two common cases: (1) a host application whose
// device memory is entirely reserved up front by its own pool allocator, so a
// stray cudaMalloc would fail or fragment its arena; (2) a time-critical loop
// sharing the GPU with other streams, where cudaFree (and often cudaMalloc)
// synchronises the whole device and stalls the other work.  Such callers
// already hold the traces and the residual buffer on the device; this entry
// point only needs scratch for the per-trace partial sums and a divergence
// flag, and keeps that scratch in a fixed file-scope device array.
//
// The scratch array lives in every GPU that loads the library until the
// process exits.  All calls share it and it keeps the last call's contents, so
// the flag is cleared at the start of every call, and calls that overlap on the
// GPU (different streams or host threads at the same time) race on it.
// Its device address is looked up once per device (with that device current)
// and kept for the life of the process: a caller that destroys the device's
// primary context between calls (cudaDeviceReset) invalidates it, so such a
// caller must not use this entry point afterwards.  Every call ends with a
// copy into host memory and a wait on its stream, so it cannot be made while
// that stream is being captured into a CUDA graph.
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>
#include <string>

#include "../../include/fwi_psv.h"
#include "fwi_host.h"

namespace {

// Per-trace partial misfits, their ordered sum, and the divergence flag.
constexpr int kMaxRows = FWI_NOALLOC_MAX_ROWS;
struct Scratch {
    double partial[kMaxRows];
    double total;
    int blowup;
};
static __device__ __align__(256) Scratch g_scratch;

// Scratch address per device, taken once with that device current.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
Scratch* g_addr[kMaxDevices] = {};

__global__ void clear_flag(Scratch* s) { s->blowup = 0; }

// One block per trace: residual = syn - obs (FP32 out, FP64 difference), and
// the trace's partial misfit sum 0.5 dt diff^2 in FP64.
__global__ void residual_rows(const float* __restrict__ syn, const float* __restrict__ obs,
                              float* __restrict__ resid, int nt, double half_dt, Scratch* s) {
    const int r = blockIdx.x;
    const size_t o = (size_t)r * nt;
    double acc = 0.0;
    int big = 0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        const double diff = (double)syn[o + t] - (double)obs[o + t];
        acc += half_dt * diff * diff;
        resid[o + t] = (float)diff;
        big |= fabs(diff) > 1.0e10;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    if (big) atomicOr(&s->blowup, 1);
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) s->partial[r] = sh[0];
}

// Sum of the partial misfits in trace order (deterministic), one thread.
__global__ void sum_rows(Scratch* s, int nrows) {
    double t = 0.0;
    for (int r = 0; r < nrows; r++) t += s->partial[r];
    s->total = t;
}

int scratch_for_current_device(Scratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fwi::fail(FWI_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fwi::fail(FWI_ERR_UNSUPPORTED, "device index above 63");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess)
            return fwi::fail(FWI_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_addr[dev] = static_cast<Scratch*>(p);
    }
    *out = g_addr[dev];
    return FWI_OK;
}

}  // namespace

extern "C" int fwi_psv_misfit_noalloc(const float* d_syn, const float* d_obs, int nrows, int nt,
                                      double dt, float* d_resid, double* misfit, void* stream) {
    if (nrows < 0 || nt < 1 || !misfit || (nrows > 0 && (!d_syn || !d_obs || !d_resid)))
        return fwi::fail(FWI_ERR_INVALID, "bad arguments to fwi_psv_misfit_noalloc");
    if (nrows > kMaxRows)
        return fwi::fail(FWI_ERR_INVALID, "fwi_psv_misfit_noalloc: " + std::to_string(nrows) +
                                              " traces exceed the fixed scratch of " +
                                              std::to_string(kMaxRows) + " (FWI_NOALLOC_MAX_ROWS)");
    // an error left pending by earlier, unrelated work is reported as such
    // (and left for its owner: peek, do not clear)
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
        return fwi::fail(FWI_ERR_CUDA, std::string("fwi_psv_misfit_noalloc: a CUDA error was pending before the "
                                                   "call: ") + cudaGetErrorString(pending));
    Scratch* s = nullptr;
    int st = scratch_for_current_device(&s);
    if (st != FWI_OK) return st;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // the flag is the only scratch that must start at zero (every partial used
    // below is written by this call before it is read)
    clear_flag<<<1, 1, 0, cs>>>(s);
    if (nrows > 0) residual_rows<<<nrows, 256, 0, cs>>>(d_syn, d_obs, d_resid, nt, 0.5 * dt, s);
    sum_rows<<<1, 1, 0, cs>>>(s, nrows);
    double total = 0.0;
    int flag = 0;
    // &s->total, &s->blowup: address arithmetic on the device address only
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, &s->total, sizeof(double), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, &s->blowup, sizeof(int), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess)
        return fwi::fail(FWI_ERR_CUDA, std::string("fwi_psv_misfit_noalloc: ") + cudaGetErrorString(e));
    *misfit = nrows > 0 ? total : 0.0;
    if (flag) return fwi::fail(FWI_ERR_DIVERGED, "|syn - obs| exceeded 1e10");
    return FWI_OK;
}
