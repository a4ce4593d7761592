// fwi_engine.cu -- device engine behind include/fwi_psv.h.
//
// One engine = one padded grid (fd_grid.cu:52-71 conventions), one set of
// materials and one acquisition (sources/receivers with their shot ids).  A
// forward/backward call runs a *batch* of shots together: every launch covers
// all shots of the batch (tile work-list), so the per-launch overhead is paid
// once per time step instead of once per shot and step, and the material tile
// is shared in L2 by the shots processed back to back.  The time loop is
// captured into CUDA graphs and replayed.
//
// Reference call sequence kept (Mohammad-debug/CUDA_FWI, CUDA_week2/):
//   forward per shot  fd_wave_model.cu:791-803   -> fwi_psv_forward
//   residual/misfit   fd_wave_model.cu:972-1002  -> residual_kernel
//   adjoint per shot  fd_wave_model.cu:848-859   -> fwi_psv_backward
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/fwi_psv.h"
#include "fwi_alloc.hpp"
#include "fwi_host.h"
#include "fwi_exact.cuh"
#include "fwi_kernels.cuh"
#include "fwi_tma.cuh"
#include "fwi_fused.cuh"

namespace fwi {

#define CUDA_TRY(expr)                                                                   \
    do {                                                                                 \
        cudaError_t _e = (expr);                                                         \
        if (_e != cudaSuccess)                                                           \
            return fail(FWI_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

#define FWI_TRY(expr)            \
    do {                         \
        int _s = (expr);         \
        if (_s != FWI_OK) return _s; \
    } while (0)

// ---------------------------------------------------------------------------
// small device kernels
// ---------------------------------------------------------------------------

// residual = syn - obs (in place into resid), per-row partial misfit sums in FP64
// (fd_wave_model.cu:972-1002).  One block per receiver row.
__global__ void residual_kernel(const float* __restrict__ syn, const float* __restrict__ obs,
                                const int* __restrict__ row_rec, float* __restrict__ resid,
                                double* __restrict__ row_misfit, int* __restrict__ blowup, int nt,
                                double half_dt) {
    const int r = blockIdx.x;
    const size_t o = (size_t)r * nt;
    const float* ob = obs + (size_t)row_rec[r] * nt;
    double acc = 0.0;
    int big = 0;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        const double diff = (double)syn[o + t] - (double)ob[t];
        acc += half_dt * diff * diff;
        resid[o + t] = (float)diff;
        big |= !(fabs(diff) <= 1.0e10);  // also NaN / Inf
    }
    __shared__ double sh[256];
    __shared__ int sb;
    if (threadIdx.x == 0) sb = 0;
    sh[threadIdx.x] = acc;
    __syncthreads();
    if (big) atomicOr(&sb, 1);
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        row_misfit[r] = sh[0];
        if (sb) atomicOr(blowup, 1);
    }
}

// Device watchdog: a non-finite value among samples [t0, t1) of the recorded
// traces ([nrows][nt]) sets bit 16 of the error word (the host reports
// FWI_ERR_DIVERGED; the TMA kernels of later steps return at once).
__global__ void watch_traces_kernel(const float* __restrict__ rec, int nrows, int nt, int t0, int t1,
                                    int* __restrict__ err) {
    const int n = t1 - t0;
    const size_t total = (size_t)nrows * n;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        if (!isfinite(rec[(i / n) * nt + t0 + i % n])) {
            atomicOr(err, 16);
            return;
        }
    }
}
// the same over a flat array (the gradients)
__global__ void watch_array_kernel(const float* __restrict__ a, size_t n, int* __restrict__ err) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (!isfinite(a[i])) {
            atomicOr(err, 16);
            return;
        }
    }
}
constexpr int kWatchSteps = 64;  // recorded steps between two watchdog checks

// Source injection and receiver recording of one batch slot per block, after
// a velocity pass that did neither (the TMA mapping): the injections of a
// cell are added in event order by one thread (events are sorted by column,
// row, injections first), then the receivers read vz
// (forward_kernel_PSV_GPU.cu:1033-1063 order).
__device__ __forceinline__ void slot_events(const ItemDesc& D, int it, unsigned flags);
__global__ void events_kernel(const ItemDesc* __restrict__ items, int it, unsigned flags) {
    slot_events(items[blockIdx.x], it, flags);
}
// the same for the models listed in ids (one block each)
__global__ void events_list_kernel(const ItemDesc* __restrict__ items, const int* __restrict__ ids, int it,
                                   unsigned flags) {
    slot_events(items[ids[blockIdx.x]], it, flags);
}
__device__ __forceinline__ void slot_events(const ItemDesc& D, int it, unsigned flags) {
    const int e0 = D.ev_col[0], e1 = D.ev_col[D.nxt];
    const int nt = D.nt, P = D.pitch;
    if (flags & FL_INJECT)
        for (int e = e0 + (int)threadIdx.x; e < e1; e += blockDim.x) {
            const int2 v = D.ev[e];
            const int x = D.ev_x[e];
            if (v.y < 0) continue;
            if (e > e0 && D.ev_x[e - 1] == x && D.ev[e - 1].x == v.x) continue;  // not the cell's first
            float* c = D.vz + (size_t)v.x * P + x;
            float val = *c;
            const bool undo = (flags & FL_REVERSE) != 0;  // remove the injection of step it
            for (int q = e; q < e1 && D.ev_x[q] == x && D.ev[q].x == v.x && D.ev[q].y >= 0; q++)
                val = undo ? val - D.inj[(size_t)D.ev[q].y * nt + it] : val + D.inj[(size_t)D.ev[q].y * nt + it];
            *c = val;
        }
    __syncthreads();
    if (flags & FL_RECORD)
        for (int e = e0 + (int)threadIdx.x; e < e1; e += blockDim.x) {
            const int2 v = D.ev[e];
            if (v.y < 0) D.rec[(size_t)(~v.y) * nt + it] = D.vz[(size_t)v.x * P + D.ev_x[e]];
        }
}

// FDMedium::average_parameters (fd_medium.cu:128-159) on the device, fused
// with the dt scaling of the engine's material layout: FP64 lam, mu, rho
// [nzt][nxt] -> FP32 L, M2, MZX, BX, BZ [nzt][pitch].  Same FP64 expressions
// as the host path (fwi_host.cpp), so both give identical materials.
__global__ void materials_kernel(const double* __restrict__ lam, const double* __restrict__ mu,
                                 const double* __restrict__ rho, int nzt, int nxt, int pitch, int fpad,
                                 double dt, float* __restrict__ mat, size_t field, int* __restrict__ zero_mu) {
    const size_t n = (size_t)nzt * nxt;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / nxt), ix = (int)(i % nxt);
        const size_t o = (size_t)iz * pitch + ix;
        mat[o] = (float)(dt * lam[i]);
        mat[field + o] = (float)(2.0 * dt * mu[i]);
        if (mu[i] == 0.0 && iz >= fpad && iz < nzt - fpad && ix >= fpad && ix < nxt - fpad) atomicOr(zero_mu, 1);
        float mz = 0.f, bx = 0.f, bz = 0.f;
        if (iz < nzt - 1 && ix < nxt - 1) {
            const double m00 = mu[i], m01 = mu[i + 1], m10 = mu[i + nxt], m11 = mu[i + nxt + 1];
            const bool zero = m00 == 0.0 || m01 == 0.0 || m10 == 0.0 || m11 == 0.0;
            const double h = zero ? 0.0 : 4.0 / ((1.0 / m00) + (1.0 / m01) + (1.0 / m10) + (1.0 / m11));
            const double r00 = rho[i], r10 = rho[i + nxt], r01 = rho[i + 1];
            double rzp = 1.0 / (0.5 * (r00 + r10));
            const double rxp = 1.0 / (0.5 * (r00 + r01));
            if (r00 < 1e-4 && r10 < 1e-4) rzp = 0.0;
            if (r00 < 1e-4 && r01 < 1e-4) rzp = 0.0;  // the reference's second guard (fd_medium.cu:152-154)
            mz = (float)(dt * h);
            bx = (float)(dt * rxp);
            bz = (float)(dt * rzp);
        }
        mat[2 * field + o] = mz;
        mat[3 * field + o] = bx;
        mat[4 * field + o] = bz;
    }
}

// Random-boundary frame (Clapp's random boundaries for reverse-time
// reconstruction, SEG 2009): copy the materials and, in the padding around the
// model, scale the velocities by f = 1 - alpha (d / ppad) u, with d the depth
// into the padding and u a hashed uniform number in [0, 1) per block of
// kRandomGrain x kRandomGrain cells, i.e. L, M2, MZX by f^2 with density
// unchanged.  Velocities only decrease, so the time step stays stable; the
// frame scatters boundary reflections instead of absorbing them, which keeps
// the scheme reversible (no damping).  Blocks rather than single cells: at the
// workloads' wavelengths (10-45 cells) per-cell noise averages out into a
// smooth slowdown that reflects coherently; 16-cell blocks scatter more (on
// 8 shots of the 1068x568 order-8 workload the interior rho gradient's
// difference to the binomial one fell from 0.59 to 0.49, mu's from 0.21 to
// 0.18; 4- and 8-cell blocks gave 0.53 and 0.55 for rho).
__device__ __forceinline__ unsigned hash_u32(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
constexpr int kRandomGrain = 16;
__global__ void random_frame_kernel(const float* __restrict__ mat, float* __restrict__ rb, size_t field, int nzt,
                                    int nxt, int pitch, int ppad, int fsurf, unsigned seed, float alpha) {
    const size_t n = (size_t)nzt * nxt;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i / nxt), ix = (int)(i % nxt);
        int d = 0;
        d = max(d, ppad - ix);
        d = max(d, ix - (nxt - 1 - ppad));
        if (!fsurf) d = max(d, ppad - iz);
        d = max(d, iz - (nzt - 1 - ppad));
        float f2 = 1.f;
        if (d > 0 && ppad > 0) {
            const unsigned key = (unsigned)(iz / kRandomGrain) * 65599u + (unsigned)(ix / kRandomGrain);
            const float u = (float)(hash_u32(key * 2654435761u + seed) >> 8) * (1.f / 16777216.f);
            const float f = 1.f - alpha * ((float)d / (float)ppad) * u;
            f2 = f * f;
        }
        const size_t o = (size_t)iz * pitch + ix;
        rb[o] = mat[o] * f2;
        rb[field + o] = mat[field + o] * f2;
        rb[2 * field + o] = mat[2 * field + o] * f2;
        rb[3 * field + o] = mat[3 * field + o];
        rb[4 * field + o] = mat[4 * field + o];
    }
}

// Energy weights of one batch slot per blockIdx.y (fd_wave_model.cu:1004-1052):
// the largest sqrt(Ws * Wr) over the FWI window samples (non-negative, so the
// float bits order like the values).
__global__ void we_max_kernel(const ItemDesc* __restrict__ items, const float* __restrict__ ws,
                              const float* __restrict__ wr, size_t field, unsigned* __restrict__ wmax) {
    const int b = blockIdx.y;
    const ItemDesc& D = items[b];
    const size_t nf = (size_t)D.nfz * D.nfx;
    float m = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += (size_t)gridDim.x * blockDim.x) {
        const int zf = (int)(i / D.nfx), xf = (int)(i % D.nfx);
        const int iz = D.wz1 + zf * D.fwi_dz, ix = D.wx1 + xf * D.fwi_dx;
        if (iz >= D.wz2 || ix >= D.wx2) continue;
        const size_t c = (size_t)b * field + (size_t)iz * D.pitch + ix;
        m = fmaxf(m, (float)sqrt((double)ws[c] * (double)wr[c]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(wmax + b, __float_as_uint(m));
}

// Divide each slot's gradient by its regularised energy weight
// sqrt(Ws Wr) + 0.005 max; the constant 1/C^2 factors are applied in FP64
// when the gradients leave the device (FP32 would underflow them).
__global__ void precondition_kernel(const ItemDesc* __restrict__ items, const float* __restrict__ ws,
                                    const float* __restrict__ wr, size_t field, const unsigned* __restrict__ wmax) {
    const int b = blockIdx.y;
    const ItemDesc& D = items[b];
    const size_t nf = (size_t)D.nfz * D.nfx;
    const double reg = 0.005 * (double)__uint_as_float(wmax[b]);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += (size_t)gridDim.x * blockDim.x) {
        const int zf = (int)(i / D.nfx), xf = (int)(i % D.nfx);
        const int iz = D.wz1 + zf * D.fwi_dz, ix = D.wx1 + xf * D.fwi_dx;
        if (iz >= D.wz2 || ix >= D.wx2) continue;
        const size_t c = (size_t)b * field + (size_t)iz * D.pitch + ix;
        const double we = sqrt((double)ws[c] * (double)wr[c]) + reg;
        D.glam[i] = (float)((double)D.glam[i] / we);
        D.gmu[i] = (float)((double)D.gmu[i] / we);
        D.grho[i] = (float)((double)D.grho[i] / we);
    }
}

// Device copy of whole batch states (checkpoint saves and restores) on the
// SMs: 16-byte loads and stores, four in flight per thread.  For copies of
// this size (a 14-shot state of the 1068x568 grid is ~200 MB) the SMs move
// about twice the bytes per second of the device-to-device copy engines.
__global__ void copy_kernel(float4* __restrict__ dst, const float4* __restrict__ src, size_t n4) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        const float4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n4; i += stride) dst[i] = src[i];
}

// Launch of copy_kernel for n floats (n a multiple of 4, both pointers
// 16-byte aligned: whole states).
inline cudaError_t device_copy(float* dst, const float* src, size_t n, int num_sms, cudaStream_t s) {
    const size_t n4 = n / 4;
    const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>((n4 + 255) / 256, (size_t)num_sms * 8));
    copy_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<float4*>(dst), reinterpret_cast<const float4*>(src), n4);
    return cudaGetLastError();
}

// sum the per-shot gradient triples: out[i] = sum_b in[b*n + i]
__global__ void sum_shots_kernel(const float* __restrict__ in, float* __restrict__ out, size_t n,
                                 int nb, int accumulate) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nb; b++) s += in[(size_t)b * n + i];
        out[i] = accumulate ? out[i] + s : s;
    }
}

// ---------------------------------------------------------------------------
// kernel dispatch on the half order
// ---------------------------------------------------------------------------
using LaunchFn = void (*)(dim3, cudaStream_t, const ItemDesc*, const Tile*, int, int, unsigned, int*);
using OccFn = int (*)();

template <int FP, bool ADJ, int MAP>
static void launch_stress(dim3 g, cudaStream_t s, const ItemDesc* items, const Tile* tiles,
                          int ntiles, int it, unsigned flags, int* err) {
    stress_kernel<FP, ADJ, MAP><<<g, dim3(MapDims<MAP>::x, MapDims<MAP>::y), 0, s>>>(items, tiles, ntiles,
                                                                                    it, flags, err);
}
template <int FP, int MAP>
static void launch_velocity(dim3 g, cudaStream_t s, const ItemDesc* items, const Tile* tiles,
                            int ntiles, int it, unsigned flags, int* err) {
    velocity_kernel<FP, MAP><<<g, dim3(MapDims<MAP>::x, MapDims<MAP>::y), 0, s>>>(items, tiles, ntiles, it,
                                                                                 flags, err);
}
template <int FP, bool ADJ, int MAP>
static int occ_stress() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stress_kernel<FP, ADJ, MAP>,
                                                  MapDims<MAP>::x * MapDims<MAP>::y, 0);
    return n;
}
template <int FP, int MAP>
static int occ_velocity() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, velocity_kernel<FP, MAP>,
                                                  MapDims<MAP>::x * MapDims<MAP>::y, 0);
    return n;
}

// The kernels of one thread mapping: MAP 0 = z-march, 1 = cell-parallel.
struct KernelSet {
    LaunchFn stress_f, stress_a, velocity;
    OccFn occ_f, occ_a, occ_v;
    int map;
};

// The vectorised mapping (MAP 2) keeps the adjoint stress pass on the scalar
// cell mapping: its per-cell gradient update does not vectorise and the
// register-light scalar kernel runs it faster (measured: 43 us vs 76 us for
// 2 shots of the 1068x568 grid, order 8).
template <int FP, int MAP>
static KernelSet kernel_set() {
    constexpr int AMAP = MAP == 2 ? 1 : MAP;
    return {launch_stress<FP, false, MAP>, launch_stress<FP, true, AMAP>, launch_velocity<FP, MAP>,
            occ_stress<FP, false, MAP>, occ_stress<FP, true, AMAP>, occ_velocity<FP, MAP>, MAP};
}

template <int MAP>
static KernelSet kernels_for_map(int fp) {
    switch (fp) {
        case 1: return kernel_set<1, MAP>();
        case 2: return kernel_set<2, MAP>();
        case 3: return kernel_set<3, MAP>();
        case 4: return kernel_set<4, MAP>();
        case 5: return kernel_set<5, MAP>();
        default: return kernel_set<6, MAP>();
    }
}
static KernelSet kernels_for(int fp, int map) {
    if (map == 2 && fp <= 4) return kernels_for_map<2>(fp);
    // the TMA mapping (3) runs its adjoint stress pass on the scalar cells
    return map ? kernels_for_map<1>(fp) : kernels_for_map<0>(fp);
}

// TMA-staged forward stress and velocity passes (fwi_tma.cuh).
using TmaStressFn = void (*)(dim3, cudaStream_t, const StressMaps&, const ItemDesc*, TmaGrid, int, unsigned, int*);
using TmaVelFn = void (*)(dim3, cudaStream_t, const VelMaps&, const ItemDesc*, TmaGrid, int, unsigned, int*);
using TmaAdjFn = void (*)(dim3, cudaStream_t, const AdjMaps&, const ItemDesc*, TmaGrid, int, unsigned, int*);
struct TmaSet {
    TmaStressFn stress;
    TmaVelFn velocity;
    TmaAdjFn adjoint;
    cudaError_t (*prepare)();  // opt in to the dynamic shared memory
};
template <int FP>
static void t_stress(dim3 g, cudaStream_t s, const StressMaps& m, const ItemDesc* it, TmaGrid tg, int step,
                     unsigned flags, int* err) {
    stress_tma_kernel<FP><<<g, kFwdThreads, stress_tma_smem<FP>(), s>>>(m, it, tg, step, flags, err);
}
template <int FP>
static void t_velocity(dim3 g, cudaStream_t s, const VelMaps& m, const ItemDesc* it, TmaGrid tg, int step,
                       unsigned flags, int* err) {
    velocity_tma_kernel<FP><<<g, kFwdThreads, velocity_tma_smem<FP>(), s>>>(m, it, tg, step, flags, err);
}
template <int FP>
static void t_adjoint(dim3 g, cudaStream_t s, const AdjMaps& m, const ItemDesc* it, TmaGrid tg, int step,
                      unsigned flags, int* err) {
    adjoint_tma_kernel<FP><<<g, kAdjThreads, adjoint_tma_smem<FP>(), s>>>(m, it, tg, step, flags, err);
}
template <int FP>
static cudaError_t t_prepare() {
    cudaError_t e = cudaFuncSetAttribute(stress_tma_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)stress_tma_smem<FP>());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(adjoint_tma_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)adjoint_tma_smem<FP>());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(velocity_tma_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)velocity_tma_smem<FP>());
}
template <int FP>
static TmaSet tma_set() {
    return {t_stress<FP>, t_velocity<FP>, t_adjoint<FP>, t_prepare<FP>};
}
static TmaSet tma_for(int fp) {
    switch (fp) {
        case 1: return tma_set<1>();
        case 2: return tma_set<2>();
        case 3: return tma_set<3>();
        case 4: return tma_set<4>();
        case 5: return tma_set<5>();
        default: return tma_set<6>();
    }
}

// Fused forward step (fwi_fused.cuh), fdorder 2..8.
using FusedFn = void (*)(dim3, cudaStream_t, const FusedMaps&, const ItemDesc*, FusedGrid, int, unsigned, int*);
template <int FP>
static void t_fused(dim3 g, cudaStream_t s, const FusedMaps& m, const ItemDesc* it, FusedGrid fg, int step,
                    unsigned flags, int* err) {
    step_fused_kernel<FP><<<g, kFusedThreads, fused_smem<FP>(), s>>>(m, it, fg, step, flags, err);
}
template <int FP>
static cudaError_t f_prepare() {
    return cudaFuncSetAttribute(step_fused_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fused_smem<FP>());
}
struct FusedSet {
    FusedFn step = nullptr;
    cudaError_t (*prepare)() = nullptr;
};
static FusedSet fused_for(int fp) {
    switch (fp) {
        case 1: return {t_fused<1>, f_prepare<1>};
        case 2: return {t_fused<2>, f_prepare<2>};
        case 3: return {t_fused<3>, f_prepare<3>};
        case 4: return {t_fused<4>, f_prepare<4>};
        default: return {};
    }
}

// Forward steps a backward runs for a binomial plan over n units: from the
// last checkpoint of the first sweep (placed while the forward records) to
// the last unit, then every ADVANCE after that prefix, plus state n+1 of each
// reverse step of the exact adjoint.  The same count whether the plan runs
// directly or as a replayed graph.
static long long plan_recompute_steps(const std::vector<Action>& plan, int n, bool exact_steps) {
    size_t k = 0;
    int last_state = 0;
    while (k < plan.size() && plan[k].kind != Action::ADJOINT) {
        if (plan[k].kind == Action::SAVE) last_state = plan[k].b;
        k++;
    }
    long long r = (long long)(n - 1) - last_state;
    for (; k < plan.size(); k++) {
        if (plan[k].kind == Action::ADVANCE) r += plan[k].b - plan[k].a;
        if (plan[k].kind == Action::ADJOINT && exact_steps) r += 1;
    }
    return r;
}

// TMA-staged passes over a work-list of tiles of several models (the
// multi-model engine; maps per model in device memory).
// Arguments: maps of the source and destination buffers, descriptors writing
// to the destination, tiles, count, step, flags, adjoint state (velocity
// pass), CPML-memory offset source - destination (floats), error word.
using TmaMultiFn = void (*)(dim3, cudaStream_t, const MultiMaps*, const MultiMaps*, const ItemDesc*, const Tile*, int,
                            int, unsigned, int, long long, int*);
struct TmaMultiSet {
    TmaMultiFn stress, velocity, adjoint;
    cudaError_t (*prepare)();
};
template <int FP>
static void tm_stress(dim3 g, cudaStream_t s, const MultiMaps* mx, const MultiMaps* my, const ItemDesc* it,
                      const Tile* t, int nt, int step, unsigned flags, int, long long msrc, int* err) {
    stress_tma_multi_kernel<FP><<<g, kFwdThreads, stress_tma_smem<FP>(), s>>>(mx, my, it, t, nt, step, flags, msrc,
                                                                                 err);
}
template <int FP>
static void tm_velocity(dim3 g, cudaStream_t s, const MultiMaps* mx, const MultiMaps* my, const ItemDesc* it,
                        const Tile* t, int nt, int step, unsigned flags, int adj, long long msrc, int* err) {
    velocity_tma_multi_kernel<FP><<<g, kFwdThreads, velocity_tma_smem<FP>(), s>>>(mx, my, it, t, nt, step, flags,
                                                                                     adj, msrc, err);
}
template <int FP>
static void tm_adjoint(dim3 g, cudaStream_t s, const MultiMaps* mx, const MultiMaps*, const ItemDesc* it,
                       const Tile* t, int nt, int step, unsigned flags, int, long long, int* err) {
    adjoint_tma_multi_kernel<FP><<<g, kAdjThreads, adjoint_tma_smem<FP>(), s>>>(mx, it, t, nt, step, flags, err);
}
template <int FP>
static cudaError_t tm_prepare() {
    cudaError_t e = cudaFuncSetAttribute(stress_tma_multi_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)stress_tma_smem<FP>());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(adjoint_tma_multi_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)adjoint_tma_smem<FP>());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(velocity_tma_multi_kernel<FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)velocity_tma_smem<FP>());
}
template <int FP>
static TmaMultiSet tma_multi_set() {
    return {tm_stress<FP>, tm_velocity<FP>, tm_adjoint<FP>, tm_prepare<FP>};
}
static TmaMultiSet tma_multi_for(int fp) {
    switch (fp) {
        case 1: return tma_multi_set<1>();
        case 2: return tma_multi_set<2>();
        case 3: return tma_multi_set<3>();
        case 4: return tma_multi_set<4>();
        case 5: return tma_multi_set<5>();
        default: return tma_multi_set<6>();
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link-time
// dependency on libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// FP32 tensor map of nb slices [nz][nx] (row stride row_bytes, slice stride
// slice_bytes; nb == 0 makes a 2-D map), box bx x bz (x 1), zero fill outside.
static int make_map(CUtensorMap* m, const float* base, int nx, int nz, int nb, size_t row_bytes,
                    size_t slice_bytes, int bx, int bz) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return fail(FWI_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)nz, (cuuint64_t)std::max(nb, 1)};
    const cuuint64_t strides[2] = {(cuuint64_t)row_bytes, (cuuint64_t)slice_bytes};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)bz, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const cuuint32_t rank = nb > 0 ? 3 : 2;
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<float*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(FWI_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return FWI_OK;
}

// Exact discrete adjoint (fwi_exact.cuh): four cell-parallel kernels per
// reverse step plus the final chain rule onto lam, mu, rho.
constexpr int kExactThreads = 256;
constexpr int kDefaultMap = 3;  // thread mapping of a new engine (TMA-staged tiles)
using ExactStepFn = void (*)(dim3, cudaStream_t, const ItemDesc*, const ExactDesc*, int, int, long long);
struct ExactSet {
    ExactStepFn vel_local, vel_stencil, str_local, str_stencil;
};
template <int FP>
static void x_vel_local(dim3 g, cudaStream_t s, const ItemDesc* it, const ExactDesc* ex, int nb, int step,
                        long long cells) {
    vel_adj_local<FP><<<g, kExactThreads, 0, s>>>(it, ex, nb, step, cells);
}
template <int FP>
static void x_vel_stencil(dim3 g, cudaStream_t s, const ItemDesc* it, const ExactDesc* ex, int nb, int,
                          long long cells) {
    vel_adj_stencil<FP><<<g, kExactThreads, 0, s>>>(it, ex, nb, cells);
}
template <int FP>
static void x_str_local(dim3 g, cudaStream_t s, const ItemDesc* it, const ExactDesc* ex, int nb, int,
                        long long cells) {
    str_adj_local<FP><<<g, kExactThreads, 0, s>>>(it, ex, nb, cells);
}
template <int FP>
static void x_str_stencil(dim3 g, cudaStream_t s, const ItemDesc* it, const ExactDesc* ex, int nb, int,
                          long long cells) {
    str_adj_stencil<FP><<<g, kExactThreads, 0, s>>>(it, ex, nb, cells);
}
template <int FP>
static ExactSet exact_set() {
    return {x_vel_local<FP>, x_vel_stencil<FP>, x_str_local<FP>, x_str_stencil<FP>};
}
static ExactSet exact_for(int fp) {
    switch (fp) {
        case 1: return exact_set<1>();
        case 2: return exact_set<2>();
        case 3: return exact_set<3>();
        case 4: return exact_set<4>();
        case 5: return exact_set<5>();
        default: return exact_set<6>();
    }
}

// ---------------------------------------------------------------------------
// device buffer
// ---------------------------------------------------------------------------
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DeviceAllocator al;  // the allocator that made p
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        device_free(p, al);
        p = nullptr;
        bytes = 0;
    }
    int ensure(size_t n) {
        if (n <= bytes && p) return FWI_OK;
        release();
        if (n == 0) return FWI_OK;
        cudaError_t e = device_alloc(&p, n, &al);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return fail(FWI_ERR_NOMEM, "device allocation of " + std::to_string(n) + " bytes failed: " +
                                           (e == cudaErrorMisalignedAddress
                                                ? std::string("the allocator's pointer is not 256-byte aligned")
                                                : std::string(cudaGetErrorString(e))));
        }
        bytes = n;
        return FWI_OK;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

static size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }

// Bounds-checked build (FWI_BOUNDS_CHECK): the first out-of-range access a
// kernel recorded since the last call, reported and cleared.
static int check_bounds_record() {
#if FWI_BOUNDS_CHECK
    unsigned long long v = 0;
    CUDA_TRY(cudaMemcpyFromSymbol(&v, g_fwi_oob, sizeof(v)));
    if (v) {
        const unsigned long long zero = 0;
        CUDA_TRY(cudaMemcpyToSymbol(g_fwi_oob, &zero, sizeof(zero)));
        return fail(FWI_ERR_CUDA, "out-of-range index " + std::to_string((long long)(v & 0xFFFFFFFFFFFFull)) +
                                      " at access site " + std::to_string((int)(v >> 48)) + "; results discarded");
    }
#endif
    return FWI_OK;
}

// page-locked host staging buffer (fast, asynchronous copies)
struct HBuf {
    void* p = nullptr;
    size_t bytes = 0;
    HBuf() = default;
    HBuf(const HBuf&) = delete;
    HBuf& operator=(const HBuf&) = delete;
    ~HBuf() {
        if (p) cudaFreeHost(p);
    }
    int ensure(size_t n) {
        if (n <= bytes && p) return FWI_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        if (cudaMallocHost(&p, n) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return fail(FWI_ERR_NOMEM, "cudaMallocHost of " + std::to_string(n) + " bytes failed");
        }
        bytes = n;
        return FWI_OK;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------
struct Engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // geometry / scheme
    int nt, nzt, nxt, fpad, ppad, npml, fsurf, fdorder, tp, pitch, pnx, pnz;
    double dt, dx, dz, hc[7];
    std::vector<float> cpml_h;  // [6][tp], then the same per column: [tp][6]
    // FWI window
    int fwi_dt = 1, fwi_dx = 1, fwi_dz = 1, wx1 = 0, wx2 = 0, wz1 = 0, wz2 = 0;
    int nft = 0, nfz = 0, nfx = 0;
    // strategy
    int strategy = FWI_STORE_FULL, snapshots_req = 0, grad_mode = FWI_GRAD_REFERENCE;
    size_t budget = 0;
    int use_graphs = 1, bx_req = 0, tz_req = 0;
    // sizes (floats)
    size_t field = 0, xstrip = 0, zstrip = 0, state = 0, nf = 0;
    // device constants
    DBuf d_mat, d_cpml, d_srcsig;
    bool have_model = false;
    // acquisition
    std::vector<int> sx, sz, scomp, sshot, rx, rz, rcomp, rshot;
    int nsrc = 0, nrec = 0;
    // batch
    int B = 0;
    std::vector<int> shots;
    std::vector<int> rows;  // receiver index of each batch row
    std::vector<int> row_slot;
    DBuf d_fwd, d_adj, d_ws, d_wr, d_ux, d_uz, d_grad, d_gsum, d_store, d_snap;
    DBuf d_evcol_f, d_ev_f, d_evcol_a, d_ev_a, d_evx_f, d_evx_a, d_rec, d_resid, d_rowmis, d_blow;
    DBuf d_items_f, d_items_a;
    // exact discrete adjoint: forward state n+1, derivative adjoints + sensitivities, descriptors
    DBuf d_nxt, d_exact, d_exd, d_items_n;
    ExactSet xs{};
    // TMA mapping: kernels, tensor maps per state buffer (0 fwd, 1 adj, 2 state n+1,
    // 3 fwd with the random-boundary materials), tile grid
    TmaSet tset{};
    StressMaps smaps[4];
    VelMaps vmaps[4];
    AdjMaps amap;
    // Copy-free checkpointing (TMA mapping, binomial plan): buffer k < slots is
    // checkpoint memory, buffer `slots` is d_fwd; per buffer the stress and
    // velocity maps of its state, the adjoint maps reading the forward fields
    // from it, and the forward descriptors writing to it.
    std::vector<StressMaps> smaps_b;
    std::vector<VelMaps> vmaps_b;
    std::vector<AdjMaps> amaps_b;
    DBuf d_items_b;
    const AdjMaps* amap_cur = nullptr;  // forward fields of the adjoint pass (null: amap)
    TmaGrid tgrid{}, tgrid_a{};
    int grid_tma = 1, grid_tma_a = 1;
    // Fused forward step (one launch per step, state double-buffered): the
    // working state alternates between d_fwd and d_fwd2; per buffer k (the
    // buffers of buf()) the maps the step reads from it.
    bool fuse = false;  // set_exec: 512 the fused step, 0/256 the two TMA passes
    FusedSet fset{};
    DBuf d_fwd2;
    std::vector<FusedMaps> fmaps_b;
    FusedGrid fgrid{};
    int grid_fused = 1;
    unsigned long long wait_ns = kWaitNs;  // limit of the kernels' bounded waits
    bool stall_next = false, stall_pending = false;  // test hook: one forward step whose wait runs out
    bool zero_mu = false;  // some interior cell has mu == 0 (exact mode unsupported)
    // energy-weight preconditioning of each shot's gradient (fd_wave_model.cu:1004-1052)
    bool pre_on = false;
    double pre_c[3] = {1.0, 1.0, 1.0};  // C_lam, C_mu, C_rho
    DBuf d_wmax;
    double out_scale(int q) const { return pre_on ? 1.0 / (pre_c[q] * pre_c[q]) : 1.0; }
    // wavefield snapshots of the recording sweep (forward_kernel_PSV_GPU.cu:1067-1080)
    int snap_interval = 0, snap_field = F_SZZ, nsnap = 0;
    DBuf d_snapshots;  // [B][nsnap][field]
    // random-boundary strategy: frame materials, their validity, whether the
    // current batch's forward items use them
    DBuf d_mat_rb, d_items_rb;
    bool rb_valid = false, rb_active = false;
    unsigned rb_seed = 20090625u;
    float rb_alpha = 0.5f;
    HBuf h_stage, h_rec, h_grad;
    DBuf d_err;  // kernel error flags (bounded waits that timed out)
    bool obs_valid = false;
    int ntiles = 0, bx = 128, tz = 32;
    KernelSet ks{};
    int kmap = kDefaultMap;  // thread mapping of the stencil kernels (0 z-march, 1 cells, 2 vector cells, 3 TMA tiles)
    int grid_sf = 1, grid_sa = 1, grid_v = 1, num_sms = 1;
    int slots = 0;  // checkpoint slots per shot (binomial)
    bool fwd_kept = false, have_resid = false, bwd_done = false, grad_on = true;
    std::vector<Action> plan;
    long long plan_cost = 0;
    // graphs keyed by a phase name; invalidated when the batch layout changes
    std::map<std::string, cudaGraphExec_t> graphs;
    fwi_psv_stats stats{};
    int64_t launches_now = 0;

    ~Engine() {
        drop_graphs();
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    int bind() { CUDA_TRY(cudaSetDevice(device)); return FWI_OK; }

    // ---- setup ---------------------------------------------------------
    int init(const fwi_psv_desc* d) {
        nt = d->nt; nzt = d->nzt; nxt = d->nxt; fpad = d->fpad; ppad = d->ppad;
        npml = d->npml; fsurf = d->fsurf ? 1 : 0; fdorder = d->fdorder;
        dt = d->dt; dx = d->dx; dz = d->dz;
        std::memcpy(hc, d->hc, sizeof hc);
        if (fdorder < 2 || fdorder > 12 || (fdorder & 1))
            return fail(FWI_ERR_UNSUPPORTED, "fdorder must be even and in 2..12");
        if (fpad != fdorder / 2) return fail(FWI_ERR_INVALID, "fpad must equal fdorder/2");
        if (npml < 0 || ppad != npml + fpad) return fail(FWI_ERR_INVALID, "ppad must equal npml + fpad");
        if (nt < 1) return fail(FWI_ERR_INVALID, "nt must be >= 1");
        if (nxt < 2 * ppad + 2 || nzt < (fsurf ? ppad + fpad + 2 : 2 * ppad + 2))
            return fail(FWI_ERR_INVALID, "grid too small: need at least 2 interior cells per axis");
        if (!(dt > 0) || !(dx > 0) || !(dz > 0)) return fail(FWI_ERR_INVALID, "dt, dx, dz must be > 0");
        tp = 2 * (npml + 1);
        pitch = (int)round_up(nxt, 32);
        pnx = nxt - 2 * ppad + fpad - 1;
        // bottom CPML offset: the reference's for fdorder 2; with a free surface at
        // higher orders the offset keeps the layer on indices npml+1..2npml+1
        pnz = fsurf ? nzt - 2 * ppad + fpad - 2 : nzt - 2 * ppad + fpad - 1;
        cpml_h.assign(12 * (size_t)tp, 0.f);
        if (npml > 0) {
            if (!d->a || !d->b || !d->K || !d->a_half || !d->b_half || !d->K_half)
                return fail(FWI_ERR_INVALID, "CPML profiles are required when npml > 0");
            // Index npml is used by both the left and the right strip of the
            // stress pass (forward_kernel_PSV_GPU.cu:847-869); it must be the
            // identity (zero damping there), which cpml_pro yields for npower > 0.
            if (d->a[npml] != 0.0 || d->a_half[npml] != 0.0 || d->K[npml] != 1.0 ||
                d->K_half[npml] != 1.0)
                return fail(FWI_ERR_UNSUPPORTED,
                            "CPML profile index npml must be damping-free (npower > 0)");
            for (int i = 0; i < tp; i++) {
                cpml_h[0 * tp + i] = (float)d->a[i];
                cpml_h[1 * tp + i] = (float)d->b[i];
                cpml_h[2 * tp + i] = (float)(1.0 / d->K[i]);
                cpml_h[3 * tp + i] = (float)d->a_half[i];
                cpml_h[4 * tp + i] = (float)d->b_half[i];
                cpml_h[5 * tp + i] = (float)(1.0 / d->K_half[i]);
            }
            interleave_cpml(cpml_h.data(), tp);
        }
        field = (size_t)nzt * pitch;
        xstrip = round_up((size_t)nzt * tp, 32);
        zstrip = (size_t)tp * pitch;
        state = round_up(5 * field + 4 * xstrip + 4 * zstrip, 64);
        wx1 = 0; wx2 = nxt; wz1 = fsurf ? fpad : 0; wz2 = nzt;
        update_window();
        FWI_TRY(bind());
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        own_stream = true;
        ks = kernels_for(fpad, kmap);
        xs = exact_for(fpad);
        tset = tma_for(fpad);
        fset = fused_for(fpad);
        if (kmap == 3) CUDA_TRY(tset.prepare());
        if (kmap == 3 && fset.prepare) CUDA_TRY(fset.prepare());
        CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
        FWI_TRY(d_err.ensure(16));
        CUDA_TRY(cudaMemset(d_err.p, 0, 16));
        FWI_TRY(d_cpml.ensure(cpml_h.size() * sizeof(float) + 16));
        CUDA_TRY(cudaMemcpy(d_cpml.p, cpml_h.data(), cpml_h.size() * sizeof(float),
                            cudaMemcpyHostToDevice));
        return FWI_OK;
    }

    void update_window() {
        nft = 1 + (nt - 1) / fwi_dt;
        nfz = 1 + (wz2 - wz1) / fwi_dz;
        nfx = 1 + (wx2 - wx1) / fwi_dx;
        nf = (size_t)nfz * nfx;
    }

    // The exact adjoint always runs the checkpointed schedule, one time step per unit.
    bool exact() const { return grad_mode == FWI_GRAD_EXACT; }
    bool ckpt_mode() const { return strategy == FWI_STORE_BINOMIAL || exact(); }
    bool store_mode() const { return strategy == FWI_STORE_FULL && !exact(); }
    bool random_mode() const { return strategy == FWI_STORE_RANDOM && !exact(); }
    bool state_source() const { return ckpt_mode() || random_mode(); }  // gradient reads the forward state
    // The forward sweeps run the fused step (TMA mapping, fdorder <= 8; the
    // exact adjoint keeps its in-place two-pass steps).
    bool fused() const { return kmap == 3 && fuse && fset.step != nullptr && !exact(); }
    int unit() const { return exact() ? 1 : fwi_dt; }
    int nunits() const { return exact() ? nt : nft; }

    void invalidate_batch() {
        drop_graphs();
        for (auto& kv : tilesets) kv.second->ntiles = 0;
        B = 0;
        fwd_kept = false;
        bwd_done = false;
    }

    int set_model(const double* lam, const double* mu, const double* mu_zx, const double* rho_zp,
                  const double* rho_xp) {
        if (!lam || !mu || !mu_zx || !rho_zp || !rho_xp) return fail(FWI_ERR_INVALID, "null material array");
        FWI_TRY(bind());
        std::vector<float> h(5 * field, 0.f);
        zero_mu = false;
        for (int iz = fpad; iz < nzt - fpad; iz++)
            for (int ix = fpad; ix < nxt - fpad; ix++) zero_mu |= mu[(size_t)iz * nxt + ix] == 0.0;
        float* L = h.data();
        float* M2 = L + field;
        float* MZ = M2 + field;
        float* BXp = MZ + field;
        float* BZp = BXp + field;
        for (int iz = 0; iz < nzt; iz++)
            for (int ix = 0; ix < nxt; ix++) {
                const size_t o = (size_t)iz * pitch + ix, c = (size_t)iz * nxt + ix;
                L[o] = (float)(dt * lam[c]);
                M2[o] = (float)(2.0 * dt * mu[c]);
                if (iz < nzt - 1 && ix < nxt - 1) {
                    const size_t a = (size_t)iz * (nxt - 1) + ix;
                    MZ[o] = (float)(dt * mu_zx[a]);
                    BXp[o] = (float)(dt * rho_xp[a]);
                    BZp[o] = (float)(dt * rho_zp[a]);
                }
            }
        FWI_TRY(d_mat.ensure(h.size() * sizeof(float)));
        CUDA_TRY(cudaMemcpyAsync(d_mat.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice,
                                 stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        have_model = true;
        rb_valid = false;
        return FWI_OK;
    }

    // Raw FP64 models already on the device; averages and dt scaling by a kernel.
    int set_model_device(const double* dl, const double* dm, const double* dr) {
        if (!dl || !dm || !dr) return fail(FWI_ERR_INVALID, "null material array");
        FWI_TRY(bind());
        FWI_TRY(d_mat.ensure(5 * field * sizeof(float)));
        FWI_TRY(d_blow.ensure(16));
        CUDA_TRY(cudaMemsetAsync(d_mat.p, 0, 5 * field * sizeof(float), stream));
        CUDA_TRY(cudaMemsetAsync(d_blow.p, 0, 4, stream));
        const size_t n = (size_t)nzt * nxt;
        const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms * 8);
        materials_kernel<<<blocks, 256, 0, stream>>>(dl, dm, dr, nzt, nxt, pitch, fpad, dt, d_mat.as<float>(),
                                                     field, d_blow.as<int>());
        CUDA_TRY(cudaGetLastError());
        int z = 0;
        CUDA_TRY(cudaMemcpyAsync(&z, d_blow.p, 4, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        zero_mu = z != 0;
        have_model = true;
        rb_valid = false;
        return FWI_OK;
    }

    int set_sources(int n, const int* x, const int* z, const int* comp, const int* shot,
                    const double* sig) {
        if (n < 0 || (n > 0 && (!x || !z || !comp || !shot || !sig)))
            return fail(FWI_ERR_INVALID, "bad source arrays");
        for (int i = 0; i < n; i++)
            if (comp[i] == 2 && (x[i] < fpad || x[i] >= nxt - fpad || z[i] < fpad || z[i] >= nzt - fpad))
                return fail(FWI_ERR_INVALID, "source " + std::to_string(i) + " outside the interior");
        FWI_TRY(bind());
        nsrc = n;
        sx.assign(x, x + n); sz.assign(z, z + n); scomp.assign(comp, comp + n); sshot.assign(shot, shot + n);
        std::vector<float> s((size_t)std::max(n, 1) * nt, 0.f);
        for (size_t i = 0; i < (size_t)n * nt; i++) s[i] = (float)sig[i];
        FWI_TRY(d_srcsig.ensure(s.size() * sizeof(float)));
        CUDA_TRY(cudaMemcpy(d_srcsig.p, s.data(), s.size() * sizeof(float), cudaMemcpyHostToDevice));
        invalidate_batch();
        return FWI_OK;
    }

    int set_receivers(int n, const int* x, const int* z, const int* comp, const int* shot) {
        if (n < 0 || (n > 0 && (!x || !z || !comp || !shot)))
            return fail(FWI_ERR_INVALID, "bad receiver arrays");
        for (int i = 0; i < n; i++)
            if (comp[i] == 2 && (x[i] < fpad || x[i] >= nxt - fpad || z[i] < fpad || z[i] >= nzt - fpad))
                return fail(FWI_ERR_INVALID, "receiver " + std::to_string(i) + " outside the interior");
        nrec = n;
        rx.assign(x, x + n); rz.assign(z, z + n); rcomp.assign(comp, comp + n); rshot.assign(shot, shot + n);
        obs_valid = false;
        invalidate_batch();
        return FWI_OK;
    }

    int set_fwi(int fdt, int fdx, int fdz, int x1, int x2, int z1, int z2) {
        if (fdt < 1 || fdx < 1 || fdz < 1) return fail(FWI_ERR_INVALID, "FWI intervals must be >= 1");
        if (x1 < 0 || z1 < 0 || x2 > nxt || z2 > nzt || x2 <= x1 || z2 <= z1)
            return fail(FWI_ERR_INVALID, "FWI window outside the padded grid");
        // Above a free surface the reference correlates mirrored stresses; the
        // engine's gradient covers the rows from the surface down only.
        if (fsurf && z1 < fpad)
            return fail(FWI_ERR_UNSUPPORTED, "with a free surface the FWI window must start at row fpad or below");
        fwi_dt = fdt; fwi_dx = fdx; fwi_dz = fdz; wx1 = x1; wx2 = x2; wz1 = z1; wz2 = z2;
        update_window();
        invalidate_batch();
        return FWI_OK;
    }

    // ---- tiles -----------------------------------------------------------
    void plan_tiles(int nb, std::vector<Tile>& t) {
        const int nz_int = nzt - 2 * fpad;
        bx = kTileX;  // tile columns = threads per block
        const int ntx = (nxt + bx - 1) / bx;
        if (ks.map == 1 || ks.map == 2) {
            tz = ks.map == 1 ? MapDims<1>::rows : MapDims<2>::rows;  // one tile = one block's cells
        } else if (tz_req > 0) {
            tz = tz_req;
        } else {
            // about four tiles per resident block (load balance), rows >= 8
            const long long resident = (long long)num_sms * std::max(1, ks.occ_f());
            const long long per_shot = std::max<long long>(1, 4 * resident / std::max(1, nb));
            const long long ntz = std::max<long long>(1, per_shot / ntx);
            tz = (int)std::max<long long>(8, std::min<long long>(128, (nz_int + ntz - 1) / ntz));
        }
        t.clear();
        for (int x0 = 0; x0 < nxt; x0 += bx)
            for (int z0 = fpad; z0 < nzt - fpad; z0 += tz)
                for (int b = 0; b < nb; b++) t.push_back({b, x0, z0, std::min(z0 + tz, nzt - fpad)});
    }

    // ---- batch setup --------------------------------------------------------
    // Buffers are sized for the largest batch seen (Bcap) and never shrink, so
    // the device pointers captured in CUDA graphs stay valid for every smaller
    // batch; a graph is keyed by the batch shape (B, receiver rows, slots,
    // strategy), never by shot ids.  A reallocation drops all graphs.
    size_t batch_bytes(int nb, int nslots, int strat) const {
        size_t f = 4;
        size_t b = 0;
        b += (fused() ? 3 : 2) * (size_t)nb * state * f;  // fwd (+ second working buffer) + adj state
        b += 4 * (size_t)nb * field * f;        // ws, wr, ux, uz
        b += 3 * (size_t)nb * nf * f + 6 * nf * f;  // grads, sum, accumulator
        const bool ck = strat == FWI_STORE_BINOMIAL || (strat >= 0 && exact());
        if (strat == FWI_STORE_FULL && !ck) b += (size_t)nb * nft * 5 * nf * f;
        if (ck) b += (size_t)nslots * nb * state * f;
        if (exact()) b += (size_t)nb * (state + 9 * field) * f;  // state n+1, tmp + acc
        return b;
    }

    // grow a buffer whose address is captured in graphs
    int grow(DBuf& buf, size_t n) {
        if (buf.p && n <= buf.bytes) return FWI_OK;
        drop_graphs();
        return buf.ensure(n);
    }

    struct TileSet {
        DBuf buf;
        int ntiles = 0, bx = 0, tz = 0, grid_sf = 1, grid_sa = 1, grid_v = 1;
    };
    std::map<int, std::unique_ptr<TileSet>> tilesets;  // by batch size
    int Bcap = 0;
    size_t rows_cap = 0;
    DBuf d_obsf, d_rowrec, d_gacc;

    int tiles_for(int nb) {
        auto& ts = tilesets[nb];
        if (!ts) ts.reset(new TileSet());
        if (ts->ntiles == 0) {
            std::vector<Tile> t;
            plan_tiles(nb, t);
            FWI_TRY(grow(ts->buf, t.size() * sizeof(Tile)));
            CUDA_TRY(cudaMemcpyAsync(ts->buf.p, t.data(), t.size() * sizeof(Tile), cudaMemcpyHostToDevice,
                                     stream));
            ts->ntiles = (int)t.size();
            ts->bx = bx;
            ts->tz = tz;
            // persistent grids: resident capacity, never more blocks than tiles
            ts->grid_sf = std::max(1, std::min(ts->ntiles, num_sms * std::max(1, ks.occ_f())));
            ts->grid_sa = std::max(1, std::min(ts->ntiles, num_sms * std::max(1, ks.occ_a())));
            ts->grid_v = std::max(1, std::min(ts->ntiles, num_sms * std::max(1, ks.occ_v())));
        }
        ntiles = ts->ntiles;
        bx = ts->bx;
        tz = ts->tz;
        grid_sf = ts->grid_sf;
        grid_sa = ts->grid_sa;
        grid_v = ts->grid_v;
        d_tiles_p = ts->buf.as<Tile>();
        return FWI_OK;
    }
    const Tile* d_tiles_p = nullptr;

    int slots_for(int nb, bool keep, int* out) {
        *out = 0;
        if (!(keep && ckpt_mode())) return FWI_OK;
        size_t bud = budget;
        if (bud == 0) {
            size_t fr = 0, tot = 0;
            CUDA_TRY(cudaMemGetInfo(&fr, &tot));
            bud = (size_t)(0.9 * (double)(fr + allocated_bytes()));
        }
        const int cap = std::max(Bcap, nb);
        const size_t base = batch_bytes(cap, 0, FWI_STORE_BINOMIAL) + fixed_bytes();
        const size_t per_slot = (size_t)cap * state * 4;
        long long fit = bud > base ? (long long)((bud - base) / per_slot) : 0;
        int want = 0;
        if (snapshots_req > 0) {
            if (fit < std::min(snapshots_req, nunits() - 1))
                return fail(FWI_ERR_NOMEM, "budget too small for " + std::to_string(snapshots_req) +
                                               " checkpoints per shot");
            want = snapshots_req;
        } else {
            want = (int)std::min<long long>(fit, nunits() - 1);
        }
        *out = std::max(0, std::min(want, nunits() - 1));
        return FWI_OK;
    }

    int setup_batch(int nb, const int* ids, bool keep) {
        if (!have_model) return fail(FWI_ERR_STATE, "set a model first");
        if (nb < 1 || !ids) return fail(FWI_ERR_INVALID, "empty shot batch");
        int want_slots = 0;
        FWI_TRY(slots_for(nb, keep, &want_slots));
        const int cap = std::max(Bcap, nb);
        if (budget > 0 && batch_bytes(cap, want_slots, keep ? strategy : -1) + fixed_bytes() > budget)
            return fail(FWI_ERR_NOMEM, "batch does not fit the memory budget");
        // receiver rows of this batch
        std::vector<int> nrows_v, nslot_v;
        for (int b = 0; b < nb; b++)
            for (int r = 0; r < nrec; r++)
                if (rshot[r] == ids[b] && rcomp[r] == 2) {
                    nrows_v.push_back(r);
                    nslot_v.push_back(b);
                }
        const size_t nrows = nrows_v.size();
        // buffers (capacity; addresses captured in graphs)
        FWI_TRY(grow(d_fwd, (size_t)cap * state * 4));
        FWI_TRY(grow(d_adj, (size_t)cap * state * 4));
        if (fused()) {
            // the second working buffer: cells no step writes (grid borders) must
            // read as zero, so fresh memory is zeroed once
            const size_t before = d_fwd2.bytes;
            FWI_TRY(grow(d_fwd2, (size_t)cap * state * 4));
            if (d_fwd2.bytes != before) CUDA_TRY(cudaMemsetAsync(d_fwd2.p, 0, d_fwd2.bytes, stream));
        }
        FWI_TRY(grow(d_ws, (size_t)cap * field * 4));
        FWI_TRY(grow(d_wr, (size_t)cap * field * 4));
        FWI_TRY(grow(d_ux, (size_t)cap * field * 4));
        FWI_TRY(grow(d_uz, (size_t)cap * field * 4));
        FWI_TRY(grow(d_grad, (size_t)cap * 3 * nf * 4));
        FWI_TRY(grow(d_gsum, (size_t)3 * nf * 4));
        FWI_TRY(grow(d_gacc, (size_t)3 * nf * 4));
        if (keep && store_mode()) FWI_TRY(grow(d_store, (size_t)cap * nft * 5 * nf * 4));
        rb_active = keep && random_mode();
        if (rb_active && !rb_valid) {
            if (fsurf) return fail(FWI_ERR_UNSUPPORTED, "random boundaries need the model without a free surface");
            if (kmap != 3)
                return fail(FWI_ERR_UNSUPPORTED, "random-boundary reconstruction runs on the TMA mapping only");
            FWI_TRY(d_mat_rb.ensure(5 * field * sizeof(float)));
            drop_graphs();
            CUDA_TRY(cudaMemsetAsync(d_mat_rb.p, 0, 5 * field * sizeof(float), stream));
            const size_t n = (size_t)nzt * nxt;
            random_frame_kernel<<<(int)std::min<size_t>((n + 255) / 256, (size_t)num_sms * 8), 256, 0, stream>>>(
                d_mat.as<float>(), d_mat_rb.as<float>(), field, nzt, nxt, pitch, ppad, fsurf, rb_seed, rb_alpha);
            CUDA_TRY(cudaGetLastError());
            rb_valid = true;
        }
        if (keep && ckpt_mode() && want_slots > 0) {
            const size_t before = d_snap.bytes;  // ensure() only ever reallocates larger
            FWI_TRY(grow(d_snap, (size_t)want_slots * cap * state * 4));
            // the copy-free plan steps into any checkpoint buffer: cells that no
            // pass writes (grid borders) must read as zero there too.  Fresh
            // memory is zeroed once; everything written into it later is a
            // whole state, whose border cells are zero.
            if (d_snap.bytes != before) CUDA_TRY(cudaMemsetAsync(d_snap.p, 0, d_snap.bytes, stream));
        }
        if (exact()) {
            FWI_TRY(grow(d_nxt, (size_t)cap * state * 4));
            FWI_TRY(grow(d_exact, (size_t)cap * 9 * field * 4));
            FWI_TRY(grow(d_exd, (size_t)cap * sizeof(ExactDesc)));
            FWI_TRY(grow(d_items_n, (size_t)cap * sizeof(ItemDesc)));
        }
        rows_cap = std::max(rows_cap, std::max<size_t>(1, nrows));
        FWI_TRY(grow(d_rec, rows_cap * nt * 4));
        FWI_TRY(grow(d_resid, rows_cap * nt * 4));
        FWI_TRY(grow(d_rowmis, rows_cap * 8));
        FWI_TRY(grow(d_rowrec, rows_cap * 4));
        FWI_TRY(grow(d_blow, 16));
        FWI_TRY(grow(d_obsf, std::max<size_t>(1, (size_t)nrec) * nt * 4));
        FWI_TRY(grow(d_items_f, (size_t)cap * sizeof(ItemDesc)));
        if (keep && random_mode()) FWI_TRY(grow(d_items_rb, (size_t)cap * sizeof(ItemDesc)));
        nsnap = snap_interval > 0 ? 1 + (nt - 1) / snap_interval : 0;
        if (nsnap) FWI_TRY(grow(d_snapshots, (size_t)cap * nsnap * field * 4));
        FWI_TRY(grow(d_items_a, (size_t)cap * sizeof(ItemDesc)));
        Bcap = cap;
        B = nb;
        shots.assign(ids, ids + nb);
        slots = want_slots;
        rows = nrows_v;
        row_slot = nslot_v;
        fwd_kept = false;
        bwd_done = false;
        // events per slot, grouped by column, sorted by (z, inject-before-record, index)
        struct Ev { int x, z, kind, idx, code; };
        std::vector<int> colf((size_t)B * (nxt + 1)), cola((size_t)B * (nxt + 1));
        std::vector<int2> evf, eva;
        std::vector<int> evxf, evxa;
        for (int b = 0; b < B; b++) {
            std::vector<Ev> ef, ea;
            for (int i = 0; i < nsrc; i++)
                if (sshot[i] == shots[b] && scomp[i] == 2) ef.push_back({sx[i], sz[i], 0, i, i});
            for (size_t k = 0; k < nrows; k++)
                if (row_slot[k] == b) {
                    const int r = rows[k];
                    ef.push_back({rx[r], rz[r], 1, r, ~(int)k});
                    ea.push_back({rx[r], rz[r], 0, r, (int)k});
                }
            auto cmp = [](const Ev& u, const Ev& v) {
                if (u.x != v.x) return u.x < v.x;
                if (u.z != v.z) return u.z < v.z;
                if (u.kind != v.kind) return u.kind < v.kind;
                return u.idx < v.idx;
            };
            std::sort(ef.begin(), ef.end(), cmp);
            std::sort(ea.begin(), ea.end(), cmp);
            auto fill = [&](std::vector<Ev>& ev, std::vector<int>& col, std::vector<int2>& flat, std::vector<int>& fx) {
                const int base = (int)flat.size();
                int* c = col.data() + (size_t)b * (nxt + 1);
                size_t k = 0;
                for (int x = 0; x <= nxt; x++) {
                    while (k < ev.size() && ev[k].x < x) k++;
                    c[x] = base + (int)k;
                }
                for (auto& e : ev) {
                    flat.push_back(make_int2(e.z, e.code));
                    fx.push_back(e.x);
                }
            };
            fill(ef, colf, evf, evxf);
            fill(ea, cola, eva, evxa);
        }
        // event tables are reached through the item descriptors only (not captured)
        FWI_TRY(d_evcol_f.ensure(colf.size() * 4));
        FWI_TRY(d_evcol_a.ensure(cola.size() * 4));
        FWI_TRY(d_ev_f.ensure(std::max<size_t>(1, evf.size()) * 8));
        FWI_TRY(d_ev_a.ensure(std::max<size_t>(1, eva.size()) * 8));
        FWI_TRY(d_evx_f.ensure(std::max<size_t>(1, evxf.size()) * 4));
        FWI_TRY(d_evx_a.ensure(std::max<size_t>(1, evxa.size()) * 4));
        if (!evxf.empty())
            CUDA_TRY(cudaMemcpyAsync(d_evx_f.p, evxf.data(), evxf.size() * 4, cudaMemcpyHostToDevice, stream));
        if (!evxa.empty())
            CUDA_TRY(cudaMemcpyAsync(d_evx_a.p, evxa.data(), evxa.size() * 4, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(d_evcol_f.p, colf.data(), colf.size() * 4, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(d_evcol_a.p, cola.data(), cola.size() * 4, cudaMemcpyHostToDevice, stream));
        if (!evf.empty())
            CUDA_TRY(cudaMemcpyAsync(d_ev_f.p, evf.data(), evf.size() * 8, cudaMemcpyHostToDevice, stream));
        if (!eva.empty())
            CUDA_TRY(cudaMemcpyAsync(d_ev_a.p, eva.data(), eva.size() * 8, cudaMemcpyHostToDevice, stream));
        if (nrows)
            CUDA_TRY(cudaMemcpyAsync(d_rowrec.p, rows.data(), nrows * 4, cudaMemcpyHostToDevice, stream));
        std::vector<ItemDesc> itf(B), ita(B), itn(B), itr(B);
        std::vector<ExactDesc> exd(B);
        for (int b = 0; b < B; b++) {
            fill_item(itf[b], b, false);
            fill_item(ita[b], b, true);
            if (rb_active) fill_item(itr[b], b, false, nullptr, true);
            if (exact()) {
                fill_item(itn[b], b, false, d_nxt.as<float>());
                ExactDesc& x = exd[b];
                x.tmp = d_exact.as<float>() + (size_t)b * 9 * field;
                x.acc = x.tmp + 4 * field;
                x.next = d_nxt.as<float>() + (size_t)b * state;
                x.src_col = itf[b].ev_col;
                x.src_ev = itf[b].ev;
                x.src_sig = d_srcsig.as<float>();
                x.field = (long long)field;
            }
        }
        if (copy_free() || fused()) {
            const int nbuf = nbufs();
            std::vector<ItemDesc> itb((size_t)nbuf * B);
            for (int k = 0; k < nbuf; k++)
                for (int b = 0; b < B; b++) fill_item(itb[(size_t)k * B + b], b, false, buf(k));
            FWI_TRY(grow(d_items_b, itb.size() * sizeof(ItemDesc)));
            CUDA_TRY(cudaMemcpyAsync(d_items_b.p, itb.data(), itb.size() * sizeof(ItemDesc), cudaMemcpyHostToDevice,
                                     stream));
        }
        CUDA_TRY(cudaMemcpyAsync(d_items_f.p, itf.data(), B * sizeof(ItemDesc), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(d_items_a.p, ita.data(), B * sizeof(ItemDesc), cudaMemcpyHostToDevice, stream));
        if (rb_active)
            CUDA_TRY(cudaMemcpyAsync(d_items_rb.p, itr.data(), B * sizeof(ItemDesc), cudaMemcpyHostToDevice, stream));
        if (exact()) {
            CUDA_TRY(cudaMemcpyAsync(d_items_n.p, itn.data(), B * sizeof(ItemDesc), cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaMemcpyAsync(d_exd.p, exd.data(), B * sizeof(ExactDesc), cudaMemcpyHostToDevice, stream));
        }
        FWI_TRY(tiles_for(B));
        if (kmap == 3) FWI_TRY(build_tma_maps());
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (keep && ckpt_mode()) plan = plan_binomial(nunits(), slots, &plan_cost);
        return FWI_OK;
    }
    // Maps of the fused step, per buffer it can read from.
    int build_fused_maps() {
        using G = FusedGeom<1>;  // box widths do not depend on the order; the heights do
        const int vz_rows = kFusedTZ + 2 * fpad;
        const size_t rb = (size_t)pitch * 4, sb = state * 4;
        const float* mat = d_mat.as<float>();
        const int nbuf = nbufs();
        fmaps_b.assign(nbuf, FusedMaps{});
        for (int k = 0; k < nbuf; k++) {
            float* st = buf(k);
            const int nb = k < slots ? B : Bcap;  // a checkpoint buffer holds B states
            FusedMaps& F = fmaps_b[k];
            FWI_TRY(make_map(&F.vx, st + F_VX * field, nxt, nzt, nb, rb, sb, G::VX, vz_rows));
            FWI_TRY(make_map(&F.vz, st + F_VZ * field, nxt, nzt, nb, rb, sb, G::VX, vz_rows));
            FWI_TRY(make_map(&F.sxx, st + F_SXX * field, nxt, nzt, nb, rb, sb, G::SX, kFusedTZ));
            FWI_TRY(make_map(&F.szx, st + F_SZX * field, nxt, nzt, nb, rb, sb, G::SX, kFusedTZ));
            FWI_TRY(make_map(&F.szz, st + F_SZZ * field, nxt, nzt, nb, rb, sb, G::SX, kFusedTZ));
            FWI_TRY(make_map(&F.L, mat, nxt, nzt, 0, rb, 0, G::SX, kFusedTZ));
            FWI_TRY(make_map(&F.M2, mat + field, nxt, nzt, 0, rb, 0, G::SX, kFusedTZ));
            FWI_TRY(make_map(&F.MZ, mat + 2 * field, nxt, nzt, 0, rb, 0, G::SX, kFusedTZ));
            FWI_TRY(make_map(&F.BX, mat + 3 * field, nxt, nzt, 0, rb, 0, G::W, kFusedTZ));
            FWI_TRY(make_map(&F.BZ, mat + 4 * field, nxt, nzt, 0, rb, 0, G::W, kFusedTZ));
        }
        return FWI_OK;
    }

    // One fused forward step of the batch from the state of step `it` in buffer
    // x to the state of step it+1 in buffer y (x != y), then the source/receiver
    // events on y.
    void fused_step(int x, int y, int it, unsigned flags, unsigned ev) {
        FusedGrid fg = fgrid;
        fg.msrc = (long long)(buf(x) - buf(y));
        fg.stall = stall_pending ? 1 : 0;
        stall_pending = false;
        const ItemDesc* items = d_items_b.as<ItemDesc>() + (size_t)y * B;
        fset.step(dim3(grid_fused), stream, fmaps_b[x], items, fg, it, flags, d_err.as<int>());
        launches_now++;
        if (ev) {
            events_kernel<<<B, 256, 0, stream>>>(items, it, ev);
            launches_now++;
        }
    }
    // Recording forward steps [t0, t1) with the fused step, the state moving
    // between the two working buffers (*cur: the one holding it); snapshots as
    // forward_steps takes them.
    void fused_steps(int t0, int t1, int* cur, bool record, bool store) {
        for (int it = t0; it < t1; it++) {
            const int other = *cur == slots ? slots + 1 : slots;
            const unsigned f = ((store && it % fwi_dt == 0) ? FL_STORE : 0u) | (record ? FL_WE : 0u);
            fused_step(*cur, other, it, f, FL_INJECT | (record ? FL_RECORD : 0u));
            *cur = other;
            if (record) watch(t0, it);
            if (record && snap_interval > 0 && it % snap_interval == 0) {
                const int k = it / snap_interval;
                for (int b = 0; b < B; b++)
                    cudaMemcpyAsync(d_snapshots.as<float>() + ((size_t)b * nsnap + k) * field,
                                    buf(*cur) + (size_t)b * state + (size_t)snap_field * field, field * 4,
                                    cudaMemcpyDeviceToDevice, stream);
            }
        }
    }

    // Tensor maps of the TMA passes for the current buffers (addresses are
    // captured by value in the launches; buffers only grow, and a regrowth
    // drops every graph, so maps are rebuilt here with each batch layout).
    int build_tma_maps() {
        const int FPv = fpad;
        const int hx = (FPv + 3) / 4 * 4;
        const int wx = kTmaTX + 2 * hx, wz = kTmaTZ + 2 * FPv;
        const size_t rb = (size_t)pitch * 4, sb = state * 4;
        float* bases[4] = {d_fwd.as<float>(), d_adj.as<float>(), d_nxt.p ? d_nxt.as<float>() : nullptr,
                           rb_active ? d_fwd.as<float>() : nullptr};
        float* webase[4] = {d_ws.as<float>(), d_wr.as<float>(), d_ws.as<float>(), d_ws.as<float>()};
        for (int w = 0; w < 4; w++) {
            float* st = bases[w];
            if (!st) continue;
            const float* mat = w == 3 ? d_mat_rb.as<float>() : d_mat.as<float>();
            StressMaps& S = smaps[w];
            FWI_TRY(make_map(&S.vx, st + F_VX * field, nxt, nzt, Bcap, rb, sb, wx, wz));
            FWI_TRY(make_map(&S.vz, st + F_VZ * field, nxt, nzt, Bcap, rb, sb, wx, wz));
            FWI_TRY(make_map(&S.L, mat, nxt, nzt, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&S.M2, mat + field, nxt, nzt, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&S.MZ, mat + 2 * field, nxt, nzt, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&S.sxx, st + F_SXX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&S.szx, st + F_SZX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&S.szz, st + F_SZZ * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kTmaTZ));
            VelMaps& V = vmaps[w];
            FWI_TRY(make_map(&V.sxx, st + F_SXX * field, nxt, nzt, Bcap, rb, sb, wx, kTmaTZ));
            FWI_TRY(make_map(&V.szx, st + F_SZX * field, nxt, nzt, Bcap, rb, sb, wx, wz));
            FWI_TRY(make_map(&V.szz, st + F_SZZ * field, nxt, nzt, Bcap, rb, sb, kTmaTX, wz));
            FWI_TRY(make_map(&V.BX, mat + 3 * field, nxt, nzt, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&V.BZ, mat + 4 * field, nxt, nzt, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&V.vx, st + F_VX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&V.vz, st + F_VZ * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&V.We, webase[w], nxt, nzt, Bcap, rb, field * 4, kTmaTX, kTmaTZ));
        }
        {
            // adjoint stress pass (128 x 8 tiles): adjoint state, ux/uz, forward state
            const float* mat = d_mat.as<float>();
            const int wza = kAdjTZ + 2 * FPv;
            float* a = d_adj.as<float>();
            float* f = d_fwd.as<float>();
            const size_t fb = field * 4;
            AdjMaps& A = amap;
            FWI_TRY(make_map(&A.vx, a + F_VX * field, nxt, nzt, Bcap, rb, sb, wx, wza));
            FWI_TRY(make_map(&A.vz, a + F_VZ * field, nxt, nzt, Bcap, rb, sb, wx, wza));
            FWI_TRY(make_map(&A.L, mat, nxt, nzt, 0, rb, 0, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.M2, mat + field, nxt, nzt, 0, rb, 0, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.MZ, mat + 2 * field, nxt, nzt, 0, rb, 0, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.sxx, a + F_SXX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.szx, a + F_SZX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.szz, a + F_SZZ * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.ux, d_ux.as<float>(), nxt, nzt, Bcap, rb, fb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.uz, d_uz.as<float>(), nxt, nzt, Bcap, rb, fb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fvx, f + F_VX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fvz, f + F_VZ * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fsxx, f + F_SXX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fszx, f + F_SZX * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fszz, f + F_SZZ * field, nxt, nzt, Bcap, rb, sb, kTmaTX, kAdjTZ));
        }
        if (copy_free() || fused()) {
            const int nbuf = nbufs();
            smaps_b.assign(nbuf, smaps[0]);
            vmaps_b.assign(nbuf, vmaps[0]);
            amaps_b.assign(nbuf, amap);
            const int wza = kAdjTZ + 2 * FPv;
            for (int k = 0; k < nbuf; k++) {
                float* st = buf(k);
                const int nb = k < slots ? B : Bcap;  // a checkpoint buffer holds B states
                StressMaps& S = smaps_b[k];
                FWI_TRY(make_map(&S.vx, st + F_VX * field, nxt, nzt, nb, rb, sb, wx, wz));
                FWI_TRY(make_map(&S.vz, st + F_VZ * field, nxt, nzt, nb, rb, sb, wx, wz));
                FWI_TRY(make_map(&S.sxx, st + F_SXX * field, nxt, nzt, nb, rb, sb, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&S.szx, st + F_SZX * field, nxt, nzt, nb, rb, sb, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&S.szz, st + F_SZZ * field, nxt, nzt, nb, rb, sb, kTmaTX, kTmaTZ));
                VelMaps& V = vmaps_b[k];
                FWI_TRY(make_map(&V.sxx, st + F_SXX * field, nxt, nzt, nb, rb, sb, wx, kTmaTZ));
                FWI_TRY(make_map(&V.szx, st + F_SZX * field, nxt, nzt, nb, rb, sb, wx, wz));
                FWI_TRY(make_map(&V.szz, st + F_SZZ * field, nxt, nzt, nb, rb, sb, kTmaTX, wz));
                FWI_TRY(make_map(&V.vx, st + F_VX * field, nxt, nzt, nb, rb, sb, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&V.vz, st + F_VZ * field, nxt, nzt, nb, rb, sb, kTmaTX, kTmaTZ));
                AdjMaps& A = amaps_b[k];
                FWI_TRY(make_map(&A.fvx, st + F_VX * field, nxt, nzt, nb, rb, sb, kTmaTX, kAdjTZ));
                FWI_TRY(make_map(&A.fvz, st + F_VZ * field, nxt, nzt, nb, rb, sb, kTmaTX, kAdjTZ));
                FWI_TRY(make_map(&A.fsxx, st + F_SXX * field, nxt, nzt, nb, rb, sb, kTmaTX, kAdjTZ));
                FWI_TRY(make_map(&A.fszx, st + F_SZX * field, nxt, nzt, nb, rb, sb, kTmaTX, kAdjTZ));
                FWI_TRY(make_map(&A.fszz, st + F_SZZ * field, nxt, nzt, nb, rb, sb, kTmaTX, kAdjTZ));
                (void)wza;
            }
        }
        if (fused()) FWI_TRY(build_fused_maps());
        const int ntx = (nxt + kTmaTX - 1) / kTmaTX;
        const int ntz = (nzt - 2 * fpad + kTmaTZ - 1) / kTmaTZ;
        tgrid.nb = B;
        tgrid.ntz = ntz;
        tgrid.ntiles = B * ntz * ntx;
        // plain-stencil cells of both forward passes (the CPML rule also covers
        // the random-frame sweeps, which have no strips)
        tgrid.cxl = fpad;
        tgrid.cxh = nxt - fpad - 1;
        tgrid.czl = fpad;
        tgrid.czh = nzt - fpad - 1;
        if (npml > 0) {
            tgrid.cxl = std::max(tgrid.cxl, ppad + 1);
            tgrid.cxh = std::min(tgrid.cxh, nxt - ppad - 2);
            tgrid.czh = std::min(tgrid.czh, nzt - ppad - 2);
            if (!fsurf) tgrid.czl = std::max(tgrid.czl, ppad + 1);
        }
        if (fsurf) tgrid.czl = std::max(tgrid.czl, 2 * fpad + 1);
        tgrid.gxl = tgrid.gzl = 0;
        tgrid.gxh = tgrid.gzh = -1;
        if (fwi_dx == 1 && fwi_dz == 1) {
            tgrid.gxl = wx1;
            tgrid.gxh = wx2 - 1;
            tgrid.gzl = wz1;
            tgrid.gzh = wz2 - 1;
        }
        tgrid.wait_ns = wait_ns;
        grid_tma = std::max(1, std::min(tgrid.ntiles, num_sms));
        if (fused()) {
            constexpr int Wf = FusedGeom<1>::W;  // owned columns per strip (the same for fdorder 2..8)
            fgrid.nb = B;
            fgrid.nunits = B * ((nxt + Wf - 1) / Wf);
            fgrid.nch = (nzt - fpad + kFusedTZ - 1) / kFusedTZ;
            fgrid.cxl = tgrid.cxl;
            fgrid.cxh = tgrid.cxh;
            fgrid.czl = tgrid.czl;
            fgrid.czh = tgrid.czh;
            fgrid.msrc = 0;
            fgrid.wait_ns = wait_ns;
            grid_fused = std::max(1, std::min(fgrid.nunits, num_sms));
        }
        const int ntz_a = (nzt - 2 * fpad + kAdjTZ - 1) / kAdjTZ;
        tgrid_a = tgrid;
        tgrid_a.ntz = ntz_a;
        tgrid_a.ntiles = B * ntz_a * ntx;
        grid_tma_a = std::max(1, std::min(tgrid_a.ntiles, num_sms));
        return FWI_OK;
    }

    // Forward stress and velocity passes of one state buffer (0 fwd, 1 adj, 2 state n+1).
    void pass_stress_fwd(int w, const ItemDesc* items, int it, unsigned flags) {
        if (kmap == 3) {
            TmaGrid g = tgrid;
            g.stall = stall_pending ? 1 : 0;
            stall_pending = false;
            tset.stress(dim3(grid_tma), stream, smaps[w], items, g, it, flags, d_err.as<int>());
        } else {
            ks.stress_f(dim3(grid_sf), stream, items, d_tiles_p, ntiles, it, flags, d_err.as<int>());
        }
    }
    void pass_velocity(int w, const ItemDesc* items, int it, unsigned flags) {
        if (kmap == 3) {
            const unsigned ev = flags & (FL_INJECT | FL_RECORD);
            tset.velocity(dim3(grid_tma), stream, vmaps[w], items, tgrid, it, flags & ~ev, d_err.as<int>());
            if (ev) {
                events_kernel<<<B, 256, 0, stream>>>(items, it, ev);
                launches_now++;
            }
        } else {
            ks.velocity(dim3(grid_v), stream, items, d_tiles_p, ntiles, it, flags, d_err.as<int>());
        }
    }

    std::string shape_key() const {
        return "|B" + std::to_string(B) + "|r" + std::to_string(rows.size()) + "|s" +
               std::to_string(slots) + "|st" + std::to_string(strategy) + "|t" + std::to_string(ntiles) +
               "|g" + std::to_string(grad_on ? 1 : 0) + "|m" + std::to_string(grad_mode) + "|rb" +
               std::to_string(rb_active ? 1 : 0) + "|fu" + std::to_string(fused() ? 1 : 0) + "|sn" +
               std::to_string(snap_interval) + "." + std::to_string(snap_field);
    }

    // FP64 host observed data -> resident FP32 rows [nrec][nt] for the given receivers.
    int upload_obs(const double* obs, const std::vector<int>& recs) {
        if (recs.empty()) return FWI_OK;
        FWI_TRY(grow(d_obsf, std::max<size_t>(1, (size_t)nrec) * nt * 4));
        FWI_TRY(h_stage.ensure(recs.size() * nt * 4));
        float* o = h_stage.as<float>();
        for (size_t k = 0; k < recs.size(); k++)
            for (int t = 0; t < nt; t++) o[k * nt + t] = (float)obs[(size_t)recs[k] * nt + t];
        // one copy per run of consecutive receiver indices
        size_t k = 0;
        while (k < recs.size()) {
            size_t j = k + 1;
            while (j < recs.size() && recs[j] == recs[j - 1] + 1) j++;
            CUDA_TRY(cudaMemcpyAsync(d_obsf.as<float>() + (size_t)recs[k] * nt, o + k * nt,
                                     (j - k) * nt * 4, cudaMemcpyHostToDevice, stream));
            k = j;
        }
        CUDA_TRY(cudaStreamSynchronize(stream));
        obs_valid = true;
        last_h2d = (int64_t)(recs.size() * nt * 4);
        return FWI_OK;
    }
    int64_t last_h2d = 0;

    size_t fixed_bytes() const { return d_mat.bytes + d_cpml.bytes + d_srcsig.bytes; }
    size_t allocated_bytes() const {
        size_t t = d_fwd.bytes + d_fwd2.bytes + d_adj.bytes + d_ws.bytes + d_wr.bytes + d_ux.bytes + d_uz.bytes +
                   d_grad.bytes + d_gsum.bytes + d_gacc.bytes + d_store.bytes + d_snap.bytes +
                   d_rec.bytes + d_obsf.bytes + d_resid.bytes + d_nxt.bytes + d_exact.bytes;
        return t;
    }

    void fill_item(ItemDesc& d, int b, bool adj, float* state_base = nullptr, bool rbf = false) {
        std::memset(&d, 0, sizeof d);
        d.nzt = nzt; d.nxt = nxt; d.pitch = pitch; d.fpad = fpad;
        d.ppad = ppad; d.npml = npml; d.tp = tp; d.pnx = pnx;
        d.pnz = pnz; d.fsurf = fsurf; d.nt = nt; d.fwi_dt = fwi_dt;
        d.fwi_dx = fwi_dx; d.fwi_dz = fwi_dz; d.wx1 = wx1; d.wx2 = wx2;
        d.wz1 = wz1; d.wz2 = wz2; d.nfz = nfz; d.nfx = nfx;
        d.dt = (float)dt;
        d.inv_dt = (float)(1.0 / dt);
        d.gscale = (float)(fwi_dt * dt);
        for (int k = 0; k < kMaxHalf; k++) {
            d.hx[k] = k < fpad ? (float)((1.0 / dx) * hc[k + 1]) : 0.f;
            d.hz[k] = k < fpad ? (float)((1.0 / dz) * hc[k + 1]) : 0.f;
        }
        d.cpml = d_cpml.as<float>();
        // the random-boundary forward: frame materials, no CPML
        if (rbf) d.npml = 0;
        const float* m = rbf ? d_mat_rb.as<float>() : d_mat.as<float>();
        d.L = m; d.M2 = m + field; d.MZX = m + 2 * field; d.BX = m + 3 * field; d.BZ = m + 4 * field;
        float* st = (state_base ? state_base : adj ? d_adj.as<float>() : d_fwd.as<float>()) + (size_t)b * state;
        d.vx = st + F_VX * field; d.vz = st + F_VZ * field; d.sxx = st + F_SXX * field;
        d.szx = st + F_SZX * field; d.szz = st + F_SZZ * field;
        float* cp = st + 5 * field;
        d.mvx_x = cp; d.mvz_x = cp + xstrip; d.msxx_x = cp + 2 * xstrip; d.mszx_x = cp + 3 * xstrip;
        float* zp = cp + 4 * xstrip;
        d.mvx_z = zp; d.mvz_z = zp + zstrip; d.mszz_z = zp + 2 * zstrip; d.mszx_z = zp + 3 * zstrip;
        d.We = (adj ? d_wr.as<float>() : d_ws.as<float>()) + (size_t)b * field;
        d.ev_col = (adj ? d_evcol_a.as<int>() : d_evcol_f.as<int>()) + (size_t)b * (nxt + 1);
        d.ev = adj ? d_ev_a.as<int2>() : d_ev_f.as<int2>();
        d.ev_x = adj ? d_evx_a.as<int>() : d_evx_f.as<int>();
        d.inj = adj ? d_resid.as<float>() : d_srcsig.as<float>();
        d.rec = d_rec.as<float>();
        d.store = d_store.p ? d_store.as<float>() + (size_t)b * nft * 5 * nf : nullptr;
        if (adj) {
            d.ux = d_ux.as<float>() + (size_t)b * field;
            d.uz = d_uz.as<float>() + (size_t)b * field;
            d.glam = d_grad.as<float>() + (size_t)b * 3 * nf;
            d.gmu = d.glam + nf;
            d.grho = d.gmu + nf;
            if (state_source()) {
                d.fwd_kind = 1;
                d.fwd = d_fwd.as<float>() + (size_t)b * state;
                d.fwd_fs = (long long)field;
            } else {
                d.fwd_kind = 0;
                d.fwd = d.store;
            }
        }
    }

    // ---- launches ----------------------------------------------------------
    // Adjoint stress pass with the reference gradient; the TMA kernel reads the
    // forward fields from the checkpointed working state (fwd_kind 1).
    void pass_stress_adj(const ItemDesc* items, int it, unsigned flags) {
        if (kmap == 3 && state_source())
            tset.adjoint(dim3(grid_tma_a), stream, amap_cur ? *amap_cur : amap, items, tgrid_a, it, flags,
                         d_err.as<int>());
        else
            ks.stress_a(dim3(grid_sa), stream, items, d_tiles_p, ntiles, it, flags, d_err.as<int>());
    }
    void step(bool adj, int it, unsigned sflags, unsigned vflags) {
        const ItemDesc* items = adj ? d_items_a.as<ItemDesc>() : d_items_f.as<ItemDesc>();
        if (adj) pass_stress_adj(items, it, sflags);
        else pass_stress_fwd(0, items, it, sflags);
        pass_velocity(adj ? 1 : 0, items, it, vflags);
        launches_now += 2;
    }

    // Watchdog after recording step `it` (the recording sweep runs steps 0 ..
    // nt-1 in order): every kWatchSteps steps and at the last step, the traces
    // recorded since the previous check are scanned for NaN / Inf.
    void watch(int t0, int it) {
        (void)t0;
        const int done = it + 1;
        if (rows.empty() || (done % kWatchSteps != 0 && done != nt)) return;
        const int a = done - (done % kWatchSteps ? done % kWatchSteps : kWatchSteps);
        const size_t n = rows.size() * (size_t)(it + 1 - a);
        const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms * 4);
        watch_traces_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(d_rec.as<float>(), (int)rows.size(), nt, a,
                                                                     it + 1, d_err.as<int>());
        launches_now++;
    }

    // Error flags raised by the kernels: bit 4 a bounded wait that ran out
    // (bit 8 misaligned shared memory), bit 16 the watchdog's non-finite values.
    int check_kernel_flags() {
        FWI_TRY(check_bounds_record());
        int h = 0;
        CUDA_TRY(cudaMemcpy(&h, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) {
            CUDA_TRY(cudaMemset(d_err.p, 0, sizeof(int)));
            if (h & 16)
                return fail(FWI_ERR_DIVERGED, "non-finite values in the recorded traces or the gradients "
                                              "(device watchdog); results discarded");
            return fail(FWI_ERR_CUDA, "a kernel's shared-memory pipeline wait timed out (flag " +
                                          std::to_string(h) + "); results discarded");
        }
        return FWI_OK;
    }

    // forward steps [t0, t1) of the working forward state; the recording sweep
    // also takes the snapshots (after the step, as the reference writes them)
    void forward_steps(int t0, int t1, bool record, bool store) {
        for (int it = t0; it < t1; it++) {
            unsigned sf = (store && it % fwi_dt == 0) ? FL_STORE : 0u;
            unsigned vf = FL_INJECT | (record ? (FL_RECORD | FL_WE) : 0u);
            step(false, it, sf, vf);
            if (record) watch(t0, it);
            if (record && snap_interval > 0 && it % snap_interval == 0) {
                const int k = it / snap_interval;
                for (int b = 0; b < B; b++)
                    cudaMemcpyAsync(d_snapshots.as<float>() + ((size_t)b * nsnap + k) * field,
                                    d_fwd.as<float>() + (size_t)b * state + (size_t)snap_field * field,
                                    field * 4, cudaMemcpyDeviceToDevice, stream);
            }
        }
    }
    // adjoint steps t1-1 down to t0 (inclusive), gradient at sampled steps
    void adjoint_steps(int t0, int t1) {
        for (int it = t1 - 1; it >= t0; it--) {
            unsigned sf = (grad_on && it % fwi_dt == 0) ? FL_GRAD : 0u;
            step(true, it, sf, FL_INJECT | FL_WE);
        }
    }
    // One reverse step of the exact discrete adjoint at time step n: the
    // working forward state (d_fwd) holds state n; state n+1 is made from it
    // in d_nxt by one more forward step, then the four transposed passes run.
    int exact_step(int n) {
        FWI_TRY(state_copy(d_nxt.as<float>(), d_fwd.as<float>()));
        const ItemDesc* itn = d_items_n.as<ItemDesc>();
        pass_stress_fwd(2, itn, n, 0u);
        pass_velocity(2, itn, n, FL_INJECT);
        const long long cells = (long long)(nzt - 2 * fpad) * (nxt - 2 * fpad);
        const dim3 g((unsigned)((cells + kExactThreads - 1) / kExactThreads), (unsigned)B);
        const ItemDesc* ia = d_items_a.as<ItemDesc>();
        const ExactDesc* ex = d_exd.as<ExactDesc>();
        xs.vel_local(g, stream, ia, ex, B, n, cells);
        xs.vel_stencil(g, stream, ia, ex, B, n, cells);
        xs.str_local(g, stream, ia, ex, B, n, cells);
        xs.str_stencil(g, stream, ia, ex, B, n, cells);
        launches_now += 6;
        return FWI_OK;
    }
    // Forward steps the backward runs for the plan (in units of fwi_dt): from
    // the last checkpoint of the first sweep (placed by forward()) to the last
    // unit, then every ADVANCE after that prefix, plus state n+1 of each exact
    // reverse step.  The same count whether the plan runs directly or as a
    // replayed graph.
    long long plan_recompute() const { return plan_recompute_steps(plan, nunits(), exact()); }
    int state_copy(float* dst, const float* src) {
        CUDA_TRY(device_copy(dst, src, (size_t)B * state, num_sms, stream));
        launches_now++;
        return FWI_OK;
    }
    float* snap(int slot) { return d_snap.as<float>() + (size_t)slot * B * state; }
    // The binomial plan runs without state copies on the TMA mapping (the
    // other mappings and the exact adjoint copy states in and out of slots).
    bool copy_free() const { return kmap == 3 && ckpt_mode() && !exact() && slots > 0; }
    float* buf(int k) { return k < slots ? snap(k) : k == slots ? d_fwd.as<float>() : d_fwd2.as<float>(); }
    // Buffers a step can read or write: the checkpoint slots, d_fwd and, for
    // the fused step, d_fwd2.
    int nbufs() const { return slots + (fused() ? 2 : 1); }
    // One recompute step (stress, velocity, source injection) from the state
    // of step `it` in buffer x to the state of step it+1 in buffer y (x == y:
    // in place).  Out of place, the stress pass reads velocities and
    // stresses from x and writes the stresses to y; the velocity pass reads
    // those stresses from y and the velocities from x; CPML memories are read
    // from x and written to y.
    void step_bufs(int x, int y, int it) {
        TmaGrid gg = tgrid;
        gg.msrc = (long long)(buf(x) - buf(y));
        const ItemDesc* items = d_items_b.as<ItemDesc>() + (size_t)y * B;
        tset.stress(dim3(grid_tma), stream, smaps_b[x], items, gg, it, 0u, d_err.as<int>());
        VelMaps vm = vmaps_b[x];
        vm.sxx = vmaps_b[y].sxx;
        vm.szx = vmaps_b[y].szx;
        vm.szz = vmaps_b[y].szz;
        tset.velocity(dim3(grid_tma), stream, vm, items, gg, it, 0u, d_err.as<int>());
        events_kernel<<<B, 256, 0, stream>>>(items, it, FL_INJECT);
        launches_now += 3;
    }

    // Run `body` directly or as a cached CUDA graph.
    template <class F>
    int run_phase(const std::string& key, F&& body) {
        if (!use_graphs) {
            FWI_TRY(body());
            CUDA_TRY(cudaGetLastError());
            return FWI_OK;
        }
        auto itg = graphs.find(key);
        if (itg == graphs.end()) {
            const int64_t before = launches_now;
            CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            int st = body();
            cudaGraph_t g = nullptr;
            cudaError_t ec = cudaStreamEndCapture(stream, &g);
            if (st != FWI_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (ec != cudaSuccess) return fail(FWI_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
            cudaGraphExec_t ex = nullptr;
            ec = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (ec != cudaSuccess) return fail(FWI_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ec));
            itg = graphs.emplace(key, ex).first;
            graph_launches[key] = launches_now - before;
            launches_now = before;
        }
        launches_now += graph_launches[key];
        CUDA_TRY(cudaGraphLaunch(itg->second, stream));
        return FWI_OK;
    }
    std::map<std::string, int64_t> graph_launches;

    // ---- forward -------------------------------------------------------------
    int forward(int nb, const int* ids, const double* obs_in, double* rec_out, double* misfit, int flags) {
        FWI_TRY(bind());
        const int keep = flags & FWI_FWD_KEEP;
        const bool resident = (flags & FWI_FWD_RESIDENT_OBS) != 0;
        FWI_TRY(setup_batch(nb, ids, keep != 0));
        if (resident && !obs_valid)
            return fail(FWI_ERR_STATE, "no observed data resident on the device");
        const size_t nrows = rows.size();
        const bool obs = resident || obs_in != nullptr;  // misfit + residual wanted
        last_h2d = 0;
        if (obs_in && !resident) FWI_TRY(upload_obs(obs_in, rows));
        cudaEvent_t e0, e1;
        CUDA_TRY(cudaEventCreate(&e0));
        CUDA_TRY(cudaEventCreate(&e1));
        launches_now = 0;
        CUDA_TRY(cudaEventRecord(e0, stream));
        const bool store = keep && store_mode();
        const bool ckpt = keep && ckpt_mode();
        // checkpoint positions of the first sweep: the SAVE actions before the first ADJOINT
        std::vector<std::pair<int, int>> saves;  // (state, slot)
        if (ckpt)
            for (auto& a : plan) {
                if (a.kind == Action::ADJOINT) break;
                if (a.kind == Action::SAVE) saves.push_back({a.b, a.a});
            }
        stall_pending = stall_next && (fused() || (kmap == 3 && !exact()));
        stall_next = false;
        const std::string key = std::string("fwd") + (store ? "S" : "") + (ckpt ? "C" : "") +
                                (obs ? "O" : "") + (stall_pending ? "X" : "") + shape_key();
        FWI_TRY(run_phase(key, [&]() -> int {
            CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, (size_t)B * state * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_ws.p, 0, (size_t)B * field * 4, stream));
            int t = 0;
            if (fused()) {
                int cur = slots;  // d_fwd
                for (auto& sv : saves) {
                    const int tstate = sv.first * unit();
                    fused_steps(t, tstate, &cur, true, false);
                    t = tstate;
                    FWI_TRY(state_copy(snap(sv.second), buf(cur)));
                }
                fused_steps(t, nt, &cur, true, store);
                // the final state in d_fwd, as the in-place steps leave it
                if (cur != slots) FWI_TRY(state_copy(d_fwd.as<float>(), buf(cur)));
            } else {
                for (auto& sv : saves) {
                    const int tstate = sv.first * unit();
                    forward_steps(t, tstate, true, false);
                    t = tstate;
                    FWI_TRY(state_copy(snap(sv.second), d_fwd.as<float>()));
                }
                forward_steps(t, nt, true, store);
            }
            if (rb_active) {
                // the random-boundary forward, from rest, for the backward's
                // reconstruction (the recording sweep above keeps the CPML, so
                // seismograms and residuals are the absorbing-boundary ones)
                CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, (size_t)B * state * 4, stream));
                const ItemDesc* itr = d_items_rb.as<ItemDesc>();
                for (int it = 0; it < nt; it++) {
                    pass_stress_fwd(3, itr, it, 0u);
                    pass_velocity(3, itr, it, FL_INJECT);
                    launches_now += 2;
                }
            }
            if (obs && nrows) {
                CUDA_TRY(cudaMemsetAsync(d_blow.p, 0, 4, stream));
                residual_kernel<<<(unsigned)nrows, 256, 0, stream>>>(
                    d_rec.as<float>(), d_obsf.as<float>(), d_rowrec.as<int>(), d_resid.as<float>(),
                    d_rowmis.as<double>(), d_blow.as<int>(), nt, 0.5 * dt);
                launches_now++;
            }
            return FWI_OK;
        }));
        CUDA_TRY(cudaEventRecord(e1, stream));
        FWI_TRY(h_rec.ensure(rec_out ? nrows * nt * 4 : 16));
        float* rec = h_rec.as<float>();
        std::vector<double> rm(nrows);
        int blow = 0;
        if (nrows && rec_out)
            CUDA_TRY(cudaMemcpyAsync(rec, d_rec.p, nrows * nt * 4, cudaMemcpyDeviceToHost, stream));
        if (nrows && obs) {
            CUDA_TRY(cudaMemcpyAsync(rm.data(), d_rowmis.p, nrows * 8, cudaMemcpyDeviceToHost, stream));
            CUDA_TRY(cudaMemcpyAsync(&blow, d_blow.p, 4, cudaMemcpyDeviceToHost, stream));
        }
        CUDA_TRY(cudaStreamSynchronize(stream));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        FWI_TRY(check_kernel_flags());
        stats.last_forward_ms = ms;
        stats.launches = launches_now;
        stats.forward_steps = (int64_t)nt;
        stats.recompute_steps = 0;
        stats.adjoint_steps = 0;
        stats.device_bytes = (int64_t)(allocated_bytes() + fixed_bytes());
        stats.snapshots = slots;
        if (rec_out)
            for (size_t k = 0; k < nrows; k++)
                for (int t = 0; t < nt; t++) rec_out[(size_t)rows[k] * nt + t] = (double)rec[k * nt + t];
        stats.h2d_bytes = last_h2d;
        stats.d2h_bytes = (int64_t)((rec_out ? nrows * nt * 4 : 0) + (obs ? nrows * 8 + 4 : 0));
        if (misfit) {
            for (int b = 0; b < B; b++) misfit[b] = 0.0;
            if (obs)
                for (size_t k = 0; k < nrows; k++) misfit[row_slot[k]] += rm[k];
        }
        have_resid = obs;
        fwd_kept = keep != 0;
        bwd_done = false;
        if (blow) return fail(FWI_ERR_DIVERGED, "|syn - obs| exceeded 1e10 (the reference aborts here)");
        return FWI_OK;
    }

    // Average device time of each hot kernel on the current batch.
    int time_kernels(int reps, double ms[4]) {
        FWI_TRY(bind());
        if (B == 0) return fail(FWI_ERR_STATE, "run a forward first (it lays out the batch)");
        if (reps < 1) return fail(FWI_ERR_INVALID, "reps must be >= 1");
        cudaEvent_t a, b;
        CUDA_TRY(cudaEventCreate(&a));
        CUDA_TRY(cudaEventCreate(&b));
        const ItemDesc* itf = d_items_f.as<ItemDesc>();
        const ItemDesc* ita = d_items_a.as<ItemDesc>();
        const bool have_adj_src = state_source() ? true : d_store.p != nullptr;
        for (int k = 0; k < 4; k++) {
            const bool adj = k >= 2;
            if (adj && !have_adj_src) { ms[k] = 0.0; continue; }
            if (k == 1 && fused()) { ms[k] = 0.0; continue; }  // the fused step is entry 0
            const int it = fwi_dt * (nft - 1);  // a sampled step: the gradient runs
            auto launch = [&]() {
                // the forms of the recompute sweeps (forward) and of the adjoint
                // sweep; source/receiver events (a separate small kernel in the
                // TMA mapping) are left out
                if (k == 0 && fused()) fused_step(slots, slots + 1, it, 0u, 0u);
                if (k == 0 && !fused()) pass_stress_fwd(0, itf, it, 0u);
                if (k == 1) pass_velocity(0, itf, it, 0u);
                if (k == 2) pass_stress_adj(ita, it, FL_GRAD);
                if (k == 3) pass_velocity(1, ita, it, FL_WE);
            };
            launch();  // warm-up
            CUDA_TRY(cudaEventRecord(a, stream));
            for (int r = 0; r < reps; r++) launch();
            CUDA_TRY(cudaEventRecord(b, stream));
            CUDA_TRY(cudaEventSynchronize(b));
            float t = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&t, a, b));
            ms[k] = t / reps;
        }
        CUDA_TRY(cudaGetLastError());
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        fwd_kept = false;
        return FWI_OK;
    }

    // ---- backward --------------------------------------------------------------
    int backward(double* gl, double* gm, double* gr, int sum_shots, bool accumulate = false) {
        FWI_TRY(bind());
        if (!fwd_kept) return fail(FWI_ERR_NOFORWARD, "backward needs a forward(keep=1)");
        if (!have_resid) return fail(FWI_ERR_STATE, "backward needs observed data (forward obs) or a loaded residual");
        if (bwd_done && state_source())
            return fail(FWI_ERR_STATE, "the checkpointed forward was consumed by the previous backward");
        if (random_mode() && !rb_active)
            return fail(FWI_ERR_STATE, "the forward was not run with random boundaries");
        if (exact() && zero_mu)
            return fail(FWI_ERR_UNSUPPORTED, "the exact adjoint needs mu > 0 on every interior cell");
        cudaEvent_t e0, e1;
        CUDA_TRY(cudaEventCreate(&e0));
        CUDA_TRY(cudaEventCreate(&e1));
        launches_now = 0;
        long long recompute = 0;
        CUDA_TRY(cudaEventRecord(e0, stream));
        const std::string key = std::string(ckpt_mode() ? "bwdC" : random_mode() ? "bwdR" : "bwdS") + shape_key();
        FWI_TRY(run_phase(key, [&]() -> int {
            CUDA_TRY(cudaMemsetAsync(d_adj.p, 0, (size_t)B * state * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_wr.p, 0, (size_t)B * field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_ux.p, 0, (size_t)B * field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_uz.p, 0, (size_t)B * field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_grad.p, 0, (size_t)B * 3 * nf * 4, stream));
            if (exact()) CUDA_TRY(cudaMemsetAsync(d_exact.p, 0, (size_t)B * 9 * field * 4, stream));
            if (random_mode()) {
                // reverse-time reconstruction of the source wavefield, one step
                // ahead of the adjoint step that correlates with it
                const ItemDesc* itr = d_items_rb.as<ItemDesc>();
                for (int it = nt - 1; it >= 0; it--) {
                    events_kernel<<<B, 256, 0, stream>>>(itr, it, FL_INJECT | FL_REVERSE);
                    pass_velocity(3, itr, it, FL_REVERSE);
                    pass_stress_fwd(3, itr, it, FL_REVERSE);
                    launches_now += 3;
                    const unsigned sf = (grad_on && it % fwi_dt == 0) ? FL_GRAD : 0u;
                    step(true, it, sf, FL_INJECT | FL_WE);
                }
                recompute += nt;
                return FWI_OK;
            }
            if (!ckpt_mode()) {
                adjoint_steps(0, nt);
                return FWI_OK;
            }
            // Execute the binomial plan.  The first sweep of forward() already
            // placed the SAVEs that precede the first ADJOINT; start after them.
            size_t k = 0;
            int last_slot = -1, last_state = 0;
            while (k < plan.size() && plan[k].kind != Action::ADJOINT) {
                if (plan[k].kind == Action::SAVE) { last_slot = plan[k].a; last_state = plan[k].b; }
                k++;
            }
            const int u = unit();
            if (copy_free()) {
                FWI_TRY(run_plan_copy_free(k, last_slot, last_state));
                return FWI_OK;
            }
            // working buffer: state of the last prefix checkpoint, advanced to nft-1
            if (last_slot >= 0) FWI_TRY(state_copy(d_fwd.as<float>(), snap(last_slot)));
            else CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, (size_t)B * state * 4, stream));
            forward_steps(last_state * u, (nunits() - 1) * u, false, false);
            recompute += (nunits() - 1) - last_state;
            for (; k < plan.size(); k++) {
                const Action& a = plan[k];
                switch (a.kind) {
                    case Action::ADVANCE:
                        forward_steps(a.a * u, a.b * u, false, false);
                        recompute += a.b - a.a;
                        break;
                    case Action::SAVE:
                        FWI_TRY(state_copy(snap(a.a), d_fwd.as<float>()));
                        break;
                    case Action::RESTORE:
                        if (a.a < 0) CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, (size_t)B * state * 4, stream));
                        else FWI_TRY(state_copy(d_fwd.as<float>(), snap(a.a)));
                        break;
                    case Action::ADJOINT: {
                        if (exact()) {
                            FWI_TRY(exact_step(a.a));
                            recompute += 1;  // state n+1 of the reverse step
                            break;
                        }
                        const int t0 = a.a * fwi_dt, t1 = std::min(nt, (a.a + 1) * fwi_dt);
                        adjoint_steps(t0, t1);
                        break;
                    }
                }
            }
            if (exact()) {
                const dim3 g((unsigned)((nf + kExactThreads - 1) / kExactThreads), (unsigned)B);
                chain_rule<<<g, kExactThreads, 0, stream>>>(d_items_a.as<ItemDesc>(), d_exd.as<ExactDesc>(), B);
                launches_now++;
            }
            return FWI_OK;
        }));
        if (pre_on) {
            FWI_TRY(d_wmax.ensure((size_t)std::max(B, 1) * sizeof(unsigned)));
            CUDA_TRY(cudaMemsetAsync(d_wmax.p, 0, (size_t)B * sizeof(unsigned), stream));
            const dim3 g((unsigned)std::min<size_t>((nf + 255) / 256, 1024), (unsigned)B);
            we_max_kernel<<<g, 256, 0, stream>>>(d_items_a.as<ItemDesc>(), d_ws.as<float>(), d_wr.as<float>(), field,
                                                d_wmax.as<unsigned>());
            precondition_kernel<<<g, 256, 0, stream>>>(d_items_a.as<ItemDesc>(), d_ws.as<float>(), d_wr.as<float>(),
                                                       field, d_wmax.as<unsigned>());
            launches_now += 2;
        }
        watch_array_kernel<<<num_sms * 4, 256, 0, stream>>>(d_grad.as<float>(), (size_t)B * 3 * nf, d_err.as<int>());
        launches_now++;
        if (accumulate) {
            sum_shots_kernel<<<592, 256, 0, stream>>>(d_grad.as<float>(), d_gacc.as<float>(), 3 * nf, B, 1);
            launches_now++;
        } else if (sum_shots && B > 1) {
            sum_shots_kernel<<<592, 256, 0, stream>>>(d_grad.as<float>(), d_gsum.as<float>(), 3 * nf, B, 0);
            launches_now++;
        }
        CUDA_TRY(cudaEventRecord(e1, stream));
        const bool summed = sum_shots && B > 1;
        const size_t ntrip = summed ? 1 : (size_t)B;
        const bool want = !accumulate && (gl || gm || gr);
        FWI_TRY(h_grad.ensure(want ? ntrip * 3 * nf * 4 : 16));
        const float* g = h_grad.as<float>();
        if (want)
            CUDA_TRY(cudaMemcpyAsync(h_grad.p, summed ? d_gsum.p : d_grad.p, ntrip * 3 * nf * 4,
                                     cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        stats.h2d_bytes = 0;
        stats.d2h_bytes = want ? (int64_t)(ntrip * 3 * nf * 4) : 0;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        FWI_TRY(check_kernel_flags());
        stats.last_backward_ms = ms;
        stats.launches = launches_now;
        stats.adjoint_steps = nt;
        (void)recompute;  // counted while the body runs; a graph replay runs the same plan
        stats.recompute_steps = ckpt_mode()     ? plan_recompute() * unit()
                                : random_mode() ? (int64_t)2 * nt
                                                : 0;
        const double k0 = out_scale(0), k1 = out_scale(1), k2 = out_scale(2);
        for (size_t s = 0; s < ntrip && want; s++)
            for (size_t i = 0; i < nf; i++) {
                const float* t = g + s * 3 * nf;
                if (gl) gl[s * nf + i] = t[i] * k0;
                if (gm) gm[s * nf + i] = t[nf + i] * k1;
                if (gr) gr[s * nf + i] = t[2 * nf + i] * k2;
            }
        bwd_done = true;
        return FWI_OK;
    }

    // The binomial plan from action k on (the first sweep's checkpoints are in
    // place; the last of them is `last_slot` with state `last_state`) without
    // state copies.  The working state is tracked as the buffer that holds it:
    // RESTORE only points at the slot's buffer, the next ADVANCE steps out of
    // it into the working buffer, SAVE swaps the working buffer with the
    // slot's free one (the state stays where it is), and ADJOINT reads the
    // forward fields from whichever buffer holds them.
    int run_plan_copy_free(size_t k, int last_slot, int last_state) {
        if (fused()) return run_plan_fused(k, last_slot, last_state);
        const int u = unit();
        std::vector<int> phys(slots);
        for (int i = 0; i < slots; i++) phys[i] = i;
        int wb = slots;  // the working buffer (d_fwd)
        int src = last_slot >= 0 ? phys[last_slot] : wb;
        if (last_slot < 0) CUDA_TRY(cudaMemsetAsync(buf(wb), 0, (size_t)B * state * 4, stream));
        auto advance = [&](int t0, int t1) {
            for (int it = t0; it < t1; it++) {
                step_bufs(src, wb, it);
                src = wb;
            }
        };
        advance(last_state * u, (nunits() - 1) * u);
        for (; k < plan.size(); k++) {
            const Action& a = plan[k];
            switch (a.kind) {
                case Action::ADVANCE:
                    advance(a.a * u, a.b * u);
                    break;
                case Action::SAVE:
                    if (src == wb) {
                        std::swap(phys[a.a], wb);
                        src = phys[a.a];
                    } else {
                        FWI_TRY(state_copy(buf(phys[a.a]), buf(src)));
                        src = phys[a.a];
                    }
                    break;
                case Action::RESTORE:
                    if (a.a < 0) {
                        CUDA_TRY(cudaMemsetAsync(buf(wb), 0, (size_t)B * state * 4, stream));
                        src = wb;
                    } else {
                        src = phys[a.a];
                    }
                    break;
                case Action::ADJOINT: {
                    const int t0 = a.a * fwi_dt, t1 = std::min(nt, (a.a + 1) * fwi_dt);
                    amap_cur = &amaps_b[src];
                    adjoint_steps(t0, t1);
                    amap_cur = nullptr;
                    break;
                }
            }
        }
        return FWI_OK;
    }

    // The same plan with the fused step: two working buffers (a step never
    // writes the buffer it reads); SAVE of a state in a working buffer hands
    // that buffer to the slot and takes the slot's free one in exchange.
    int run_plan_fused(size_t k, int last_slot, int last_state) {
        const int u = unit();
        std::vector<int> phys(slots);
        for (int i = 0; i < slots; i++) phys[i] = i;
        int wbs[2] = {slots, slots + 1};  // the working buffers (initially d_fwd, d_fwd2)
        int src = last_slot >= 0 ? phys[last_slot] : wbs[0];
        if (last_slot < 0) CUDA_TRY(cudaMemsetAsync(buf(wbs[0]), 0, (size_t)B * state * 4, stream));
        auto advance = [&](int t0, int t1) {
            for (int it = t0; it < t1; it++) {
                const int dst = src == wbs[0] ? wbs[1] : wbs[0];
                fused_step(src, dst, it, 0u, FL_INJECT);
                src = dst;
            }
        };
        advance(last_state * u, (nunits() - 1) * u);
        for (; k < plan.size(); k++) {
            const Action& a = plan[k];
            switch (a.kind) {
                case Action::ADVANCE:
                    advance(a.a * u, a.b * u);
                    break;
                case Action::SAVE:
                    if (src == wbs[0] || src == wbs[1]) {
                        int& w = src == wbs[0] ? wbs[0] : wbs[1];
                        std::swap(phys[a.a], w);
                        src = phys[a.a];
                    } else {
                        FWI_TRY(state_copy(buf(phys[a.a]), buf(src)));
                        src = phys[a.a];
                    }
                    break;
                case Action::RESTORE:
                    if (a.a < 0) {
                        CUDA_TRY(cudaMemsetAsync(buf(wbs[0]), 0, (size_t)B * state * 4, stream));
                        src = wbs[0];
                    } else {
                        src = phys[a.a];
                    }
                    break;
                case Action::ADJOINT: {
                    const int t0 = a.a * fwi_dt, t1 = std::min(nt, (a.a + 1) * fwi_dt);
                    amap_cur = &amaps_b[src];
                    adjoint_steps(t0, t1);
                    amap_cur = nullptr;
                    break;
                }
            }
        }
        return FWI_OK;
    }

    // ---- gradient over many shots in sub-batches --------------------------------
    int batch_override = 0;

    // Shots per launch: about 20 M cells per launch (measured on the 1068x568
    // grid, order 8, TMA mapping, 64 shots: 7.98 shot-gradients/s at 14 shots
    // per launch, 8.11 at 16, 8.25 at 32, 8.20 at 64), the shots split evenly
    // over the sub-batches, and a batch (its checkpoints or storage included)
    // within 80 % of the device memory or the engine's budget.
    int auto_batch(int n) const {
        const double cells = (double)(nxt - 2 * fpad) * (double)(nzt - 2 * fpad);
        int bmax = std::max(1, std::min(n, (int)std::ceil(2.0e7 / std::max(1.0, cells))));
        size_t bud = budget;
        if (bud == 0) {
            size_t fr = 0, tot = 0;
            if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) bud = (size_t)(0.8 * (double)(fr + allocated_bytes()));
        }
        const int sl = snapshots_req > 0 ? std::min(snapshots_req, std::max(1, nunits() - 1)) : 0;
        while (bud > 0 && bmax > 1 && batch_bytes(bmax, sl, strategy) + fixed_bytes() > bud) bmax--;
        const int nsub = (n + bmax - 1) / bmax;
        return std::max(1, (n + nsub - 1) / nsub);
    }

    int gradient(int n, const int* ids, const double* obs, double* misfit, double* gl, double* gm,
                 double* gr, int flags) {
        FWI_TRY(bind());
        if (n < 1 || !ids) return fail(FWI_ERR_INVALID, "empty shot list");
        const bool resident = (flags & FWI_FWD_RESIDENT_OBS) != 0;
        if (!resident && !obs) return fail(FWI_ERR_INVALID, "observed data required");
        if (resident && !obs_valid) return fail(FWI_ERR_STATE, "no observed data resident on the device");
        if (!resident) {
            std::vector<int> recs;
            for (int r = 0; r < nrec; r++) {
                if (rcomp[r] != 2) continue;
                for (int b = 0; b < n; b++)
                    if (rshot[r] == ids[b]) { recs.push_back(r); break; }
            }
            FWI_TRY(upload_obs(obs, recs));
        }
        const int64_t h2d = resident ? 0 : last_h2d;
        const int bs = batch_override > 0 ? std::min(batch_override, n) : auto_batch(n);
        CUDA_TRY(cudaMemsetAsync(d_gacc.p ? d_gacc.p : nullptr, 0, d_gacc.p ? 3 * nf * 4 : 0, stream));
        double fwd_ms = 0, bwd_ms = 0;
        int64_t launches = 0, recompute = 0;
        std::vector<double> mis(bs);
        for (int k = 0; k < n; k += bs) {
            const int m = std::min(bs, n - k);
            FWI_TRY(forward(m, ids + k, nullptr, nullptr, mis.data(), FWI_FWD_KEEP | FWI_FWD_RESIDENT_OBS));
            if (misfit) std::copy(mis.begin(), mis.begin() + m, misfit + k);
            if (k == 0) CUDA_TRY(cudaMemsetAsync(d_gacc.p, 0, 3 * nf * 4, stream));
            fwd_ms += stats.last_forward_ms;
            launches += stats.launches;
            FWI_TRY(backward(nullptr, nullptr, nullptr, 1, true));
            bwd_ms += stats.last_backward_ms;
            launches += stats.launches;
            recompute += stats.recompute_steps;
        }
        const bool want = gl || gm || gr;
        FWI_TRY(h_grad.ensure(want ? 3 * nf * 4 : 16));
        if (want)
            CUDA_TRY(cudaMemcpyAsync(h_grad.p, d_gacc.p, 3 * nf * 4, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        const float* g = h_grad.as<float>();
        const double k0 = out_scale(0), k1 = out_scale(1), k2 = out_scale(2);
        for (size_t i = 0; want && i < nf; i++) {
            if (gl) gl[i] = g[i] * k0;
            if (gm) gm[i] = g[nf + i] * k1;
            if (gr) gr[i] = g[2 * nf + i] * k2;
        }
        stats.last_forward_ms = fwd_ms;
        stats.last_backward_ms = bwd_ms;
        stats.launches = launches;
        // per shot (every sub-batch runs the same schedule)
        const int nsub = (n + bs - 1) / bs;
        stats.forward_steps = (int64_t)nt;
        stats.recompute_steps = recompute / nsub;
        stats.adjoint_steps = (int64_t)nt;
        stats.h2d_bytes = h2d;
        stats.d2h_bytes = (misfit ? 0 : 0) + (want ? (int64_t)(3 * nf * 4) : 0) +
                          (int64_t)(rows_cap * 8) * ((n + bs - 1) / bs);
        stats.batch = bs;
        return FWI_OK;
    }

    // Misfits of n shots by forward-only runs in sub-batches (no storage, no
    // checkpoints): the trial runs of the step-length search.
    int misfit_only(int n, const int* ids, const double* obs, double* misfit, int flags) {
        FWI_TRY(bind());
        if (n < 1 || !ids || !misfit) return fail(FWI_ERR_INVALID, "empty shot list or null misfit");
        const bool resident = (flags & FWI_FWD_RESIDENT_OBS) != 0;
        if (!resident && !obs) return fail(FWI_ERR_INVALID, "observed data required");
        if (resident && !obs_valid) return fail(FWI_ERR_STATE, "no observed data resident on the device");
        if (!resident) {
            std::vector<int> recs;
            for (int r = 0; r < nrec; r++) {
                if (rcomp[r] != 2) continue;
                for (int b = 0; b < n; b++)
                    if (rshot[r] == ids[b]) { recs.push_back(r); break; }
            }
            FWI_TRY(upload_obs(obs, recs));
        }
        const int bs = batch_override > 0 ? std::min(batch_override, n) : auto_batch(n);
        double ms = 0;
        int64_t launches = 0;
        for (int k = 0; k < n; k += bs) {
            const int m = std::min(bs, n - k);
            FWI_TRY(forward(m, ids + k, nullptr, nullptr, misfit + k, FWI_FWD_RESIDENT_OBS));
            ms += stats.last_forward_ms;
            launches += stats.launches;
        }
        stats.last_forward_ms = ms;
        stats.launches = launches;
        stats.batch = bs;
        return FWI_OK;
    }

    // Residual rows of the current batch from a [nrec][nt] host array (receiver order).
    int load_residual(const double* sig) {
        FWI_TRY(bind());
        const size_t nrows = rows.size();
        if (!nrows) { have_resid = true; return FWI_OK; }
        std::vector<float> r(nrows * nt);
        for (size_t k = 0; k < nrows; k++)
            for (int t = 0; t < nt; t++) r[k * nt + t] = (float)sig[(size_t)rows[k] * nt + t];
        CUDA_TRY(cudaMemcpyAsync(d_resid.p, r.data(), r.size() * 4, cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        have_resid = true;
        return FWI_OK;
    }
    // FWI storage of batch slot 0 to/from the reference layout (5 arrays [nft][nfz][nfx],
    // order vx, vz, sxx, szx, szz; velocities divided by dt as the reference stores them).
    int storage_io(double* const f[5], bool upload) {
        FWI_TRY(bind());
        if (!d_store.p) return fail(FWI_ERR_STATE, "no FWI storage allocated");
        std::vector<float> h((size_t)nft * 5 * nf);
        if (!upload) CUDA_TRY(cudaMemcpy(h.data(), d_store.p, h.size() * 4, cudaMemcpyDeviceToHost));
        for (int tf = 0; tf < nft; tf++)
            for (int q = 0; q < 5; q++) {
                if (!f[q]) continue;
                float* blk = h.data() + ((size_t)tf * 5 + q) * nf;
                double* ref = f[q] + (size_t)tf * nf;
                for (size_t i = 0; i < nf; i++) {
                    if (upload) blk[i] = (float)ref[i];
                    else ref[i] = blk[i];
                }
            }
        if (upload) CUDA_TRY(cudaMemcpy(d_store.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
        return FWI_OK;
    }
    // CPML memory of batch slot 0 in the reference layouts, order
    // mem_vx_x, mem_vx_z, mem_vz_x, mem_vz_z, mem_sxx_x, mem_szx_x, mem_szz_z, mem_szx_z.
    int read_cpml(int which, double* const m[8]) {
        FWI_TRY(bind());
        const float* st = (which ? d_adj.as<float>() : d_fwd.as<float>()) + 5 * field;
        std::vector<float> h(4 * xstrip + 4 * zstrip);
        CUDA_TRY(cudaMemcpy(h.data(), st, h.size() * 4, cudaMemcpyDeviceToHost));
        // device order: x-strips vx_x, vz_x, sxx_x, szx_x; z-strips vx_z, vz_z, szz_z, szx_z
        const int xs_of[8] = {0, -1, 1, -1, 2, 3, -1, -1};
        const int zs_of[8] = {-1, 0, -1, 1, -1, -1, 2, 3};
        for (int q = 0; q < 8; q++) {
            if (!m[q]) continue;
            if (xs_of[q] >= 0) {
                const float* src = h.data() + xs_of[q] * xstrip;
                for (size_t i = 0; i < (size_t)nzt * tp; i++) m[q][i] = src[i];
            } else {
                const float* src = h.data() + 4 * xstrip + zs_of[q] * zstrip;
                for (int p = 0; p < tp; p++)
                    for (int ix = 0; ix < nxt; ix++) m[q][(size_t)p * nxt + ix] = src[(size_t)p * pitch + ix];
            }
        }
        return FWI_OK;
    }

    int energy(int slot, double* Ws, double* Wr) {
        FWI_TRY(bind());
        if (slot < 0 || slot >= B) return fail(FWI_ERR_INVALID, "bad batch slot");
        std::vector<float> h(field);
        auto get = [&](const DBuf& src, double* out) -> int {
            if (!out) return FWI_OK;
            CUDA_TRY(cudaMemcpy(h.data(), src.as<float>() + (size_t)slot * field, field * 4,
                                cudaMemcpyDeviceToHost));
            for (int iz = 0; iz < nzt; iz++)
                for (int ix = 0; ix < nxt; ix++) out[(size_t)iz * nxt + ix] = h[(size_t)iz * pitch + ix];
            return FWI_OK;
        };
        FWI_TRY(get(d_ws, Ws));
        FWI_TRY(get(d_wr, Wr));
        return FWI_OK;
    }

    int wavefield(int which, int slot, double* out[5]) {
        FWI_TRY(bind());
        if (slot < 0 || slot >= B) return fail(FWI_ERR_INVALID, "bad batch slot");
        const float* st = (which ? d_adj.as<float>() : d_fwd.as<float>()) + (size_t)slot * state;
        std::vector<float> h(5 * field);
        CUDA_TRY(cudaMemcpy(h.data(), st, h.size() * 4, cudaMemcpyDeviceToHost));
        for (int f = 0; f < 5; f++) {
            if (!out[f]) continue;
            for (int iz = 0; iz < nzt; iz++)
                for (int ix = 0; ix < nxt; ix++)
                    out[f][(size_t)iz * nxt + ix] = h[f * field + (size_t)iz * pitch + ix];
        }
        return FWI_OK;
    }
};

}  // namespace fwi

#include "fwi_multi.cuh"

// ===========================================================================
// C ABI
// ===========================================================================
using fwi::Engine;
using fwi::fail;

struct fwi_psv_engine {
    Engine e;
};

#define GUARD_ENGINE(h) \
    if (!(h)) return fail(FWI_ERR_INVALID, "null engine")

extern "C" {

int fwi_psv_abi_version(void) { return FWI_PSV_ABI_VERSION; }

const char* fwi_psv_strerror(int s) {
    switch (s) {
        case FWI_OK: return "ok";
        case FWI_ERR_INVALID: return "invalid argument";
        case FWI_ERR_UNSUPPORTED: return "unsupported configuration";
        case FWI_ERR_NOMEM: return "out of memory";
        case FWI_ERR_CUDA: return "CUDA error";
        case FWI_ERR_STATE: return "call out of order";
        case FWI_ERR_DIVERGED: return "wavefield diverged";
        case FWI_ERR_NOFORWARD: return "no retained forward pass";
        case FWI_ERR_NODEVICE: return "no CUDA device";
        case FWI_ERR_IO: return "file not written";
    }
    return "unknown status";
}

const char* fwi_psv_last_error(void) { return fwi::last_error(); }

int fwi_psv_holberg(int fdorder, int max_rel_err, double hc[7]) {
    if (!hc) return fail(FWI_ERR_INVALID, "null hc");
    return fwi::holberg(fdorder, max_rel_err, hc);
}

int fwi_psv_cpml_profile(int npml, double dh, double fpml, double npower, double k_max_pml,
                         double rcoef, double damp_v_pml, double dt, double* a, double* b,
                         double* K, double* a_half, double* b_half, double* K_half) {
    if (npml < 1 || !a || !b || !K || !a_half || !b_half || !K_half)
        return fail(FWI_ERR_INVALID, "npml must be >= 1 and all profile arrays given");
    if (!(dh > 0) || !(rcoef > 0)) return fail(FWI_ERR_INVALID, "dh and rcoef must be > 0");
    fwi::cpml_profile(npml, dh, fpml, npower, k_max_pml, rcoef, damp_v_pml, dt, a, b, K, a_half,
                      b_half, K_half);
    return FWI_OK;
}

int fwi_psv_total_grid(int nx, int nz, int fdorder, int npml, int fsurf, int* fpad, int* ppad,
                       int* nxt, int* nzt) {
    if (!fpad || !ppad || !nxt || !nzt || nx < 1 || nz < 1 || npml < 0)
        return fail(FWI_ERR_INVALID, "bad grid arguments");
    if (fdorder < 2 || fdorder > 12 || (fdorder & 1)) return fail(FWI_ERR_INVALID, "bad fdorder");
    fwi::total_grid(nx, nz, fdorder, npml, fsurf, fpad, ppad, nxt, nzt);
    return FWI_OK;
}

int fwi_psv_wavelet(double* signal, int nt, double dt, double amp, double fc, double ts, int shape) {
    if (!signal || nt < 0 || !(fc > 0)) return fail(FWI_ERR_INVALID, "bad wavelet arguments");
    if (shape != 1) return fail(FWI_ERR_UNSUPPORTED, "only shape 1 (Ricker) exists");
    fwi::wavelet(signal, nt, dt, amp, fc, ts, shape);
    return FWI_OK;
}

int fwi_psv_average_parameters(int nzt, int nxt, const double* mu, const double* rho,
                               double* mu_zx, double* rho_zp, double* rho_xp) {
    if (nzt < 2 || nxt < 2 || !mu || !rho || !mu_zx || !rho_zp || !rho_xp)
        return fail(FWI_ERR_INVALID, "bad averaging arguments");
    fwi::average_parameters(nzt, nxt, mu, rho, mu_zx, rho_zp, rho_xp);
    return FWI_OK;
}

int fwi_psv_checkpoint_plan(int nsteps, int slots, int* actions, int cap, int* count,
                            long long* forward_steps) {
    if (nsteps < 0 || slots < 0 || !count) return fail(FWI_ERR_INVALID, "bad plan arguments");
    long long cost = 0;
    const std::vector<fwi::Action> plan = fwi::plan_binomial(nsteps, slots, &cost);
    *count = (int)plan.size();
    if (forward_steps) *forward_steps = cost;
    if (!actions || cap < (int)plan.size()) return fail(FWI_ERR_INVALID, "action buffer too small");
    for (size_t i = 0; i < plan.size(); i++) {
        actions[3 * i] = plan[i].kind;
        actions[3 * i + 1] = plan[i].a;
        actions[3 * i + 2] = plan[i].b;
    }
    return FWI_OK;
}

int fwi_psv_create(const fwi_psv_desc* desc, int device, fwi_psv_engine** out) {
    if (!desc || !out) return fail(FWI_ERR_INVALID, "null argument");
    *out = nullptr;
    int n = 0;
    cudaError_t ce = cudaGetDeviceCount(&n);
    if (ce != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(FWI_ERR_NODEVICE, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    }
    if (device < 0 || device >= n) return fail(FWI_ERR_INVALID, "bad device index");
    std::unique_ptr<fwi_psv_engine> h(new (std::nothrow) fwi_psv_engine());
    if (!h) return fail(FWI_ERR_NOMEM, "host allocation failed");
    h->e.device = device;
    int s = h->e.init(desc);
    if (s != FWI_OK) return s;
    *out = h.release();
    return FWI_OK;
}

int fwi_psv_destroy(fwi_psv_engine* e) {
    if (!e) return FWI_OK;
    cudaSetDevice(e->e.device);
    if (e->e.stream) cudaStreamSynchronize(e->e.stream);
    delete e;
    return FWI_OK;
}

int fwi_psv_set_stream(fwi_psv_engine* h, void* s) {
    GUARD_ENGINE(h);
    Engine& e = h->e;
    if (e.own_stream && e.stream) {
        cudaStreamSynchronize(e.stream);
        cudaStreamDestroy(e.stream);
    }
    e.drop_graphs();
    if (s) {
        e.stream = static_cast<cudaStream_t>(s);
        e.own_stream = false;
    } else {
        cudaSetDevice(e.device);
        if (cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking) != cudaSuccess)
            return fail(FWI_ERR_CUDA, "stream creation failed");
        e.own_stream = true;
    }
    return FWI_OK;
}

int fwi_psv_set_model(fwi_psv_engine* h, const double* lam, const double* mu, const double* mu_zx,
                      const double* rho_zp, const double* rho_xp) {
    GUARD_ENGINE(h);
    return h->e.set_model(lam, mu, mu_zx, rho_zp, rho_xp);
}

int fwi_psv_set_model_lmr(fwi_psv_engine* h, const double* lam, const double* mu, const double* rho) {
    GUARD_ENGINE(h);
    if (!lam || !mu || !rho) return fail(FWI_ERR_INVALID, "null material array");
    Engine& e = h->e;
    const size_t na = (size_t)(e.nzt - 1) * (e.nxt - 1);
    std::vector<double> mz(na), rz(na), rx(na);
    fwi::average_parameters(e.nzt, e.nxt, mu, rho, mz.data(), rz.data(), rx.data());
    return e.set_model(lam, mu, mz.data(), rz.data(), rx.data());
}

struct fwi_psv_multi {
    fwi::MultiEngine m;
};

int fwi_psv_multi_create(int nmodels, const fwi_psv_model* models, int device, fwi_psv_multi** out) {
    if (!out) return fail(FWI_ERR_INVALID, "null output handle");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(FWI_ERR_NODEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return fail(FWI_ERR_INVALID, "bad device index");
    auto* h = new (std::nothrow) fwi_psv_multi();
    if (!h) return fail(FWI_ERR_NOMEM, "host allocation failed");
    const int st = h->m.init(nmodels, models, device);
    if (st != FWI_OK) {
        delete h;
        return st;
    }
    *out = h;
    return FWI_OK;
}

int fwi_psv_multi_destroy(fwi_psv_multi* h) {
    if (!h) return FWI_OK;
    cudaSetDevice(h->m.device);
    delete h;
    return FWI_OK;
}

int fwi_psv_multi_set_exec(fwi_psv_multi* h, int use_graphs, int snapshots, int autotune) {
    if (!h) return fail(FWI_ERR_INVALID, "null handle");
    if (snapshots < 0) return fail(FWI_ERR_INVALID, "snapshots must be >= 0");
    h->m.use_graphs = use_graphs ? 1 : 0;
    h->m.slots_req = snapshots;
    h->m.plan.clear();
    h->m.tune_on = autotune ? 1 : 0;
    h->m.drop_graphs();
    return FWI_OK;
}

int fwi_psv_multi_forward(fwi_psv_multi* h, double* const* rec_out) {
    if (!h) return fail(FWI_ERR_INVALID, "null handle");
    return h->m.forward(rec_out);
}

int fwi_psv_multi_gradient(fwi_psv_multi* h, const double* const* obs, double* misfit, double* const* gl,
                           double* const* gm, double* const* gr) {
    if (!h) return fail(FWI_ERR_INVALID, "null handle");
    return h->m.gradient(obs, misfit, gl, gm, gr);
}

int fwi_psv_multi_tuning(fwi_psv_multi* h, int group, int info[7], double ms[2]) {
    if (!h || !info || !ms) return fail(FWI_ERR_INVALID, "null argument");
    if (group < 0 || group >= (int)h->m.groups.size()) return fail(FWI_ERR_INVALID, "no such order group");
    const auto& g = *h->m.groups[group];
    info[0] = g.fp;
    info[1] = (int)g.members.size();
    info[2] = g.tune.fmap == 3 ? 3 : g.kf.map;  // the kernel set's map (a half order may not have map 2)
    info[3] = g.tune.ftz;
    info[4] = g.tune.amap == 3 ? 3 : g.ka.map;
    info[5] = g.tune.atz;
    info[6] = g.tune.cached ? 1 : 0;
    ms[0] = g.tune.fms;
    ms[1] = g.tune.ams;
    return FWI_OK;
}

int fwi_psv_multi_get_stats(fwi_psv_multi* h, fwi_psv_stats* out) {
    if (!h || !out) return fail(FWI_ERR_INVALID, "null argument");
    *out = h->m.stats;
    return FWI_OK;
}

int fwi_psv_set_snapshots(fwi_psv_engine* h, int interval, int which) {
    GUARD_ENGINE(h);
    if (interval < 0 || which < 0 || which > 4) return fail(FWI_ERR_INVALID, "interval >= 0, field 0..4");
    Engine& e = h->e;
    e.snap_interval = interval;
    e.snap_field = which;
    e.invalidate_batch();
    return FWI_OK;
}

int fwi_psv_snapshot(fwi_psv_engine* h, int slot, int k, double* out) {
    GUARD_ENGINE(h);
    Engine& e = h->e;
    if (!out || slot < 0 || slot >= e.B || k < 0 || k >= e.nsnap || !e.d_snapshots.p)
        return fail(FWI_ERR_INVALID, "no such snapshot (slot, index) of the last forward");
    FWI_TRY(e.bind());
    std::vector<float> hbuf(e.field);
    CUDA_TRY(cudaMemcpy(hbuf.data(), e.d_snapshots.as<float>() + ((size_t)slot * e.nsnap + k) * e.field,
                        e.field * 4, cudaMemcpyDeviceToHost));
    for (int iz = 0; iz < e.nzt; iz++)
        for (int ix = 0; ix < e.nxt; ix++) out[(size_t)iz * e.nxt + ix] = hbuf[(size_t)iz * e.pitch + ix];
    return FWI_OK;
}

int fwi_psv_get_layout(fwi_psv_engine* h, fwi_psv_layout* o) {
    GUARD_ENGINE(h);
    if (!o) return fail(FWI_ERR_INVALID, "null layout");
    const Engine& e = h->e;
    *o = {e.nt, e.nzt, e.nxt, e.fpad, e.ppad, e.npml, e.fsurf, e.fdorder, e.fwi_dt, e.fwi_dx, e.fwi_dz,
          e.wx1, e.wx2, e.wz1, e.wz2, e.nfz, e.nfx, e.device};
    return FWI_OK;
}

int fwi_psv_set_model_device(fwi_psv_engine* h, const double* d_lam, const double* d_mu, const double* d_rho) {
    GUARD_ENGINE(h);
    return h->e.set_model_device(d_lam, d_mu, d_rho);
}

int fwi_psv_set_precondition(fwi_psv_engine* h, int on, double c_lam, double c_mu, double c_rho) {
    GUARD_ENGINE(h);
    if (on && (!(c_lam > 0) || !(c_mu > 0) || !(c_rho > 0)))
        return fail(FWI_ERR_INVALID, "preconditioning needs positive medium averages");
    Engine& e = h->e;
    e.pre_on = on != 0;
    e.pre_c[0] = c_lam;
    e.pre_c[1] = c_mu;
    e.pre_c[2] = c_rho;
    return FWI_OK;
}

int fwi_psv_misfit(fwi_psv_engine* h, int nshots, const int* shots, const double* obs, double* misfit,
                   int flags) {
    GUARD_ENGINE(h);
    return h->e.misfit_only(nshots, shots, obs, misfit, flags);
}

int fwi_psv_set_sources(fwi_psv_engine* h, int n, const int* x, const int* z, const int* comp,
                        const int* shot, const double* signal) {
    GUARD_ENGINE(h);
    return h->e.set_sources(n, x, z, comp, shot, signal);
}

int fwi_psv_set_receivers(fwi_psv_engine* h, int n, const int* x, const int* z, const int* comp,
                          const int* shot) {
    GUARD_ENGINE(h);
    return h->e.set_receivers(n, x, z, comp, shot);
}

int fwi_psv_set_fwi(fwi_psv_engine* h, int fdt, int fdx, int fdz, int x1, int x2, int z1, int z2) {
    GUARD_ENGINE(h);
    return h->e.set_fwi(fdt, fdx, fdz, x1, x2, z1, z2);
}

int fwi_psv_set_strategy(fwi_psv_engine* h, int strategy, int snapshots, size_t budget) {
    GUARD_ENGINE(h);
    if (strategy != FWI_STORE_FULL && strategy != FWI_STORE_BINOMIAL && strategy != FWI_STORE_RANDOM)
        return fail(FWI_ERR_INVALID, "unknown strategy");
    if (snapshots < 0) return fail(FWI_ERR_INVALID, "snapshots must be >= 0");
    Engine& e = h->e;
    e.strategy = strategy;
    e.snapshots_req = snapshots;
    e.budget = budget;
    e.invalidate_batch();
    return FWI_OK;
}

int fwi_psv_set_gradient_mode(fwi_psv_engine* h, int mode) {
    GUARD_ENGINE(h);
    if (mode != FWI_GRAD_REFERENCE && mode != FWI_GRAD_EXACT) return fail(FWI_ERR_INVALID, "unknown mode");
    if (h->e.grad_mode != mode) h->e.invalidate_batch();
    h->e.grad_mode = mode;
    return FWI_OK;
}

int fwi_psv_set_exec(fwi_psv_engine* h, int use_graphs, int block_x, int tile_z, int batch) {
    GUARD_ENGINE(h);
    if ((block_x != 0 && block_x != 32 && block_x != 64 && block_x != fwi::kTileX && block_x != 256 &&
         block_x != 512) ||
        tile_z < 0 || batch < 0)
        return fail(FWI_ERR_INVALID, "block_x must be 0, 32, 64, 128, 256 or 512; tile_z and batch >= 0");
    Engine& e = h->e;
    e.use_graphs = use_graphs ? 1 : 0;
    e.bx_req = block_x;
    e.tz_req = tile_z;
    e.batch_override = batch;
    // block_x 128 (or a tile height) selects the z-march, 32 the scalar cell
    // mapping, 64 the vectorised cells, 256 the TMA-staged tiles, 0 the default
    // (the TMA passes as two launches per forward step, the default), 512 the
    // TMA mapping with the fused forward step (fdorder <= 8)
    const int map = (block_x == fwi::kTileX || tile_z > 0) ? 0
                    : block_x == 32                        ? 1
                    : block_x == 256 || block_x == 512     ? 3
                    : block_x == 64                        ? 2
                                                           : fwi::kDefaultMap;
    e.fuse = block_x == 512;
    if (map != e.kmap) {
        if (map == 3) {
            cudaSetDevice(e.device);
            cudaError_t ce = e.tset.prepare();
            if (ce == cudaSuccess && e.fset.prepare) ce = e.fset.prepare();
            if (ce != cudaSuccess)
                return fail(FWI_ERR_CUDA, std::string("TMA kernels: ") + cudaGetErrorString(ce));
        }
        e.kmap = map;
        e.ks = fwi::kernels_for(e.fpad, map);
    }
    e.invalidate_batch();
    for (auto& kv : e.tilesets) kv.second->ntiles = 0;
    e.drop_graphs();
    return FWI_OK;
}

int fwi_psv_set_device_allocator(fwi_psv_alloc_fn alloc, fwi_psv_free_fn release, void* ctx) {
    if ((alloc == nullptr) != (release == nullptr))
        return fail(FWI_ERR_INVALID, "give both alloc and release, or neither");
    fwi::DeviceAllocator a;
    a.alloc = alloc;
    a.release = release;
    a.ctx = alloc ? ctx : nullptr;
    fwi::set_device_allocator(a);
    return FWI_OK;
}

int fwi_psv_set_wait_limit(fwi_psv_engine* h, double seconds) {
    GUARD_ENGINE(h);
    if (!(seconds >= 1e-6 && seconds <= 60.0)) return fail(FWI_ERR_INVALID, "wait limit must be in [1e-6, 60] s");
    h->e.wait_ns = (unsigned long long)(seconds * 1e9);
    h->e.invalidate_batch();  // the limit is a launch argument (captured graphs are rebuilt)
    return FWI_OK;
}

int fwi_psv_debug_stall_next(fwi_psv_engine* h) {
    GUARD_ENGINE(h);
    if (!h->e.fused() && (h->e.kmap != 3 || h->e.exact()))
        return fail(FWI_ERR_UNSUPPORTED, "the stall hook needs a TMA forward step (block_x 256 or 512, reference gradient)");
    h->e.stall_next = true;
    return FWI_OK;
}

int fwi_psv_forward(fwi_psv_engine* h, int nshots, const int* shots, const double* obs,
                    double* rec_out, double* misfit, int flags) {
    GUARD_ENGINE(h);
    return h->e.forward(nshots, shots, obs, rec_out, misfit, flags);
}

int fwi_psv_gradient(fwi_psv_engine* h, int nshots, const int* shots, const double* obs,
                     double* misfit, double* gl, double* gm, double* gr, int flags) {
    GUARD_ENGINE(h);
    return h->e.gradient(nshots, shots, obs, misfit, gl, gm, gr, flags);
}

int fwi_psv_backward(fwi_psv_engine* h, double* gl, double* gm, double* gr, int sum_shots) {
    GUARD_ENGINE(h);
    return h->e.backward(gl, gm, gr, sum_shots);
}

int fwi_psv_energy(fwi_psv_engine* h, int slot, double* Ws, double* Wr) {
    GUARD_ENGINE(h);
    return h->e.energy(slot, Ws, Wr);
}

int fwi_psv_wavefield(fwi_psv_engine* h, int which, int slot, double* vx, double* vz, double* sxx,
                      double* szx, double* szz) {
    GUARD_ENGINE(h);
    double* out[5] = {vx, vz, sxx, szx, szz};
    return h->e.wavefield(which, slot, out);
}

int fwi_psv_time_kernels(fwi_psv_engine* h, int reps, double ms[4]) {
    GUARD_ENGINE(h);
    if (!ms) return fail(FWI_ERR_INVALID, "null ms");
    return h->e.time_kernels(reps, ms);
}

int fwi_psv_get_stats(fwi_psv_engine* h, fwi_psv_stats* out) {
    GUARD_ENGINE(h);
    if (!out) return fail(FWI_ERR_INVALID, "null stats");
    *out = h->e.stats;
    return FWI_OK;
}

// ---- reference-shaped calls ------------------------------------------------
// One engine per host thread is cached and reused while the grid, scheme and
// CPML profiles stay the same (the reference calls these once per shot).
namespace {
struct RefCache {
    std::unique_ptr<fwi_psv_engine> h;
    fwi_psv_desc d{};
    std::vector<double> prof;
};
thread_local RefCache g_ref;

int ref_engine(const fwi_psv_desc& d, Engine** out) {
    const int tp = 2 * (d.npml + 1);
    std::vector<double> prof;
    if (d.npml > 0)
        for (const double* p : {d.a, d.b, d.K, d.a_half, d.b_half, d.K_half}) {
            if (!p) return fail(FWI_ERR_INVALID, "CPML profiles are required when npml > 0");
            prof.insert(prof.end(), p, p + tp);
        }
    const bool same = g_ref.h && g_ref.d.nt == d.nt && g_ref.d.nzt == d.nzt && g_ref.d.nxt == d.nxt &&
                      g_ref.d.fpad == d.fpad && g_ref.d.ppad == d.ppad && g_ref.d.npml == d.npml &&
                      g_ref.d.fsurf == d.fsurf && g_ref.d.fdorder == d.fdorder &&
                      g_ref.d.dt == d.dt && g_ref.d.dx == d.dx && g_ref.d.dz == d.dz &&
                      std::memcmp(g_ref.d.hc, d.hc, sizeof d.hc) == 0 && g_ref.prof == prof;
    if (!same) {
        if (g_ref.h) fwi_psv_destroy(g_ref.h.release());
        fwi_psv_engine* h = nullptr;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
        FWI_TRY(fwi_psv_create(&d, dev, &h));
        g_ref.h.reset(h);
        g_ref.d = d;
        g_ref.prof = prof;
        // per-shot calls with changing models: plain launches, no graph capture
        h->e.use_graphs = 0;
    }
    *out = &g_ref.h->e;
    return FWI_OK;
}

fwi_psv_desc make_desc(int nt, int nzt, int nxt, int fpad, int ppad, double dt, double dx,
                       double dz, int fsurf, const double* hc, int fdorder, int npml,
                       const double* a, const double* b, const double* K, const double* ah,
                       const double* bh, const double* Kh) {
    fwi_psv_desc d{};
    d.nt = nt; d.nzt = nzt; d.nxt = nxt; d.fpad = fpad; d.ppad = ppad; d.npml = npml;
    d.fsurf = fsurf; d.fdorder = fdorder; d.dt = dt; d.dx = dx; d.dz = dz;
    for (int i = 0; i < 7; i++) d.hc[i] = hc ? hc[i] : 0.0;
    d.a = a; d.b = b; d.K = K; d.a_half = ah; d.b_half = bh; d.K_half = Kh;
    return d;
}
}  // namespace

int fwi_psv_forward_kernel(int ishot, int nt, int nzt, int nxt, int fpad, int ppad, double dt,
                           double dx, double dz, int snap_interval, int fsurf, const double* hc,
                           int fdorder, double* vx, double* vz, double* sxx, double* szx,
                           double* szz, double* We, const double* lam, const double* mu,
                           const double* mu_zx, const double* rho_zp, const double* rho_xp,
                           int npml, const double* a, const double* b, const double* K,
                           const double* a_half, const double* b_half, const double* K_half,
                           double* mem_vx_x, double* mem_vx_z, double* mem_vz_x,
                           double* mem_vz_z, double* mem_sxx_x, double* mem_szx_x,
                           double* mem_szz_z, double* mem_szx_z, int nsrc, const int* src_x,
                           const int* src_z, const int* src_comp, const double* src_signal,
                           const int* source_to_fire_shot, int nrec, const int* rec_x,
                           const int* rec_z, const int* rec_comp, double* rec_signal,
                           const int* receiver_to_record_shot, int fwinv, int fwi_dt,
                           int fwi_dx, int fwi_dz, int fwi_x1, int fwi_x2, int fwi_z1,
                           int fwi_z2, double* fwi_vx, double* fwi_vz, double* fwi_sxx,
                           double* fwi_szx, double* fwi_szz) {
    (void)snap_interval;  // the CSV snapshot writer is not part of the engine
    if (!hc) return fail(FWI_ERR_INVALID, "null hc");
    fwi_psv_desc d = make_desc(nt, nzt, nxt, fpad, ppad, dt, dx, dz, fsurf, hc, fdorder, npml, a,
                               b, K, a_half, b_half, K_half);
    Engine* e = nullptr;
    FWI_TRY(ref_engine(d, &e));
    FWI_TRY(e->set_model(lam, mu, mu_zx, rho_zp, rho_xp));
    FWI_TRY(e->set_sources(nsrc, src_x, src_z, src_comp, source_to_fire_shot, src_signal));
    FWI_TRY(e->set_receivers(nrec, rec_x, rec_z, rec_comp, receiver_to_record_shot));
    if (fwinv) FWI_TRY(e->set_fwi(fwi_dt, fwi_dx, fwi_dz, fwi_x1, fwi_x2, fwi_z1, fwi_z2));
    else FWI_TRY(e->set_fwi(1, 1, 1, 0, nxt, 0, nzt));
    e->strategy = FWI_STORE_FULL;
    FWI_TRY(e->forward(1, &ishot, nullptr, rec_signal, nullptr, fwinv ? 1 : 0));
    double* w[5] = {vx, vz, sxx, szx, szz};
    FWI_TRY(e->wavefield(0, 0, w));
    if (We) FWI_TRY(e->energy(0, We, nullptr));
    double* m[8] = {mem_vx_x, mem_vx_z, mem_vz_x, mem_vz_z, mem_sxx_x, mem_szx_x, mem_szz_z, mem_szx_z};
    FWI_TRY(e->read_cpml(0, m));
    if (fwinv) {
        double* f[5] = {fwi_vx, fwi_vz, fwi_sxx, fwi_szx, fwi_szz};
        FWI_TRY(e->storage_io(f, false));
    }
    return FWI_OK;
}

int fwi_psv_adjoint_kernel(int ishot, int nt, int nzt, int nxt, int fpad, int ppad, double dt,
                           double dx, double dz, int snap_interval, int fsurf, const double* hc,
                           int fdorder, double* vx, double* vz, double* sxx, double* szx,
                           double* szz, double* We, const double* lam, const double* mu,
                           const double* mu_zx, const double* rho_zp, const double* rho_xp,
                           int npml, const double* a, const double* b, const double* K,
                           const double* a_half, const double* b_half, const double* K_half,
                           double* mem_vx_x, double* mem_vx_z, double* mem_vz_x,
                           double* mem_vz_z, double* mem_sxx_x, double* mem_szx_x,
                           double* mem_szz_z, double* mem_szx_z, int nsrc, const int* src_x,
                           const int* src_z, const int* src_comp, const double* src_signal,
                           const int* source_to_fire_shot, int fwinv, int fwi_dt, int fwi_dx,
                           int fwi_dz, int fwi_x1, int fwi_x2, int fwi_z1, int fwi_z2,
                           const double* fwi_vx, const double* fwi_vz, const double* fwi_sxx,
                           const double* fwi_szx, const double* fwi_szz, double* grad_lam,
                           double* grad_mu, double* grad_rho) {
    (void)snap_interval;
    if (!hc) return fail(FWI_ERR_INVALID, "null hc");
    fwi_psv_desc d = make_desc(nt, nzt, nxt, fpad, ppad, dt, dx, dz, fsurf, hc, fdorder, npml, a,
                               b, K, a_half, b_half, K_half);
    Engine* e = nullptr;
    FWI_TRY(ref_engine(d, &e));
    FWI_TRY(e->set_model(lam, mu, mu_zx, rho_zp, rho_xp));
    // The adjoint's sources are the receivers carrying the residual
    // (fd_wave_model.cu:848-859 passes receiver.* as the source arguments).
    FWI_TRY(e->set_sources(0, nullptr, nullptr, nullptr, nullptr, nullptr));
    FWI_TRY(e->set_receivers(nsrc, src_x, src_z, src_comp, source_to_fire_shot));
    FWI_TRY(e->set_fwi(fwi_dt, fwi_dx, fwi_dz, fwi_x1, fwi_x2, fwi_z1, fwi_z2));
    e->strategy = FWI_STORE_FULL;
    FWI_TRY(e->setup_batch(1, &ishot, true));
    if (fwinv) {
        if (!fwi_vx || !fwi_vz || !fwi_sxx || !fwi_szx || !fwi_szz)
            return fail(FWI_ERR_INVALID, "FWI storage arrays required when fwinv");
        double* f[5] = {const_cast<double*>(fwi_vx), const_cast<double*>(fwi_vz),
                        const_cast<double*>(fwi_sxx), const_cast<double*>(fwi_szx),
                        const_cast<double*>(fwi_szz)};
        FWI_TRY(e->storage_io(f, true));
    }
    FWI_TRY(e->load_residual(src_signal));
    e->fwd_kept = true;
    e->bwd_done = false;
    e->grad_on = fwinv != 0;
    int st = e->backward(grad_lam, grad_mu, grad_rho, 0);
    e->grad_on = true;
    FWI_TRY(st);
    double* w[5] = {vx, vz, sxx, szx, szz};
    FWI_TRY(e->wavefield(1, 0, w));
    if (We) FWI_TRY(e->energy(0, nullptr, We));
    double* m[8] = {mem_vx_x, mem_vx_z, mem_vz_x, mem_vz_z, mem_sxx_x, mem_szx_x, mem_szz_z, mem_szx_z};
    FWI_TRY(e->read_cpml(1, m));
    return FWI_OK;
}

}  // extern "C"
