// fwi_tma.cuh -- TMA-staged stencil passes (thread mapping 3).
//
// Same arithmetic as the stress / velocity passes of fwi_kernels.cuh
// (forward_kernel_PSV_GPU.cu:830-1063 generalised to fdorder 2..12), but every
// input field of a 128 x 16 cell tile is brought into shared memory by the
// tensor memory accelerator (cp.async.bulk.tensor) before any thread touches
// it: one elected thread issues a handful of 3-D box copies per tile (one per
// field; the differentiated fields with their halo), completion is tracked by
// an mbarrier with a transaction count, and two or three stages are in flight
// per CTA.
// A persistent CTA (one per SM) walks the tile work-list; while it computes
// tile k from one stage, the copies of tile k+1 fill the other, so the HBM
// requests of a whole tile are outstanding without any thread waiting on them.
//
// Tensor maps: state fields are 3-D (x = column, y = row, z = batch slot; slot
// stride = one shot state), materials 2-D.  Boxes start at x0 - HX with HX a
// multiple of 4 floats (the 16-byte rule for the x coordinate of a tiled copy);
// boxes reaching outside the grid (x < 0, y >= nzt) are zero-filled by TMA and
// those cells are masked anyway.
//
// Waits are bounded by the global timer: a stage not complete within
// kWaitNs sets bit 2 of the error word, the CTA drains the copies it issued
// (again bounded) and returns; the host discards the results.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fwi_kernels.cuh"

namespace fwi {

constexpr int kTmaTX = 128;      // tile columns
constexpr int kTmaTZ = 16;       // tile rows
constexpr int kTmaThreads = 512; // 4 threads per column (4 rows each in a 16-row tile)
constexpr int kThreadRowsF = kTmaTZ / (kTmaThreads / kTmaTX);  // rows per thread, forward passes
// stages in flight per CTA: three while they fit the 227 KB of shared memory
// (half orders up to 4), two above
template <int FP>
__host__ __device__ constexpr int tma_stages() {
    return FP <= 4 ? 3 : 2;
}
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s

// The slot descriptor travels with each tile's stage (bulk copy), so a tile's
// compute phase starts without a global-memory round trip.
constexpr int kDescFloats = (int)((sizeof(ItemDesc) + 127) / 128 * 32);
static_assert(sizeof(ItemDesc) % 16 == 0, "bulk copies move multiples of 16 bytes");

template <int FP>
struct TmaGeom {
    static constexpr int TX = kTmaTX, TZ = kTmaTZ;
    static constexpr int HX = (FP + 3) / 4 * 4;  // x halo, multiple of 4 floats
    static constexpr int WX = TX + 2 * HX;       // halo box width
    static constexpr int WZ = TZ + 2 * FP;       // halo box height
    static constexpr int CEN = TX * TZ;
    static constexpr int pad(int n) { return (n + 31) / 32 * 32; }  // 128-byte sub-buffers
    static constexpr int HXZ = pad(WX * WZ);   // x and z halo
    static constexpr int HXO = pad(WX * TZ);   // x halo only
    static constexpr int HZO = pad(TX * WZ);   // z halo only
    // stress stage: vx, vz (x+z halo), L, M2, MZ, sxx, szx, szz, descriptor
    static constexpr int S_STAGE = 2 * HXZ + 6 * CEN + kDescFloats;
    static constexpr int S_DESC = 2 * HXZ + 6 * CEN;
    // velocity stage: sxx (x halo), szx (x+z halo), szz (z halo), BX, BZ, vx, vz, We, descriptor
    static constexpr int V_STAGE = HXO + HXZ + HZO + 5 * CEN + kDescFloats;
    static constexpr int V_DESC = HXO + HXZ + HZO + 5 * CEN;
};

struct StressMaps {
    CUtensorMap vx, vz, L, M2, MZ, sxx, szx, szz;
};
struct VelMaps {
    CUtensorMap sxx, szx, szz, BX, BZ, vx, vz, We;
};

// Tile t of a launch: slot b = t % nb (shots minor, so consecutive CTAs share
// the material tile in L2), then z-tile, then x-tile.
struct TmaGrid {
    int nb, ntz, ntiles, pad;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_2d(float* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tile_coords(const TmaGrid& g, int t, int* b, int* x0, int* z0, int FPv,
                                            int TZ = kTmaTZ) {
    *b = t % g.nb;
    const int r = t / g.nb;
    *z0 = FPv + (r % g.ntz) * TZ;
    *x0 = (r / g.ntz) * kTmaTX;
}

// ---------------------------------------------------------------------------
// stress pass
// ---------------------------------------------------------------------------
template <int FP>
__device__ __forceinline__ void stress_issue(const StressMaps& m, const ItemDesc* items, const TmaGrid& g, int t,
                                             float* st, uint64_t* bar) {
    using G = TmaGeom<FP>;
    int b, x0, z0;
    tile_coords(g, t, &b, &x0, &z0, FP);
    constexpr unsigned bytes = 4u * (2 * G::WX * G::WZ + 6 * G::CEN) + (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::S_DESC, items + b, (unsigned)sizeof(ItemDesc), bar);
    tma_load_3d(st, &m.vx, x0 - G::HX, z0 - FP, b, bar);
    tma_load_3d(st + G::HXZ, &m.vz, x0 - G::HX, z0 - FP, b, bar);
    float* c = st + 2 * G::HXZ;
    tma_load_2d(c, &m.L, x0, z0, bar);
    tma_load_2d(c + G::CEN, &m.M2, x0, z0, bar);
    tma_load_2d(c + 2 * G::CEN, &m.MZ, x0, z0, bar);
    tma_load_3d(c + 3 * G::CEN, &m.sxx, x0, z0, b, bar);
    tma_load_3d(c + 4 * G::CEN, &m.szx, x0, z0, b, bar);
    tma_load_3d(c + 5 * G::CEN, &m.szz, x0, z0, b, bar);
}

template <int FP>
__device__ __forceinline__ void stress_compute(const ItemDesc& D, const float* st, int x0, int z0, int it,
                                               unsigned flags) {
    using G = TmaGeom<FP>;
    constexpr int R = kThreadRowsF;  // rows of this thread
    const int tx = threadIdx.x & (kTmaTX - 1);
    const int r0 = (threadIdx.x / kTmaTX) * R;
    const int ix = x0 + tx;
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    if (ix < FP || ix >= nxt - FP) return;
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const float* svx = st;
    const float* svz = st + G::HXZ;
    const float* cen = st + 2 * G::HXZ;
    const int col = tx + G::HX;
    // z-windows of this thread's rows: wvx[j] = vx of row r0 + j - FP + 1,
    // wvz[j] = vz of row r0 + j - FP (each staged value read once)
    float wvx[R + 2 * FP - 1], wvz[R + 2 * FP - 1];
#pragma unroll
    for (int j = 0; j < R + 2 * FP - 1; j++) {
        wvx[j] = svx[(r0 + j + 1) * G::WX + col];
        wvz[j] = svz[(r0 + j) * G::WX + col];
    }
    const float dt = D.dt;
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    float* __restrict__ gsxx = D.sxx;
    float* __restrict__ gszx = D.szx;
    float* __restrict__ gszz = D.szz;
    float* __restrict__ mvx_x = D.mvx_x;
    float* __restrict__ mvz_x = D.mvz_x;
    float* __restrict__ mvx_z = D.mvx_z;
    float* __restrict__ mvz_z = D.mvz_z;
    int px = -1;
    if (npml > 0) {
        if (ix <= ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(cpml, tp, px);
    // CPML memories of all rows of this thread, loaded before any row is
    // computed (one memory latency per tile instead of one per row)
    float mx1[R], mx2[R], mz1[R], mz2[R];
    int pzr[R];
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const int iz = z0 + r0 + rr;
        mx1[rr] = mx2[rr] = mz1[rr] = mz2[rr] = 0.f;
        int pz = -1;
        if (npml > 0 && iz < nzt - FP) {
            if (!fsurf && iz <= ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz == npml) pz = -1;
        }
        pzr[rr] = pz;
        if (px >= 0 && iz < nzt - FP) {
            mx1[rr] = mvx_x[(size_t)iz * tp + px];
            mx2[rr] = mvz_x[(size_t)iz * tp + px];
        }
        if (pz >= 0) {
            mz1[rr] = mvz_z[(size_t)pz * P + ix];
            mz2[rr] = mvx_z[(size_t)pz * P + ix];
        }
    }
    int xf = -1;
    if ((flags & FL_STORE) && D.store && ix >= D.wx1 && ix < D.wx2 && (ix - D.wx1) % D.fwi_dx == 0)
        xf = (ix - D.wx1) / D.fwi_dx;
    // FL_REVERSE undoes the step (s^n = s^{n+1} - S(v^n)); used only without
    // CPML and free surface, where the update is a pure increment
    const float sg = (flags & FL_REVERSE) ? -1.f : 1.f;
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const int r = r0 + rr;
        const int iz = z0 + r;
        if (iz >= nzt - FP) break;
        const int row = r + FP;
        const float* vxr = svx + row * G::WX + col;
        const float* vzr = svz + row * G::WX + col;
        float vx_x = 0.f, vz_x = 0.f, vx_z = 0.f, vz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_x += hx[k - 1] * ((k == 1 ? wvx[rr + FP - 1] : vxr[k - 1]) - vxr[-k]);
            vz_x += hx[k - 1] * (vzr[k] - (k == 1 ? wvz[rr + FP] : vzr[-k + 1]));
            vx_z += hz[k - 1] * (wvx[rr + k + FP - 1] - wvx[rr - k + FP]);
            vz_z += hz[k - 1] * (wvz[rr + k - 1 + FP] - wvz[rr - k + FP]);
        }
        const size_t c = (size_t)iz * P + ix;
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * mx1[rr] + cx.a * vx_x;
            const float m2 = cx.bh * mx2[rr] + cx.ah * vz_x;
            mvx_x[m] = m1;
            mvz_x[m] = m2;
            vx_x = vx_x * cx.iK + m1;
            vz_x = vz_x * cx.iKh + m2;
        }
        if (pzr[rr] >= 0) {
            const int pz = pzr[rr];
            const Cpml cz = load_cpml(cpml, tp, pz);
            const size_t m = (size_t)pz * P + ix;
            const float m1 = cz.b * mz1[rr] + cz.a * vz_z;
            const float m2 = cz.bh * mz2[rr] + cz.ah * vx_z;
            mvz_z[m] = m1;
            mvx_z[m] = m2;
            vz_z = vz_z * cz.iK + m1;
            vx_z = vx_z * cz.iKh + m2;
        }
        const int ci = r * kTmaTX + tx;
        const float L = cen[ci], M2 = cen[G::CEN + ci], MZ = cen[2 * G::CEN + ci];
        float sxx = cen[3 * G::CEN + ci], szx = cen[4 * G::CEN + ci], szz = cen[5 * G::CEN + ci];
        if (xf >= 0 && iz >= D.wz1 && iz < D.wz2 && (iz - D.wz1) % D.fwi_dz == 0) {
            const size_t fs = (size_t)D.nfz * D.nfx;
            float* s = D.store + (size_t)(it / D.fwi_dt) * 5 * fs + (size_t)((iz - D.wz1) / D.fwi_dz) * D.nfx + xf;
            s[F_VX * fs] = wvx[rr + FP - 1] / dt;
            s[F_VZ * fs] = wvz[rr + FP] / dt;
            s[F_SXX * fs] = sxx;
            s[F_SZX * fs] = szx;
            s[F_SZZ * fs] = szz;
        }
        szx += sg * (MZ * (vz_x + vx_z));
        const float tr = L * (vx_x + vz_z);
        sxx += sg * (tr + M2 * vx_x);
        szz += sg * (tr + M2 * vz_z);
        if (fsurf && iz == FP) {
            szz = 0.f;
            szx = 0.f;
            sxx = vx_x * (2.f * M2 * (L + 0.5f * M2)) / (L + M2);
        }
        gsxx[c] = sxx;
        gszx[c] = szx;
        gszz[c] = szz;
        if (fsurf && iz > FP && iz <= 2 * FP) {
            const size_t cm = (size_t)(2 * FP - iz) * P + ix;
            gszx[cm] = -szx;
            gszz[cm] = -szz;
        }
    }
}

// ---------------------------------------------------------------------------
// velocity pass (+ energy)
// ---------------------------------------------------------------------------
template <int FP>
__device__ __forceinline__ void velocity_issue(const VelMaps& m, const ItemDesc* items, const TmaGrid& g, int t,
                                               float* st, uint64_t* bar, bool we) {
    using G = TmaGeom<FP>;
    int b, x0, z0;
    tile_coords(g, t, &b, &x0, &z0, FP);
    const unsigned bytes = 4u * (G::WX * G::TZ + G::WX * G::WZ + G::TX * G::WZ + (we ? 5 : 4) * G::CEN) +
                           (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::V_DESC, items + b, (unsigned)sizeof(ItemDesc), bar);
    tma_load_3d(st, &m.sxx, x0 - G::HX, z0, b, bar);
    tma_load_3d(st + G::HXO, &m.szx, x0 - G::HX, z0 - FP, b, bar);
    tma_load_3d(st + G::HXO + G::HXZ, &m.szz, x0, z0 - FP, b, bar);
    float* c = st + G::HXO + G::HXZ + G::HZO;
    tma_load_2d(c, &m.BX, x0, z0, bar);
    tma_load_2d(c + G::CEN, &m.BZ, x0, z0, bar);
    tma_load_3d(c + 2 * G::CEN, &m.vx, x0, z0, b, bar);
    tma_load_3d(c + 3 * G::CEN, &m.vz, x0, z0, b, bar);
    if (we) tma_load_3d(c + 4 * G::CEN, &m.We, x0, z0, b, bar);
}

// Source injection and receiver recording are not done here: the engine runs
// them in a separate small kernel after this pass (events_kernel).
template <int FP>
__device__ __forceinline__ void velocity_compute(const ItemDesc& D, const float* st, int x0, int z0, unsigned flags) {
    using G = TmaGeom<FP>;
    constexpr int R = kThreadRowsF;
    const int tx = threadIdx.x & (kTmaTX - 1);
    const int r0 = (threadIdx.x / kTmaTX) * R;
    const int ix = x0 + tx;
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    if (ix < FP || ix >= nxt - FP) return;
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const float* ssxx = st;                       // [TZ][WX]
    const float* sszx = st + G::HXO;              // [WZ][WX]
    const float* sszz = st + G::HXO + G::HXZ;     // [WZ][TX]
    const float* cen = st + G::HXO + G::HXZ + G::HZO;
    const int col = tx + G::HX;
    // z-windows: wsx[j] = szx of row r0 + j - FP, wsz[j] = szz of row r0 + j - FP + 1
    float wsx[R + 2 * FP - 1], wsz[R + 2 * FP - 1];
#pragma unroll
    for (int j = 0; j < R + 2 * FP - 1; j++) {
        wsx[j] = sszx[(r0 + j) * G::WX + col];
        wsz[j] = sszz[(r0 + j + 1) * G::TX + tx];
    }
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    float* __restrict__ gvx = D.vx;
    float* __restrict__ gvz = D.vz;
    float* __restrict__ gwe = D.We;
    float* __restrict__ msxx_x = D.msxx_x;
    float* __restrict__ mszx_x = D.mszx_x;
    float* __restrict__ mszz_z = D.mszz_z;
    float* __restrict__ mszx_z = D.mszx_z;
    int px = -1;
    if (npml > 0) {
        if (ix < ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(cpml, tp, px);
    float mx1[R], mx2[R], mz1[R], mz2[R];
    int pzr[R];
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const int iz = z0 + r0 + rr;
        mx1[rr] = mx2[rr] = mz1[rr] = mz2[rr] = 0.f;
        int pz = -1;
        if (npml > 0 && iz < nzt - FP) {
            if (!fsurf && iz < ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz == npml) pz = -1;
        }
        pzr[rr] = pz;
        if (px >= 0 && iz < nzt - FP) {
            mx1[rr] = msxx_x[(size_t)iz * tp + px];
            mx2[rr] = mszx_x[(size_t)iz * tp + px];
        }
        if (pz >= 0) {
            mz1[rr] = mszz_z[(size_t)pz * P + ix];
            mz2[rr] = mszx_z[(size_t)pz * P + ix];
        }
    }
    const bool we = (flags & FL_WE) != 0;
    const float sg = (flags & FL_REVERSE) ? -1.f : 1.f;  // v^n = v^{n+1} - V(s^{n+1})
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const int r = r0 + rr;
        const int iz = z0 + r;
        if (iz >= nzt - FP) break;
        const float* sxr = ssxx + r * G::WX + col;
        const float* szr = sszx + (r + FP) * G::WX + col;
        float sxx_x = 0.f, szx_x = 0.f, szx_z = 0.f, szz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            sxx_x += hx[k - 1] * (sxr[k] - sxr[-k + 1]);
            szx_x += hx[k - 1] * ((k == 1 ? wsx[rr + FP] : szr[k - 1]) - szr[-k]);
            szx_z += hz[k - 1] * (wsx[rr + k - 1 + FP] - wsx[rr - k + FP]);
            szz_z += hz[k - 1] * (wsz[rr + k + FP - 1] - wsz[rr - k + FP]);
        }
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * mx1[rr] + cx.a * sxx_x;
            const float m2 = cx.bh * mx2[rr] + cx.ah * szx_x;
            msxx_x[m] = m1;
            mszx_x[m] = m2;
            sxx_x = sxx_x * cx.iK + m1;
            szx_x = szx_x * cx.iKh + m2;
        }
        if (pzr[rr] >= 0) {
            const int pz = pzr[rr];
            const Cpml cz = load_cpml(cpml, tp, pz);
            const size_t m = (size_t)pz * P + ix;
            const float m1 = cz.b * mz1[rr] + cz.a * szz_z;
            const float m2 = cz.bh * mz2[rr] + cz.ah * szx_z;
            mszz_z[m] = m1;
            mszx_z[m] = m2;
            szz_z = szz_z * cz.iK + m1;
            szx_z = szx_z * cz.iKh + m2;
        }
        const int ci = r * kTmaTX + tx;
        const float vxn = cen[2 * G::CEN + ci] + sg * (cen[ci] * (sxx_x + szx_z));
        const float vzn = cen[3 * G::CEN + ci] + sg * (cen[G::CEN + ci] * (szx_x + szz_z));
        const size_t c = (size_t)iz * P + ix;
        if (we) gwe[c] = cen[4 * G::CEN + ci] + (vxn * vxn + vzn * vzn);
        gvx[c] = vxn;
        gvz[c] = vzn;
    }
}

// ---------------------------------------------------------------------------
// persistent pipelined kernels
// ---------------------------------------------------------------------------
// Body shared by the passes.  ISSUE(t, stage_ptr, bar) queues the copies of
// tile t; COMPUTE(b, x0, z0, stage_ptr) runs the cells; TZ is the tile height.
template <int FP, int STAGE_FLOATS, int TZ, class Issue, class Compute>
__device__ __forceinline__ void tma_pipeline(const TmaGrid& g, int* err, Issue issue, Compute compute) {
    constexpr int kTmaStages = tma_stages<FP>();
    // dynamic shared memory only: the stages (128-byte multiples) then the barriers
    extern __shared__ __align__(128) float tma_smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(tma_smem + kTmaStages * STAGE_FLOATS);
    const int tid = threadIdx.x;
    // an earlier launch gave up (error word set): return at once, so a failing
    // pipeline costs one bounded wait and not one per launch; the decision is
    // CTA-uniform (every thread reaches the barrier below)
    if (__syncthreads_or(*(volatile int*)err != 0)) return;
    if (smem_u32(tma_smem) & 127u) {  // TMA destinations need 128-byte alignment
        if (tid == 0) atomicOr(err, 8);
        return;
    }
    if (tid == 0) {
        for (int s = 0; s < kTmaStages; s++) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int first = blockIdx.x, step = gridDim.x;
    if (tid == 0)
        for (int s = 0; s < kTmaStages; s++) {
            const int t = first + s * step;
            if (t < g.ntiles) issue(t, tma_smem + s * STAGE_FLOATS, &bar[s]);
        }
    for (int k = 0;; k++) {
        const int t = first + k * step;
        if (t >= g.ntiles) break;
        const int s = k % kTmaStages;
        const unsigned parity = (unsigned)((k / kTmaStages) & 1);
        const bool ok = mbar_wait_bounded(&bar[s], parity);
        int b, x0, z0;
        tile_coords(g, t, &b, &x0, &z0, FP, TZ);
        if (ok) compute(b, x0, z0, tma_smem + s * STAGE_FLOATS);
        // every thread is done with stage s (or some thread's wait gave up)
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(err, 4);
                // drain the copies this CTA issued and has not consumed (bounded)
                for (int j = k; j < k + kTmaStages; j++) {
                    const int tj = first + j * step;
                    if (tj < g.ntiles) mbar_wait_bounded(&bar[j % kTmaStages], (unsigned)((j / kTmaStages) & 1));
                }
            }
            return;
        }
        if (tid == 0) {
            const int tn = first + (k + kTmaStages) * step;
            if (tn < g.ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(tn, tma_smem + s * STAGE_FLOATS, &bar[s]);
            }
        }
    }
}

template <int FP>
constexpr size_t stress_tma_smem() {
    return sizeof(float) * tma_stages<FP>() * TmaGeom<FP>::S_STAGE + sizeof(uint64_t) * tma_stages<FP>();
}
template <int FP>
constexpr size_t velocity_tma_smem() {
    return sizeof(float) * tma_stages<FP>() * TmaGeom<FP>::V_STAGE + sizeof(uint64_t) * tma_stages<FP>();
}
static_assert(stress_tma_smem<4>() <= 232448 && velocity_tma_smem<4>() <= 232448, "shared memory per CTA");
static_assert(stress_tma_smem<6>() <= 232448 && velocity_tma_smem<6>() <= 232448, "shared memory per CTA");

template <int FP>
__global__ void __launch_bounds__(kTmaThreads, 1)
    stress_tma_kernel(const __grid_constant__ StressMaps maps, const ItemDesc* __restrict__ items,
                      const TmaGrid g, int it, unsigned flags, int* err) {
    using G = TmaGeom<FP>;
    tma_pipeline<FP, G::S_STAGE, kTmaTZ>(
        g, err, [&](int t, float* st, uint64_t* bar) { stress_issue<FP>(maps, items, g, t, st, bar); },
        [&](int, int x0, int z0, const float* st) {
            stress_compute<FP>(*reinterpret_cast<const ItemDesc*>(st + G::S_DESC), st, x0, z0, it, flags);
        });
}

template <int FP>
__global__ void __launch_bounds__(kTmaThreads, 1)
    velocity_tma_kernel(const __grid_constant__ VelMaps maps, const ItemDesc* __restrict__ items,
                        const TmaGrid g, int it, unsigned flags, int* err) {
    using G = TmaGeom<FP>;
    const bool we = (flags & FL_WE) != 0;
    tma_pipeline<FP, G::V_STAGE, kTmaTZ>(
        g, err, [&](int t, float* st, uint64_t* bar) { velocity_issue<FP>(maps, items, g, t, st, bar, we); },
        [&](int, int x0, int z0, const float* st) {
            velocity_compute<FP>(*reinterpret_cast<const ItemDesc*>(st + G::V_DESC), st, x0, z0, flags);
        });
}


// ---------------------------------------------------------------------------
// adjoint stress pass with the reference's gradient (128 x 8 tiles)
// ---------------------------------------------------------------------------
// adjoint_kernel_PSV_GPU.cu:818-863 then :869-984: ux/uz integration, the
// correlation gradient on sampled steps (forward fields from the checkpointed
// forward state, same layout as the adjoint state), then the stress update of
// the adjoint wavefield.  Thirteen centre fields and the vx/vz halos of a
// tile are staged; the gradient triples ([nfz][nfx], rows not 16-byte
// aligned) are read with plain loads issued before the rows are computed.
constexpr int kAdjTZ = 8;

template <int FP>
struct AdjGeom {
    static constexpr int TX = kTmaTX, TZ = kAdjTZ;
    static constexpr int HX = (FP + 3) / 4 * 4;
    static constexpr int WX = TX + 2 * HX, WZ = TZ + 2 * FP;
    static constexpr int CEN = TX * TZ;
    static constexpr int HXZ = (WX * WZ + 31) / 32 * 32;
    // vx, vz halos; L, M2, MZ, sxx, szx, szz, ux, uz, fvx, fvz, fsxx, fszx, fszz; descriptor
    static constexpr int DESC = 2 * HXZ + 13 * CEN;
    static constexpr int STAGE = DESC + kDescFloats;
};

struct AdjMaps {
    CUtensorMap vx, vz, L, M2, MZ, sxx, szx, szz, ux, uz, fvx, fvz, fsxx, fszx, fszz;
};

template <int FP>
__host__ __device__ constexpr size_t adjoint_tma_smem() {
    return sizeof(float) * tma_stages<FP>() * AdjGeom<FP>::STAGE + sizeof(uint64_t) * tma_stages<FP>();
}
static_assert(adjoint_tma_smem<4>() <= 232448 && adjoint_tma_smem<6>() <= 232448, "shared memory per CTA");

template <int FP>
__device__ __forceinline__ void adjoint_issue(const AdjMaps& m, const ItemDesc* items, const TmaGrid& g, int t,
                                              float* st, uint64_t* bar, bool grad) {
    using G = AdjGeom<FP>;
    int b, x0, z0;
    tile_coords(g, t, &b, &x0, &z0, FP, kAdjTZ);
    const unsigned bytes = 4u * (2 * G::WX * G::WZ + (grad ? 13 : 8) * G::CEN) + (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::DESC, items + b, (unsigned)sizeof(ItemDesc), bar);
    tma_load_3d(st, &m.vx, x0 - G::HX, z0 - FP, b, bar);
    tma_load_3d(st + G::HXZ, &m.vz, x0 - G::HX, z0 - FP, b, bar);
    float* c = st + 2 * G::HXZ;
    tma_load_2d(c, &m.L, x0, z0, bar);
    tma_load_2d(c + G::CEN, &m.M2, x0, z0, bar);
    tma_load_2d(c + 2 * G::CEN, &m.MZ, x0, z0, bar);
    tma_load_3d(c + 3 * G::CEN, &m.sxx, x0, z0, b, bar);
    tma_load_3d(c + 4 * G::CEN, &m.szx, x0, z0, b, bar);
    tma_load_3d(c + 5 * G::CEN, &m.szz, x0, z0, b, bar);
    tma_load_3d(c + 6 * G::CEN, &m.ux, x0, z0, b, bar);
    tma_load_3d(c + 7 * G::CEN, &m.uz, x0, z0, b, bar);
    if (grad) {
        tma_load_3d(c + 8 * G::CEN, &m.fvx, x0, z0, b, bar);
        tma_load_3d(c + 9 * G::CEN, &m.fvz, x0, z0, b, bar);
        tma_load_3d(c + 10 * G::CEN, &m.fsxx, x0, z0, b, bar);
        tma_load_3d(c + 11 * G::CEN, &m.fszx, x0, z0, b, bar);
        tma_load_3d(c + 12 * G::CEN, &m.fszz, x0, z0, b, bar);
    }
}

template <int FP>
__device__ __forceinline__ void adjoint_compute(const ItemDesc& D, const float* st, int x0, int z0, int it,
                                                bool grad_step) {
    using G = AdjGeom<FP>;
    constexpr int R = kAdjTZ / (kTmaThreads / kTmaTX);
    const int tx = threadIdx.x & (kTmaTX - 1);
    const int r0 = (threadIdx.x / kTmaTX) * R;
    const int ix = x0 + tx;
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    if (ix < FP || ix >= nxt - FP) return;
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const float* svx = st;
    const float* svz = st + G::HXZ;
    const float* cen = st + 2 * G::HXZ;
    const int col = tx + G::HX;
    float wvx[R + 2 * FP - 1], wvz[R + 2 * FP - 1];
#pragma unroll
    for (int j = 0; j < R + 2 * FP - 1; j++) {
        wvx[j] = svx[(r0 + j + 1) * G::WX + col];
        wvz[j] = svz[(r0 + j) * G::WX + col];
    }
    const float dt = D.dt, inv_dt = D.inv_dt, gs = D.gscale;
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    float* __restrict__ gsxx = D.sxx;
    float* __restrict__ gszx = D.szx;
    float* __restrict__ gszz = D.szz;
    float* __restrict__ gux = D.ux;
    float* __restrict__ guz = D.uz;
    float* __restrict__ mvx_x = D.mvx_x;
    float* __restrict__ mvz_x = D.mvz_x;
    float* __restrict__ mvx_z = D.mvx_z;
    float* __restrict__ mvz_z = D.mvz_z;
    int px = -1;
    if (npml > 0) {
        if (ix <= ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(cpml, tp, px);
    // gradient window column of this thread
    int xf = -1;
    const int wz1 = D.wz1, wz2 = D.wz2, fdz = D.fwi_dz, nfx = D.nfx;
    if (grad_step && ix >= D.wx1 && ix < D.wx2) {
        // unit intervals (the common case) need no integer division
        const int dxw = ix - D.wx1;
        if (D.fwi_dx == 1) xf = dxw;
        else if (dxw % D.fwi_dx == 0) xf = dxw / D.fwi_dx;
    }
    float* __restrict__ glam = D.glam;
    float* __restrict__ gmu = D.gmu;
    float* __restrict__ grho = D.grho;
    float mx1[R], mx2[R], mz1[R], mz2[R], g0[R], g1[R], g2[R];
    int pzr[R], gi[R];
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const int iz = z0 + r0 + rr;
        mx1[rr] = mx2[rr] = mz1[rr] = mz2[rr] = g0[rr] = g1[rr] = g2[rr] = 0.f;
        int pz = -1;
        if (npml > 0 && iz < nzt - FP) {
            if (!fsurf && iz <= ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz == npml) pz = -1;
        }
        pzr[rr] = pz;
        if (px >= 0 && iz < nzt - FP) {
            mx1[rr] = mvx_x[(size_t)iz * tp + px];
            mx2[rr] = mvz_x[(size_t)iz * tp + px];
        }
        if (pz >= 0) {
            mz1[rr] = mvz_z[(size_t)pz * P + ix];
            mz2[rr] = mvx_z[(size_t)pz * P + ix];
        }
        gi[rr] = -1;
        if (xf >= 0 && iz < nzt - FP && iz >= wz1 && iz < wz2 && (fdz == 1 || (iz - wz1) % fdz == 0)) {
            gi[rr] = (fdz == 1 ? iz - wz1 : (iz - wz1) / fdz) * nfx + xf;
            g0[rr] = glam[gi[rr]];
            g1[rr] = gmu[gi[rr]];
            g2[rr] = grho[gi[rr]];
        }
    }
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
        const int r = r0 + rr;
        const int iz = z0 + r;
        if (iz >= nzt - FP) break;
        const int row = r + FP;
        const float* vxr = svx + row * G::WX + col;
        const float* vzr = svz + row * G::WX + col;
        float vx_x = 0.f, vz_x = 0.f, vx_z = 0.f, vz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_x += hx[k - 1] * ((k == 1 ? wvx[rr + FP - 1] : vxr[k - 1]) - vxr[-k]);
            vz_x += hx[k - 1] * (vzr[k] - (k == 1 ? wvz[rr + FP] : vzr[-k + 1]));
            vx_z += hz[k - 1] * (wvx[rr + k + FP - 1] - wvx[rr - k + FP]);
            vz_z += hz[k - 1] * (wvz[rr + k - 1 + FP] - wvz[rr - k + FP]);
        }
        const size_t c = (size_t)iz * P + ix;
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * mx1[rr] + cx.a * vx_x;
            const float m2 = cx.bh * mx2[rr] + cx.ah * vz_x;
            mvx_x[m] = m1;
            mvz_x[m] = m2;
            vx_x = vx_x * cx.iK + m1;
            vz_x = vz_x * cx.iKh + m2;
        }
        if (pzr[rr] >= 0) {
            const int pz = pzr[rr];
            const Cpml cz = load_cpml(cpml, tp, pz);
            const size_t m = (size_t)pz * P + ix;
            const float m1 = cz.b * mz1[rr] + cz.a * vz_z;
            const float m2 = cz.bh * mz2[rr] + cz.ah * vx_z;
            mvz_z[m] = m1;
            mvx_z[m] = m2;
            vz_z = vz_z * cz.iK + m1;
            vx_z = vx_z * cz.iKh + m2;
        }
        const int ci = r * kTmaTX + tx;
        const float L = cen[ci], M2 = cen[G::CEN + ci], MZ = cen[2 * G::CEN + ci];
        float sxx = cen[3 * G::CEN + ci], szx = cen[4 * G::CEN + ci], szz = cen[5 * G::CEN + ci];
        const float ux = cen[6 * G::CEN + ci] + dt * wvx[rr + FP - 1];
        const float uz = cen[7 * G::CEN + ci] + dt * wvz[rr + FP];
        gux[c] = ux;
        guz[c] = uz;
        if (gi[rr] >= 0) {
            // the stored velocities are v/dt; reciprocals computed once per cell
            // (two divisions instead of five; rounding within the gradient tolerance)
            const float fvx = cen[8 * G::CEN + ci] * inv_dt, fvz = cen[9 * G::CEN + ci] * inv_dt;
            const float fsxx = cen[10 * G::CEN + ci], fszx = cen[11 * G::CEN + ci], fszz = cen[12 * G::CEN + ci];
            const float lpm = (L + 0.5f * M2) * inv_dt;
            const float mu = 0.5f * M2 * inv_dt;
            const float ilpm2 = 0.25f / (lpm * lpm);
            const float imu2 = 1.f / (mu * mu);
            const float s1 = (fsxx + fszz) * (sxx + szz) * ilpm2;
            const float s2 = (fsxx - fszz) * (sxx - szz) * imu2;
            const float s3 = (fszx * szx) * imu2;
            const float s4 = ux * fvx + uz * fvz;
            glam[gi[rr]] = g0[rr] + gs * s1;
            gmu[gi[rr]] = g1[rr] + gs * (s3 + s1 + s2);
            grho[gi[rr]] = g2[rr] - gs * s4;
        }
        szx += MZ * (vz_x + vx_z);
        const float tr = L * (vx_x + vz_z);
        sxx += tr + M2 * vx_x;
        szz += tr + M2 * vz_z;
        if (fsurf && iz == FP) {
            szz = 0.f;
            szx = 0.f;
            sxx = vx_x * (2.f * M2 * (L + 0.5f * M2)) / (L + M2);
        }
        gsxx[c] = sxx;
        gszx[c] = szx;
        gszz[c] = szz;
        if (fsurf && iz > FP && iz <= 2 * FP) {
            const size_t cm = (size_t)(2 * FP - iz) * P + ix;
            gszx[cm] = -szx;
            gszz[cm] = -szz;
        }
    }
}

template <int FP>
__global__ void __launch_bounds__(kTmaThreads, 1)
    adjoint_tma_kernel(const __grid_constant__ AdjMaps maps, const ItemDesc* __restrict__ items, const TmaGrid g,
                       int it, unsigned flags, int* err) {
    using G = AdjGeom<FP>;
    const bool grad = (flags & FL_GRAD) != 0;
    tma_pipeline<FP, G::STAGE, kAdjTZ>(
        g, err, [&](int t, float* st, uint64_t* bar) { adjoint_issue<FP>(maps, items, g, t, st, bar, grad); },
        [&](int, int x0, int z0, const float* st) {
            adjoint_compute<FP>(*reinterpret_cast<const ItemDesc*>(st + G::DESC), st, x0, z0, it, grad);
        });
}

}  // namespace fwi
