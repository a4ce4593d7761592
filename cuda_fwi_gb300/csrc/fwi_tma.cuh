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

// Forward tile rows (a variant build may set 20 or 24: 640 or 768 threads, two
// stages, 96 or 80 registers with spills; on 32 shots of the 1068x568 grid,
// order 8, they ran at 0.159 / 0.192 ms per stress launch against 0.143 for 16).
#ifndef FWI_TMA_ROWS
#define FWI_TMA_ROWS 16
#endif
constexpr int kTmaTX = 128;           // tile columns
constexpr int kTmaTZ = FWI_TMA_ROWS;  // forward tile rows
constexpr int kPairRows = 2;          // forward: a thread owns a column pair of two rows
constexpr int kFwdThreads = (kTmaTX / 2) * (kTmaTZ / kPairRows);
constexpr int kAdjThreads = 512;      // adjoint: a thread owns a column pair of one row (128 x 8 tiles)
static_assert(kTmaTZ % kPairRows == 0 && kFwdThreads <= 1024, "forward tile rows");
// stages in flight per CTA for a stage of the given size: as many as fit the
// 227 KB of shared memory (with the barriers), at most six -- three for the
// forward passes up to half order 4 and for every adjoint pass, two for the
// forward passes above
template <int STAGE_FLOATS>
__host__ __device__ constexpr int stages_for() {
    return (232448 - 512) / (STAGE_FLOATS * 4) < 6 ? (232448 - 512) / (STAGE_FLOATS * 4) : 6;
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
// [cxl, cxh] x [czl, czh] (inclusive) are the cells that both forward passes
// update with the plain stencil: no border column, no CPML strip (taken one
// cell wider than either pass uses it), no free-surface row or mirror row.
// [gxl, gxh] x [gzl, gzh]: the gradient window when it is sampled at unit
// intervals (empty otherwise).
struct TmaGrid {
    int nb, ntz, ntiles;
    int stall;  // test hook: CTA 0's first stage expects 16 bytes its copies do not deliver
    int cxl, cxh, czl, czh;
    int gxl, gxh, gzl, gzh;
    // forward passes: offset (floats) from the written state to the state the
    // CPML memories are read from (0 in place; a step out of a checkpoint
    // buffer into the working buffer reads them from the checkpoint)
    long long msrc;
    unsigned long long wait_ns;  // limit of each bounded wait (0: kWaitNs)
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
// Raise the transaction count of the current phase without arriving.
__device__ __forceinline__ void mbar_expect_tx_only(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
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
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    return mbar_wait_bounded(bar, parity, kWaitNs);
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
// two-cell arithmetic of the forward passes
// ---------------------------------------------------------------------------
// In the stress and velocity passes a thread owns two neighbouring columns of
// two rows.  Staged values are read as 8-byte pairs and every stencil operation
// is one FP32x2 instruction for both columns (each lane rounded like the
// scalar operation), which halves the load and arithmetic instructions per
// cell of the one-column mapping.
static_assert(kTmaTX == 128 && kPairRows == 2, "a warp covers 64 columns of one row pair");

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ float lane(float2 v, int l) { return l ? v.y : v.x; }
// store a pair, or only its lanes inside the updated columns
__device__ __forceinline__ void st2(float* p, float2 v, bool on0, bool on1) {
    if (on0 && on1) {
        *reinterpret_cast<float2*>(p) = v;
    } else {
        if (on0) p[0] = v.x;
        if (on1) p[1] = v.y;
    }
}

// One staged row around a column pair (pointer p at the pair's first column,
// 8-byte aligned): q[j] is the pair at column offset 2j - E, E = FP rounded up
// to even, so at(i) covers offsets -E .. FP+1.  The pair at offset 0 is the
// caller's (it is the centre of a z-window already in registers).
template <int FP>
struct RowPairs {
    static constexpr int E = 2 * ((FP + 1) / 2);
    static constexpr int NQ = (E + FP + 1) / 2 + 1;
    float2 q[NQ];
    __device__ __forceinline__ void load(const float* p, float2 centre) {
#pragma unroll
        for (int j = 0; j < NQ; j++) q[j] = (2 * j == E) ? centre : ld2(p + 2 * j - E);
    }
    __device__ __forceinline__ float at(int i) const {
        const int u = i + E;
        return (u & 1) ? q[u >> 1].y : q[u >> 1].x;
    }
    // (f[c+i] - f[c+j], f[c+i+1] - f[c+j+1]); an odd offset is a pair that
    // straddles two loaded pairs, and then the lanes are subtracted one by one
    // straight into a fresh register pair (no copies to assemble the operand)
    __device__ __forceinline__ float2 diff(int i, int j) const {
        if ((((i + E) | (j + E)) & 1) == 0) return sub2(q[(i + E) >> 1], q[(j + E) >> 1]);
        return make_float2(__fsub_rn(at(i), at(j)), __fsub_rn(at(i + 1), at(j + 1)));
    }
    // sum_k h_k (f[c+k-1] - f[c-k]) for c and c+1
    __device__ __forceinline__ float2 dminus(const float2* h) const {
        float2 d = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 1; k <= FP; k++) d = fma2(h[k - 1], diff(k - 1, -k), d);
        return d;
    }
    // sum_k h_k (f[c+k] - f[c-k+1]) for c and c+1
    __device__ __forceinline__ float2 dplus(const float2* h) const {
        float2 d = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 1; k <= FP; k++) d = fma2(h[k - 1], diff(k, 1 - k), d);
        return d;
    }
};

// The warp's 64 columns x kPairRows rows lie inside the grid's plain-stencil
// cells and no storage sample is taken: it runs the branch-free row loop.
// The decision is the same for every thread of the warp.
__device__ __forceinline__ bool interior_warp(const TmaGrid& g, int x0, int z0, unsigned flags, int lt) {
    const int w = lt >> 5;
    const int wx0 = x0 + (w & 1) * 64, wz0 = z0 + (w >> 1) * 2;
    return !(flags & FL_STORE) && wx0 >= g.cxl && wx0 + 63 <= g.cxh && wz0 >= g.czl && wz0 + 1 <= g.czh;
}

// Columns of a pair that the pass updates, and their x-strip indices.
struct PairCols {
    bool on0, on1;
    int px[2];
};
template <int FP>
__device__ __forceinline__ PairCols pair_cols(const ItemDesc& D, int ix, bool stress) {
    PairCols pc;
    pc.on0 = ix >= FP && ix < D.nxt - FP;
    pc.on1 = ix + 1 >= FP && ix + 1 < D.nxt - FP;
#pragma unroll
    for (int l = 0; l < 2; l++) {
        const int i = ix + l;
        int px = -1;
        if (D.npml > 0 && (l ? pc.on1 : pc.on0)) {
            // the stress pass's left strip includes column ppad, the velocity pass's does not
            if (stress ? i <= D.ppad : i < D.ppad) px = i - FP;
            else if (i >= D.nxt - D.ppad - 1) px = i - D.pnx;
            if (px == D.npml) px = -1;
        }
        pc.px[l] = px;
    }
    return pc;
}

// CPML of lane l of an x-derivative pair inside an x-strip (d1 with the
// integer-grid coefficients, d2 with the half-grid ones): its memories m1/m2
// at m are advanced from o1/o2 and stored (unless `store` is false), and its
// derivatives corrected.  The roundings are spelled out (b*o + round(a*d),
// then d*iK + m, as the packed z-strip update does) so that every kernel
// inlining this computes the same bits.
__device__ __forceinline__ void cpml_x_lane(const Cpml& c, size_t m, float o1, float o2, float* __restrict__ a1,
                                            float* __restrict__ a2, float& e1, float& e2, bool store = true) {
    const float m1 = __fmaf_rn(c.b, o1, __fmul_rn(c.a, e1));
    const float m2 = __fmaf_rn(c.bh, o2, __fmul_rn(c.ah, e2));
    if (store) {
        a1[m] = m1;
        a2[m] = m2;
    }
    e1 = __fmaf_rn(e1, c.iK, m1);
    e2 = __fmaf_rn(e2, c.iKh, m2);
}
// sxx on the free-surface row (forward_kernel_PSV_GPU.cu:917-927):
// vx_x * 2 M2 (L + M2/2) / (L + M2) with L = dt lam, M2 = 2 dt mu, roundings spelled out.
__device__ __forceinline__ float fsurf_sxx(float vx_x, float L, float M2) {
    return __fdiv_rn(__fmul_rn(vx_x, __fmul_rn(__fmul_rn(2.f, M2), __fmaf_rn(0.5f, M2, L))), __fadd_rn(L, M2));
}
// Both lanes of a pair, each lane's coefficients read at the row (L1 hits):
// the stress and adjoint passes, where holding them across rows costs spills.
__device__ __forceinline__ void cpml_x_pair(const PairCols& pc, const float* __restrict__ cpml, int iz, int tp,
                                            const float (&o1)[2], const float (&o2)[2], float* __restrict__ a1,
                                            float* __restrict__ a2, float2& d1, float2& d2) {
#pragma unroll
    for (int l = 0; l < 2; l++)
        if (pc.px[l] >= 0 && inb(pc.px[l], tp, 1))
            cpml_x_lane(load_cpml6(cpml, tp, pc.px[l]), (size_t)iz * tp + pc.px[l], o1[l], o2[l], a1, a2,
                        l ? d1.y : d1.x, l ? d2.y : d2.x);
}
// Both lanes with coefficients cx[l] read once per tile (load_cpml_x): the
// velocity pass up to half order 4, whose two rows share them.
__device__ __forceinline__ void load_cpml_x(const PairCols& pc, const float* __restrict__ cpml, int tp,
                                            Cpml (&cx)[2]) {
#pragma unroll
    for (int l = 0; l < 2; l++)
        if (pc.px[l] >= 0 && inb(pc.px[l], tp, 21)) cx[l] = load_cpml6(cpml, tp, pc.px[l]);
}
__device__ __forceinline__ void cpml_x_pair(const PairCols& pc, const Cpml (&cx)[2], int iz, int tp,
                                            const float (&o1)[2], const float (&o2)[2], float* __restrict__ a1,
                                            float* __restrict__ a2, float2& d1, float2& d2) {
#pragma unroll
    for (int l = 0; l < 2; l++)
        if (pc.px[l] >= 0 && inb(pc.px[l], tp, 2))
            cpml_x_lane(cx[l], (size_t)iz * tp + pc.px[l], o1[l], o2[l], a1, a2, l ? d1.y : d1.x, l ? d2.y : d2.x);
}

// z-strip index of row iz (-1 outside the strips); the stress pass's top strip
// includes row ppad, the velocity pass's does not.
template <int FP>
__device__ __forceinline__ int strip_z(const ItemDesc& D, int iz, bool stress) {
    int pz = -1;
    if (D.npml > 0 && iz < D.nzt - FP) {
        if (!D.fsurf && (stress ? iz <= D.ppad : iz < D.ppad)) pz = iz - FP;
        else if (iz >= D.nzt - D.ppad - 1) pz = iz - D.pnz;
        if (pz == D.npml) pz = -1;
    }
    return pz;
}

// ---------------------------------------------------------------------------
// stress pass
// ---------------------------------------------------------------------------
// Copies of one tile into a stage: `desc` is the tile's slot descriptor, `b`
// the slot coordinate of the 3-D state maps.
template <int FP>
__device__ __forceinline__ void stress_issue(const StressMaps& m, const ItemDesc* desc, int b, int x0, int z0,
                                             float* st, uint64_t* bar) {
    using G = TmaGeom<FP>;
    constexpr unsigned bytes = 4u * (2 * G::WX * G::WZ + 6 * G::CEN) + (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::S_DESC, desc, (unsigned)sizeof(ItemDesc), bar);
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

template <int FP, bool INTERIOR>
__device__ __forceinline__ void stress_rows(const ItemDesc& D, const float* st, int x0, int z0, int it,
                                            unsigned flags, const float2 (&hx)[FP], const float2 (&hz)[FP],
                                            long long msrc, int lt) {
    using G = TmaGeom<FP>;
    constexpr int R = kPairRows;
    constexpr int W = R + 2 * FP - 1;
    const int cp = (lt & (kTmaTX / 2 - 1)) * 2;  // tile column of the pair
    const int r0 = (lt / (kTmaTX / 2)) * R;
    const int ix = x0 + cp;
    PairCols pc = {true, true, {-1, -1}};
    if constexpr (!INTERIOR) {
        pc = pair_cols<FP>(D, ix, true);
        if (!pc.on0 && !pc.on1) return;
    }
    const int nzt = D.nzt, P = D.pitch, tp = D.tp;
    const float* svx = st;
    const float* svz = st + G::HXZ;
    const float* cen = st + 2 * G::HXZ;
    const int col = cp + G::HX;
    // z-windows: wvx[j] = vx pair of row r0 + j - FP + 1, wvz[j] = vz pair of row r0 + j - FP
    float2 wvx[W], wvz[W];
#pragma unroll
    for (int j = 0; j < W; j++) {
        wvx[j] = ld2(svx + (r0 + j + 1) * G::WX + col);
        wvz[j] = ld2(svz + (r0 + j) * G::WX + col);
    }
    const bool fsurf = D.fsurf != 0;
    float* __restrict__ gsxx = D.sxx;
    float* __restrict__ gszx = D.szx;
    float* __restrict__ gszz = D.szz;
    float* __restrict__ mvx_x = D.mvx_x;
    float* __restrict__ mvz_x = D.mvz_x;
    float* __restrict__ mvx_z = D.mvx_z;
    float* __restrict__ mvz_z = D.mvz_z;
    // CPML memories of both rows, loaded before any row is computed
    float mx1[R][2], mx2[R][2];
    float2 mz1[R], mz2[R];
    int pzr[R];
    // z-strip coefficients loaded with the memories before the row loop (inside
    // it their loads wait behind the previous row's CPML stores); above half
    // order 4, per row, as held across the rows they cost spills
    constexpr bool kHoistCz = FP <= 4;
    Cpml czr[R];
    int xf[2] = {-1, -1};
    if constexpr (!INTERIOR) {
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int iz = z0 + r0 + rr;
            mz1[rr] = mz2[rr] = make_float2(0.f, 0.f);
#pragma unroll
            for (int l = 0; l < 2; l++) {
                mx1[rr][l] = mx2[rr][l] = 0.f;
                if (pc.px[l] >= 0 && iz < nzt - FP && inb((long long)iz * tp + pc.px[l], FWI_NXS(D), 11)) {
                    mx1[rr][l] = (mvx_x + msrc)[(size_t)iz * tp + pc.px[l]];
                    mx2[rr][l] = (mvz_x + msrc)[(size_t)iz * tp + pc.px[l]];
                }
            }
            pzr[rr] = strip_z<FP>(D, iz, true);
            if (pzr[rr] >= 0 && !(inb(pzr[rr], tp, 12) && inb((long long)pzr[rr] * P + ix + 1, FWI_NZS(D), 12)))
                pzr[rr] = -1;
            if (pzr[rr] >= 0) {
                mz1[rr] = ld2(mvz_z + msrc + (size_t)pzr[rr] * P + ix);
                mz2[rr] = ld2(mvx_z + msrc + (size_t)pzr[rr] * P + ix);
                if constexpr (kHoistCz) czr[rr] = load_cpml6(D.cpml, tp, pzr[rr]);
            }
        }
        // sampled window columns (forward storage for the gradient)
        if ((flags & FL_STORE) && D.store) {
#pragma unroll
            for (int l = 0; l < 2; l++) {
                const int i = ix + l;
                if ((l ? pc.on1 : pc.on0) && i >= D.wx1 && i < D.wx2 && (i - D.wx1) % D.fwi_dx == 0)
                    xf[l] = (i - D.wx1) / D.fwi_dx;
            }
        }
    }
    // FL_REVERSE undoes the step (s^n = s^{n+1} - S(v^n)); used only without
    // CPML and free surface, where the update is a pure increment
    const float2 sg = bc2((flags & FL_REVERSE) ? -1.f : 1.f);
    size_t c = (size_t)(z0 + r0) * P + ix;  // global index of the pair in the current row
#pragma unroll
    for (int rr = 0; rr < R; rr++, c += P) {
        const int r = r0 + rr;
        const int iz = z0 + r;
        if constexpr (!INTERIOR) {
            if (iz >= nzt - FP) break;
        }
        const int row = r + FP;
        RowPairs<FP> tvx, tvz;
        tvx.load(svx + row * G::WX + col, wvx[rr + FP - 1]);
        tvz.load(svz + row * G::WX + col, wvz[rr + FP]);
        float2 vx_x = tvx.dminus(hx);
        float2 vz_x = tvz.dplus(hx);
        float2 vx_z = make_float2(0.f, 0.f), vz_z = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_z = fma2(hz[k - 1], sub2(wvx[rr + k + FP - 1], wvx[rr - k + FP]), vx_z);
            vz_z = fma2(hz[k - 1], sub2(wvz[rr + k - 1 + FP], wvz[rr - k + FP]), vz_z);
        }
        if constexpr (!INTERIOR) {
            cpml_x_pair(pc, D.cpml, iz, tp, mx1[rr], mx2[rr], mvx_x, mvz_x, vx_x, vz_x);
            if (pzr[rr] >= 0) {
                Cpml cz;
                if constexpr (kHoistCz) cz = czr[rr];
                else cz = load_cpml6(D.cpml, tp, pzr[rr]);
                const size_t m = (size_t)pzr[rr] * P + ix;
                const float2 m1 = fma2(bc2(cz.b), mz1[rr], mul2(bc2(cz.a), vz_z));
                const float2 m2 = fma2(bc2(cz.bh), mz2[rr], mul2(bc2(cz.ah), vx_z));
                st2(mvz_z + m, m1, pc.on0, pc.on1);
                st2(mvx_z + m, m2, pc.on0, pc.on1);
                vz_z = fma2(vz_z, bc2(cz.iK), m1);
                vx_z = fma2(vx_z, bc2(cz.iKh), m2);
            }
        }
        const int ci = r * kTmaTX + cp;
        const float2 L = ld2(cen + ci), M2 = ld2(cen + G::CEN + ci), MZ = ld2(cen + 2 * G::CEN + ci);
        float2 sxx = ld2(cen + 3 * G::CEN + ci), szx = ld2(cen + 4 * G::CEN + ci), szz = ld2(cen + 5 * G::CEN + ci);
        if constexpr (!INTERIOR) {
            if ((xf[0] >= 0 || xf[1] >= 0) && iz >= D.wz1 && iz < D.wz2 && (iz - D.wz1) % D.fwi_dz == 0) {
                const size_t fs = (size_t)D.nfz * D.nfx;
                const size_t so = (size_t)(it / D.fwi_dt) * 5 * fs + (size_t)((iz - D.wz1) / D.fwi_dz) * D.nfx;
                float* s = D.store + so;
#pragma unroll
                for (int l = 0; l < 2; l++) {
                    if (xf[l] < 0 ||
                        !inb((long long)(so + xf[l] + 4 * fs), (long long)(1 + (D.nt - 1) / D.fwi_dt) * 5 * fs, 14))
                        continue;
                    float* q = s + xf[l];
                    q[F_VX * fs] = lane(wvx[rr + FP - 1], l) / D.dt;
                    q[F_VZ * fs] = lane(wvz[rr + FP], l) / D.dt;
                    q[F_SXX * fs] = lane(sxx, l);
                    q[F_SZX * fs] = lane(szx, l);
                    q[F_SZZ * fs] = lane(szz, l);
                }
            }
        }
        szx = fma2(sg, mul2(MZ, add2(vz_x, vx_z)), szx);
        const float2 tr = mul2(L, add2(vx_x, vz_z));
        sxx = fma2(sg, fma2(M2, vx_x, tr), sxx);
        szz = fma2(sg, fma2(M2, vz_z, tr), szz);
        if (!inb((long long)c + 1, FWI_NFIELD(D), 13)) continue;
        if constexpr (INTERIOR) {
            *reinterpret_cast<float2*>(gsxx + c) = sxx;
            *reinterpret_cast<float2*>(gszx + c) = szx;
            *reinterpret_cast<float2*>(gszz + c) = szz;
        } else {
            if (fsurf && iz == FP) {
                szz = make_float2(0.f, 0.f);
                szx = make_float2(0.f, 0.f);
                sxx.x = fsurf_sxx(vx_x.x, L.x, M2.x);
                sxx.y = fsurf_sxx(vx_x.y, L.y, M2.y);
            }
            st2(gsxx + c, sxx, pc.on0, pc.on1);
            st2(gszx + c, szx, pc.on0, pc.on1);
            st2(gszz + c, szz, pc.on0, pc.on1);
            if (fsurf && iz > FP && iz <= 2 * FP) {
                const size_t cm = (size_t)(2 * FP - iz) * P + ix;
                st2(gszx + cm, make_float2(-szx.x, -szx.y), pc.on0, pc.on1);
                st2(gszz + cm, make_float2(-szz.x, -szz.y), pc.on0, pc.on1);
            }
        }
    }
}

template <int FP>
__device__ __forceinline__ void stress_compute(const ItemDesc& D, const TmaGrid& g, const float* st, int x0, int z0,
                                               int it, unsigned flags, const float2 (&hx)[FP],
                                               const float2 (&hz)[FP], int lt) {
    if (interior_warp(g, x0, z0, flags, lt)) stress_rows<FP, true>(D, st, x0, z0, it, flags, hx, hz, g.msrc, lt);
    else stress_rows<FP, false>(D, st, x0, z0, it, flags, hx, hz, g.msrc, lt);
}

// ---------------------------------------------------------------------------
// velocity pass (+ energy)
// ---------------------------------------------------------------------------
template <int FP>
__device__ __forceinline__ void velocity_issue(const VelMaps& m, const ItemDesc* desc, int b, int x0, int z0,
                                               float* st, uint64_t* bar, bool we) {
    using G = TmaGeom<FP>;
    const unsigned bytes = 4u * (G::WX * G::TZ + G::WX * G::WZ + G::TX * G::WZ + (we ? 5 : 4) * G::CEN) +
                           (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::V_DESC, desc, (unsigned)sizeof(ItemDesc), bar);
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

// The same with the stresses from `ms` and velocities, buoyancies and energy
// from `mv` (a step out of one state buffer into another: the stresses were
// just written to the destination, the velocities are still in the source).
template <int FP>
__device__ __forceinline__ void velocity_issue2(const VelMaps& ms, const VelMaps& mv, const ItemDesc* desc, int b,
                                                int x0, int z0, float* st, uint64_t* bar, bool we) {
    using G = TmaGeom<FP>;
    const unsigned bytes = 4u * (G::WX * G::TZ + G::WX * G::WZ + G::TX * G::WZ + (we ? 5 : 4) * G::CEN) +
                           (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::V_DESC, desc, (unsigned)sizeof(ItemDesc), bar);
    tma_load_3d(st, &ms.sxx, x0 - G::HX, z0, b, bar);
    tma_load_3d(st + G::HXO, &ms.szx, x0 - G::HX, z0 - FP, b, bar);
    tma_load_3d(st + G::HXO + G::HXZ, &ms.szz, x0, z0 - FP, b, bar);
    float* c = st + G::HXO + G::HXZ + G::HZO;
    tma_load_2d(c, &mv.BX, x0, z0, bar);
    tma_load_2d(c + G::CEN, &mv.BZ, x0, z0, bar);
    tma_load_3d(c + 2 * G::CEN, &mv.vx, x0, z0, b, bar);
    tma_load_3d(c + 3 * G::CEN, &mv.vz, x0, z0, b, bar);
    if (we) tma_load_3d(c + 4 * G::CEN, &mv.We, x0, z0, b, bar);
}

template <int FP, bool INTERIOR>
__device__ __forceinline__ void velocity_rows(const ItemDesc& D, const float* st, int x0, int z0, unsigned flags,
                                              const float2 (&hx)[FP], const float2 (&hz)[FP], long long msrc,
                                              int lt) {
    using G = TmaGeom<FP>;
    constexpr int R = kPairRows;
    constexpr int W = R + 2 * FP - 1;
    const int cp = (lt & (kTmaTX / 2 - 1)) * 2;
    const int r0 = (lt / (kTmaTX / 2)) * R;
    const int ix = x0 + cp;
    PairCols pc = {true, true, {-1, -1}};
    if constexpr (!INTERIOR) {
        pc = pair_cols<FP>(D, ix, false);
        if (!pc.on0 && !pc.on1) return;
    }
    const int nzt = D.nzt, P = D.pitch, tp = D.tp;
    const float* ssxx = st;                    // [TZ][WX]
    const float* sszx = st + G::HXO;           // [WZ][WX]
    const float* sszz = st + G::HXO + G::HXZ;  // [WZ][TX]
    const float* cen = st + G::HXO + G::HXZ + G::HZO;
    const int col = cp + G::HX;
    // z-windows: wsx[j] = szx pair of row r0 + j - FP, wsz[j] = szz pair of row r0 + j - FP + 1
    float2 wsx[W], wsz[W];
#pragma unroll
    for (int j = 0; j < W; j++) {
        wsx[j] = ld2(sszx + (r0 + j) * G::WX + col);
        wsz[j] = ld2(sszz + (r0 + j + 1) * G::TX + cp);
    }
    float* __restrict__ gvx = D.vx;
    float* __restrict__ gvz = D.vz;
    float* __restrict__ gwe = D.We;
    float* __restrict__ msxx_x = D.msxx_x;
    float* __restrict__ mszx_x = D.mszx_x;
    float* __restrict__ mszz_z = D.mszz_z;
    float* __restrict__ mszx_z = D.mszx_z;
    float mx1[R][2], mx2[R][2];
    float2 mz1[R], mz2[R];
    int pzr[R];
    // x-strip coefficients read once per tile up to half order 4 (both rows use
    // them); above, per row, as held across the rows they cost spills
    constexpr bool kHoistCx = FP <= 4;
    Cpml cx[2];
    // z-strip coefficients likewise (as in the stress pass)
    constexpr bool kHoistCz = FP <= 4;
    Cpml czr[R];
    if constexpr (!INTERIOR) {
        if constexpr (kHoistCx) load_cpml_x(pc, D.cpml, tp, cx);
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int iz = z0 + r0 + rr;
            mz1[rr] = mz2[rr] = make_float2(0.f, 0.f);
#pragma unroll
            for (int l = 0; l < 2; l++) {
                mx1[rr][l] = mx2[rr][l] = 0.f;
                if (pc.px[l] >= 0 && iz < nzt - FP && inb((long long)iz * tp + pc.px[l], FWI_NXS(D), 22)) {
                    mx1[rr][l] = (msxx_x + msrc)[(size_t)iz * tp + pc.px[l]];
                    mx2[rr][l] = (mszx_x + msrc)[(size_t)iz * tp + pc.px[l]];
                }
            }
            pzr[rr] = strip_z<FP>(D, iz, false);
            if (pzr[rr] >= 0 && !(inb(pzr[rr], tp, 23) && inb((long long)pzr[rr] * P + ix + 1, FWI_NZS(D), 23)))
                pzr[rr] = -1;
            if (pzr[rr] >= 0) {
                mz1[rr] = ld2(mszz_z + msrc + (size_t)pzr[rr] * P + ix);
                mz2[rr] = ld2(mszx_z + msrc + (size_t)pzr[rr] * P + ix);
                if constexpr (kHoistCz) czr[rr] = load_cpml6(D.cpml, tp, pzr[rr]);
            }
        }
    }
    const bool we = (flags & FL_WE) != 0;
    const float2 sg = bc2((flags & FL_REVERSE) ? -1.f : 1.f);  // v^n = v^{n+1} - V(s^{n+1})
    size_t c = (size_t)(z0 + r0) * P + ix;
#pragma unroll
    for (int rr = 0; rr < R; rr++, c += P) {
        const int r = r0 + rr;
        const int iz = z0 + r;
        if constexpr (!INTERIOR) {
            if (iz >= nzt - FP) break;
        }
        RowPairs<FP> tsx, tzx;
        // sxx has no z halo: its centre pair is not in a window
        tsx.load(ssxx + r * G::WX + col, ld2(ssxx + r * G::WX + col));
        tzx.load(sszx + (r + FP) * G::WX + col, wsx[rr + FP]);
        float2 sxx_x = tsx.dplus(hx);
        float2 szx_x = tzx.dminus(hx);
        float2 szx_z = make_float2(0.f, 0.f), szz_z = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            szx_z = fma2(hz[k - 1], sub2(wsx[rr + k - 1 + FP], wsx[rr - k + FP]), szx_z);
            szz_z = fma2(hz[k - 1], sub2(wsz[rr + k + FP - 1], wsz[rr - k + FP]), szz_z);
        }
        if constexpr (!INTERIOR) {
            if constexpr (kHoistCx) cpml_x_pair(pc, cx, iz, tp, mx1[rr], mx2[rr], msxx_x, mszx_x, sxx_x, szx_x);
            else cpml_x_pair(pc, D.cpml, iz, tp, mx1[rr], mx2[rr], msxx_x, mszx_x, sxx_x, szx_x);
            if (pzr[rr] >= 0) {
                Cpml cz;
                if constexpr (kHoistCz) cz = czr[rr];
                else cz = load_cpml6(D.cpml, tp, pzr[rr]);
                const size_t m = (size_t)pzr[rr] * P + ix;
                const float2 m1 = fma2(bc2(cz.b), mz1[rr], mul2(bc2(cz.a), szz_z));
                const float2 m2 = fma2(bc2(cz.bh), mz2[rr], mul2(bc2(cz.ah), szx_z));
                st2(mszz_z + m, m1, pc.on0, pc.on1);
                st2(mszx_z + m, m2, pc.on0, pc.on1);
                szz_z = fma2(szz_z, bc2(cz.iK), m1);
                szx_z = fma2(szx_z, bc2(cz.iKh), m2);
            }
        }
        const int ci = r * kTmaTX + cp;
        const float2 vxn = fma2(sg, mul2(ld2(cen + ci), add2(sxx_x, szx_z)), ld2(cen + 2 * G::CEN + ci));
        const float2 vzn = fma2(sg, mul2(ld2(cen + G::CEN + ci), add2(szx_x, szz_z)), ld2(cen + 3 * G::CEN + ci));
        if (!inb((long long)c + 1, FWI_NFIELD(D), 24)) continue;
        if constexpr (INTERIOR) {
            if (we)
                *reinterpret_cast<float2*>(gwe + c) = add2(ld2(cen + 4 * G::CEN + ci), fma2(vxn, vxn, mul2(vzn, vzn)));
            *reinterpret_cast<float2*>(gvx + c) = vxn;
            *reinterpret_cast<float2*>(gvz + c) = vzn;
        } else {
            if (we) st2(gwe + c, add2(ld2(cen + 4 * G::CEN + ci), fma2(vxn, vxn, mul2(vzn, vzn))), pc.on0, pc.on1);
            st2(gvx + c, vxn, pc.on0, pc.on1);
            st2(gvz + c, vzn, pc.on0, pc.on1);
        }
    }
}

// Source injection and receiver recording are not done here: the engine runs
// them in a separate small kernel after this pass (events_kernel).
template <int FP>
__device__ __forceinline__ void velocity_compute(const ItemDesc& D, const TmaGrid& g, const float* st, int x0,
                                                 int z0, unsigned flags, const float2 (&hx)[FP],
                                                 const float2 (&hz)[FP], int lt) {
    if (interior_warp(g, x0, z0, flags, lt)) velocity_rows<FP, true>(D, st, x0, z0, flags, hx, hz, g.msrc, lt);
    else velocity_rows<FP, false>(D, st, x0, z0, flags, hx, hz, g.msrc, lt);
}

// Stencil weights of a launch (every slot of a launch has the same grid),
// read once per CTA and held in registers as broadcast pairs.
template <int FP>
__device__ __forceinline__ void load_weights(const ItemDesc* items, float2 (&hx)[FP], float2 (&hz)[FP]) {
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = bc2(__ldg(&items[0].hx[k]));
        hz[k] = bc2(__ldg(&items[0].hz[k]));
    }
}

// ---------------------------------------------------------------------------
// persistent pipelined kernels
// ---------------------------------------------------------------------------
// Body shared by the passes.  COORDS(t, &b, &x0, &z0) names tile t of the
// launch (b: its slot or model); ISSUE(b, x0, z0, stage_ptr, bar) queues its
// copies; COMPUTE(tile, next, stage_ptr, k) runs its cells.  The issuing
// thread writes each tile's coordinates beside the barriers, so the other
// threads do no integer division per tile.
// Every pass here reads nothing another tile of its launch writes, and no
// warp needs data of another, so there is no CTA barrier per tile: each warp,
// once done with a stage, counts itself on the stage's release counter, and
// the warp that completes the count refills the stage with the CTA's tile S
// ahead.  A warp may so run up to S-1 tiles ahead of the slowest one, instead
// of every warp of a tile waiting at a barrier for the warps holding its CPML
// strips.  k is the CTA's tile count, from which the passes rotate the warps'
// roles: warp w does the rows and columns of warp (w + k) mod nwarps of the
// plain mapping, so the strip work of edge tiles falls on every warp in turn
// rather than on the same ones.  With NEXT the issuing thread also stores the
// coordinates of the CTA's following tile beside each stage's own (a warp
// cannot read them from that tile's stage, which may not be refilled yet);
// without, next is (-1, 0, 0).
// A wait that gives up sets bit 2 of the error word and the abort word; the
// other warps leave at their next tile (or when their own wait gives up, the
// released count of a stage never completing), and after a CTA barrier one
// thread waits, bounded, for the last copy issued into each stage.
template <int STAGES>
__host__ __device__ constexpr size_t tma_tail_bytes() {
    return STAGES * (2 * sizeof(int4) + sizeof(uint64_t) + 2 * sizeof(unsigned)) + 16;
}

__device__ __forceinline__ unsigned atom_add_acq_rel_cta(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;"
                 : "=r"(old)
                 : "r"(smem_u32(p)), "r"(v)
                 : "memory");
    return old;
}

template <int FP, int STAGE_FLOATS, bool NEXT = false, class Coords, class Issue, class Compute>
__device__ __forceinline__ void tma_pipeline(int ntiles, int* err, Coords coords, Issue issue, Compute compute,
                                             unsigned long long wait_ns = 0, int stall = 0) {
    constexpr int S = stages_for<STAGE_FLOATS>();
    const unsigned long long lim = wait_ns ? wait_ns : kWaitNs;
    static_assert(STAGE_FLOATS % 32 == 0, "stages are 128-byte multiples");
    extern __shared__ __align__(128) float tma_smem[];
    int4* crd = reinterpret_cast<int4*>(tma_smem + S * STAGE_FLOATS);
    int4* nxt = crd + S;  // with NEXT: the CTA's tile after the stage's
    uint64_t* bar = reinterpret_cast<uint64_t*>(nxt + S);
    unsigned* released = reinterpret_cast<unsigned*>(bar + S);  // running count of warps done per stage
    unsigned* issued = released + S;                            // copies issued into each stage
    volatile int* abort = reinterpret_cast<volatile int*>(issued + S);
    const int tid = threadIdx.x, lane = tid & 31;
    const unsigned nwarps = blockDim.x >> 5;
    // an earlier launch gave up (error word set): return at once, so a failing
    // pipeline costs one bounded wait and not one per launch; the decision is
    // CTA-uniform (every thread reaches the barrier)
    if (__syncthreads_or(*(volatile int*)err != 0)) return;
    if (smem_u32(tma_smem) & 127u) {  // TMA destinations need 128-byte alignment
        if (tid == 0) atomicOr(err, 8);
        return;
    }
    const int first = blockIdx.x, step = gridDim.x;
    auto issue_tile = [&](int t, int s) {
        int b, x0, z0;
        coords(t, &b, &x0, &z0);
        crd[s] = make_int4(b, x0, z0, 0);
        if constexpr (NEXT) {
            if (t + step < ntiles) {
                int b1, x1, z1;
                coords(t + step, &b1, &x1, &z1);
                nxt[s] = make_int4(b1, x1, z1, 0);
            } else {
                nxt[s] = make_int4(-1, 0, 0, 0);
            }
        }
        issued[s] += 1u;
        issue(b, x0, z0, tma_smem + s * STAGE_FLOATS, &bar[s]);
    };
    if (tid == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&bar[s], 1);
            released[s] = 0u;
            issued[s] = 0u;
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (stall && blockIdx.x == 0) mbar_expect_tx_only(&bar[0], 16u);
        for (int s = 0; s < S; s++) {
            const int t = first + s * step;
            if (t < ntiles) issue_tile(t, s);
        }
    }
    __syncthreads();
    for (int k = 0;; k++) {
        const int t = first + k * step;
        if (t >= ntiles || __any_sync(0xffffffffu, *abort != 0)) break;
        const int s = k % S;
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(&bar[s], (unsigned)((k / S) & 1), lim))) {
            if (lane == 0) {
                *abort = 1;
                atomicOr(err, 4);
            }
            break;
        }
        compute(crd[s], NEXT ? nxt[s] : make_int4(-1, 0, 0, 0), tma_smem + s * STAGE_FLOATS, k);
        // the warp's reads of stage s are done; the release (acq_rel atomic)
        // orders them before the refill's async-proxy writes
        __syncwarp();
        if (lane == 0 && (atom_add_acq_rel_cta(&released[s], 1u) + 1u) % nwarps == 0u) {
            const int tn = first + (k + S) * step;
            if (tn < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_tile(tn, s);
            }
        }
    }
    __syncthreads();
    if (tid == 0 && *abort) {
        for (int s = 0; s < S; s++)
            if (issued[s]) mbar_wait_bounded(&bar[s], (issued[s] - 1u) & 1u, lim);
    }
}

// Logical thread of the plain mapping (NT threads) that thread threadIdx.x
// plays in the CTA's k-th tile (warp rotation, above).
template <int NT = kFwdThreads>
__device__ __forceinline__ int rotated_thread(int k) {
    static_assert(NT % 32 == 0, "whole warps");
    if constexpr ((NT & (NT - 1)) == 0) return (int)((threadIdx.x + ((unsigned)k << 5)) & (NT - 1));
    else return (int)((threadIdx.x + ((unsigned)k % (NT / 32)) * 32u) % (unsigned)NT);
}

template <int FP>
constexpr size_t stress_tma_smem() {
    constexpr int S = stages_for<TmaGeom<FP>::S_STAGE>();
    return sizeof(float) * S * TmaGeom<FP>::S_STAGE + tma_tail_bytes<S>();
}
template <int FP>
constexpr size_t velocity_tma_smem() {
    constexpr int S = stages_for<TmaGeom<FP>::V_STAGE>();
    return sizeof(float) * S * TmaGeom<FP>::V_STAGE + tma_tail_bytes<S>();
}
static_assert(stress_tma_smem<4>() <= 232448 && velocity_tma_smem<4>() <= 232448, "shared memory per CTA");
static_assert(stress_tma_smem<6>() <= 232448 && velocity_tma_smem<6>() <= 232448, "shared memory per CTA");

template <int FP>
__global__ void __launch_bounds__(kFwdThreads, 1)
    stress_tma_kernel(const __grid_constant__ StressMaps maps, const ItemDesc* __restrict__ items,
                      const TmaGrid g, int it, unsigned flags, int* err) {
    using G = TmaGeom<FP>;
    float2 hx[FP], hz[FP];
    load_weights<FP>(items, hx, hz);
    tma_pipeline<FP, G::S_STAGE>(
        g.ntiles, err, [&](int t, int* b, int* x0, int* z0) { tile_coords(g, t, b, x0, z0, FP, kTmaTZ); },
        [&](int b, int x0, int z0, float* st, uint64_t* bar) {
            stress_issue<FP>(maps, items + b, b, x0, z0, st, bar);
        },
        [&](int4 c, int4, const float* st, int k) {
            stress_compute<FP>(*reinterpret_cast<const ItemDesc*>(st + G::S_DESC), g, st, c.y, c.z, it, flags, hx,
                               hz, rotated_thread(k));
        },
        g.wait_ns, g.stall);
}

template <int FP>
__global__ void __launch_bounds__(kFwdThreads, 1)
    velocity_tma_kernel(const __grid_constant__ VelMaps maps, const ItemDesc* __restrict__ items,
                        const TmaGrid g, int it, unsigned flags, int* err) {
    using G = TmaGeom<FP>;
    const bool we = (flags & FL_WE) != 0;
    float2 hx[FP], hz[FP];
    load_weights<FP>(items, hx, hz);
    tma_pipeline<FP, G::V_STAGE>(
        g.ntiles, err, [&](int t, int* b, int* x0, int* z0) { tile_coords(g, t, b, x0, z0, FP, kTmaTZ); },
        [&](int b, int x0, int z0, float* st, uint64_t* bar) {
            velocity_issue<FP>(maps, items + b, b, x0, z0, st, bar, we);
        },
        [&](int4 c, int4, const float* st, int k) {
            velocity_compute<FP>(*reinterpret_cast<const ItemDesc*>(st + G::V_DESC), g, st, c.y, c.z, flags, hx, hz,
                                 rotated_thread(k));
        },
        g.wait_ns);
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
    constexpr int S = stages_for<AdjGeom<FP>::STAGE>();
    return sizeof(float) * S * AdjGeom<FP>::STAGE + tma_tail_bytes<S>();
}
static_assert(adjoint_tma_smem<4>() <= 232448 && adjoint_tma_smem<6>() <= 232448, "shared memory per CTA");

template <int FP>
__device__ __forceinline__ void adjoint_issue(const AdjMaps& m, const ItemDesc* desc, int b, int x0, int z0,
                                              float* st, uint64_t* bar, bool grad) {
    using G = AdjGeom<FP>;
    const unsigned bytes = 4u * (2 * G::WX * G::WZ + (grad ? 13 : 8) * G::CEN) + (unsigned)sizeof(ItemDesc);
    mbar_expect_tx(bar, bytes);
    bulk_load(st + G::DESC, desc, (unsigned)sizeof(ItemDesc), bar);
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

// The adjoint pass maps a column pair to each thread and one tile row
// (64 pairs x 8 rows); warp w covers 64 columns of tile row w / 2.
static_assert((kTmaTX / 2) * kAdjTZ == kAdjThreads, "one thread per column pair of a row");

// The warp's cells are plain-stencil cells and, on a gradient step, lie in
// the gradient window sampled at unit intervals.
__device__ __forceinline__ bool interior_warp_adj(const TmaGrid& g, int x0, int z0, bool grad_step, int lt) {
    const int w = lt >> 5;
    const int wx0 = x0 + (w & 1) * 64, wz = z0 + (w >> 1);
    bool in = wx0 >= g.cxl && wx0 + 63 <= g.cxh && wz >= g.czl && wz <= g.czh;
    if (grad_step) in = in && wx0 >= g.gxl && wx0 + 63 <= g.gxh && wz >= g.gzl && wz <= g.gzh;
    return in;
}

__device__ __forceinline__ float* ldg_ptr(float* const* p) {
    return reinterpret_cast<float*>(__ldg(reinterpret_cast<const unsigned long long*>(p)));
}

// Gradient samples of an interior warp's pair loaded one tile ahead: the
// loads are issued at the end of the previous tile, so their DRAM latency
// passes while the CTA waits for and computes the current one.
struct GradAhead {
    float g[6];  // lam, mu, rho of the two columns
    bool valid;
};

// Reciprocal with the approximate instruction (relative error ~1 ulp; the
// gradient's tolerance is 1e-4 relative L2).
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <int FP, bool INTERIOR, bool GRAD>
__device__ __forceinline__ void adjoint_rows(const ItemDesc& D, const float* st, int x0, int z0,
                                             const float2 (&hx)[FP], const float2 (&hz)[FP], const GradAhead& ga,
                                             int lt) {
    constexpr bool grad_step = GRAD;
    using G = AdjGeom<FP>;
    const int cp = (lt & (kTmaTX / 2 - 1)) * 2;
    const int r = lt / (kTmaTX / 2);  // tile row
    const int ix = x0 + cp, iz = z0 + r;
    const int P = D.pitch, tp = D.tp;
    PairCols pc = {true, true, {-1, -1}};
    if constexpr (!INTERIOR) {
        if (iz >= D.nzt - FP) return;
        pc = pair_cols<FP>(D, ix, true);
        if (!pc.on0 && !pc.on1) return;
    }
    const size_t c = (size_t)iz * P + ix;
    // gradient samples of the pair (prefetched: their loads overlap the stencil)
    int gi[2] = {-1, -1};
    float g0[2] = {0.f, 0.f}, g1[2] = {0.f, 0.f}, g2[2] = {0.f, 0.f};
    float* __restrict__ glam = D.glam;
    float* __restrict__ gmu = D.gmu;
    float* __restrict__ grho = D.grho;
    if constexpr (grad_step) {
        if constexpr (INTERIOR) {
            gi[0] = (iz - D.wz1) * D.nfx + (ix - D.wx1);
            gi[1] = gi[0] + 1;
        } else {
            const int dzw = iz - D.wz1;
            if (iz >= D.wz1 && iz < D.wz2 && (D.fwi_dz == 1 || dzw % D.fwi_dz == 0)) {
                const int zf = D.fwi_dz == 1 ? dzw : dzw / D.fwi_dz;
#pragma unroll
                for (int l = 0; l < 2; l++) {
                    const int dxw = ix + l - D.wx1;
                    if ((l ? pc.on1 : pc.on0) && dxw >= 0 && ix + l < D.wx2 && (D.fwi_dx == 1 || dxw % D.fwi_dx == 0))
                        gi[l] = zf * D.nfx + (D.fwi_dx == 1 ? dxw : dxw / D.fwi_dx);
                }
            }
        }
#pragma unroll
        for (int l = 0; l < 2; l++)
            if ((INTERIOR || gi[l] >= 0) && !inb(gi[l], FWI_NGRAD(D), 31)) gi[l] = -2;  // -2: skipped
        if (INTERIOR && ga.valid) {
#pragma unroll
            for (int l = 0; l < 2; l++) {
                g0[l] = ga.g[l];
                g1[l] = ga.g[2 + l];
                g2[l] = ga.g[4 + l];
            }
        } else {
#pragma unroll
            for (int l = 0; l < 2; l++) {
                if (gi[l] >= 0) {
                    g0[l] = glam[gi[l]];
                    g1[l] = gmu[gi[l]];
                    g2[l] = grho[gi[l]];
                }
            }
        }
    }
    // CPML memories of the pair, and the z-strip coefficients of its row (up
    // to half order 4: loaded here, not after the stencil where the load
    // would sit on the update's path)
    float mx1[2] = {0.f, 0.f}, mx2[2] = {0.f, 0.f};
    float2 mz1 = make_float2(0.f, 0.f), mz2 = make_float2(0.f, 0.f);
    int pz = -1;
    constexpr bool kHoistCz = FP <= 4;
    Cpml cz0;
    if constexpr (!INTERIOR) {
#pragma unroll
        for (int l = 0; l < 2; l++) {
            if (pc.px[l] >= 0 && inb((long long)iz * tp + pc.px[l], FWI_NXS(D), 33)) {
                mx1[l] = D.mvx_x[(size_t)iz * tp + pc.px[l]];
                mx2[l] = D.mvz_x[(size_t)iz * tp + pc.px[l]];
            }
        }
        pz = strip_z<FP>(D, iz, true);
        if (pz >= 0 && !(inb(pz, tp, 34) && inb((long long)pz * P + ix + 1, FWI_NZS(D), 34))) pz = -1;
        if (pz >= 0) {
            mz1 = ld2(D.mvz_z + (size_t)pz * P + ix);
            mz2 = ld2(D.mvx_z + (size_t)pz * P + ix);
            if constexpr (kHoistCz) cz0 = load_cpml6(D.cpml, tp, pz);
        }
    }
    const float* svx = st;
    const float* svz = st + G::HXZ;
    const float* cen = st + 2 * G::HXZ;
    const int col = cp + G::HX;
    const int row = r + FP;
    const float2 cvx = ld2(svx + row * G::WX + col), cvz = ld2(svz + row * G::WX + col);
    RowPairs<FP> tvx, tvz;
    tvx.load(svx + row * G::WX + col, cvx);
    tvz.load(svz + row * G::WX + col, cvz);
    float2 vx_x = tvx.dminus(hx);
    float2 vz_x = tvz.dplus(hx);
    // z taps straight from the stage: vx D+ (rows r+k, r-k+1), vz D- (rows r+k-1, r-k)
    float2 vx_z = make_float2(0.f, 0.f), vz_z = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 1; k <= FP; k++) {
        const float2 a = ld2(svx + (row + k) * G::WX + col);
        const float2 bb = k == 1 ? cvx : ld2(svx + (row - k + 1) * G::WX + col);
        const float2 e = k == 1 ? cvz : ld2(svz + (row + k - 1) * G::WX + col);
        const float2 f = ld2(svz + (row - k) * G::WX + col);
        vx_z = fma2(hz[k - 1], sub2(a, bb), vx_z);
        vz_z = fma2(hz[k - 1], sub2(e, f), vz_z);
    }
    if constexpr (!INTERIOR) {
        cpml_x_pair(pc, D.cpml, iz, tp, mx1, mx2, D.mvx_x, D.mvz_x, vx_x, vz_x);
        if (pz >= 0) {
            Cpml cz;
            if constexpr (kHoistCz) cz = cz0;
            else cz = load_cpml6(D.cpml, tp, pz);
            const size_t m = (size_t)pz * P + ix;
            const float2 m1 = fma2(bc2(cz.b), mz1, mul2(bc2(cz.a), vz_z));
            const float2 m2 = fma2(bc2(cz.bh), mz2, mul2(bc2(cz.ah), vx_z));
            st2(D.mvz_z + m, m1, pc.on0, pc.on1);
            st2(D.mvx_z + m, m2, pc.on0, pc.on1);
            vz_z = fma2(vz_z, bc2(cz.iK), m1);
            vx_z = fma2(vx_z, bc2(cz.iKh), m2);
        }
    }
    const int ci = r * kTmaTX + cp;
    const float2 L = ld2(cen + ci), M2 = ld2(cen + G::CEN + ci), MZ = ld2(cen + 2 * G::CEN + ci);
    float2 sxx = ld2(cen + 3 * G::CEN + ci), szx = ld2(cen + 4 * G::CEN + ci), szz = ld2(cen + 5 * G::CEN + ci);
    const float2 dt2 = bc2(D.dt);
    const float2 ux = fma2(dt2, cvx, ld2(cen + 6 * G::CEN + ci));
    const float2 uz = fma2(dt2, cvz, ld2(cen + 7 * G::CEN + ci));
    if (GRAD && (INTERIOR || gi[0] >= 0 || gi[1] >= 0)) {
        // the stored velocities are v/dt; reciprocals in place of the divisions
        // (rounding within the gradient tolerance)
        const float2 idt = bc2(D.inv_dt);
        const float2 fvx = mul2(ld2(cen + 8 * G::CEN + ci), idt), fvz = mul2(ld2(cen + 9 * G::CEN + ci), idt);
        const float2 fsxx = ld2(cen + 10 * G::CEN + ci), fszx = ld2(cen + 11 * G::CEN + ci);
        const float2 fszz = ld2(cen + 12 * G::CEN + ci);
        const float2 lpm = mul2(fma2(bc2(0.5f), M2, L), idt);
        const float2 mu = mul2(mul2(bc2(0.5f), M2), idt);
        const float2 lpm2 = mul2(lpm, lpm), mu2 = mul2(mu, mu);
        const float2 ilpm2 = make_float2(0.25f * rcp_approx(lpm2.x), 0.25f * rcp_approx(lpm2.y));
        const float2 imu2 = make_float2(rcp_approx(mu2.x), rcp_approx(mu2.y));
        const float2 s1 = mul2(mul2(add2(fsxx, fszz), add2(sxx, szz)), ilpm2);
        const float2 s2 = mul2(mul2(sub2(fsxx, fszz), sub2(sxx, szz)), imu2);
        const float2 s3 = mul2(mul2(fszx, szx), imu2);
        const float2 s4 = fma2(ux, fvx, mul2(uz, fvz));
        const float2 gs = bc2(D.gscale);
        const float2 nl = fma2(gs, s1, make_float2(g0[0], g0[1]));
        const float2 nm = fma2(gs, add2(add2(s3, s1), s2), make_float2(g1[0], g1[1]));
        const float2 nr = fma2(make_float2(-D.gscale, -D.gscale), s4, make_float2(g2[0], g2[1]));
#pragma unroll
        for (int l = 0; l < 2; l++) {
            if ((INTERIOR && (!FWI_BOUNDS_CHECK || gi[l] != -2)) || gi[l] >= 0) {
                glam[gi[l]] = lane(nl, l);
                gmu[gi[l]] = lane(nm, l);
                grho[gi[l]] = lane(nr, l);
            }
        }
    }
    szx = add2(szx, mul2(MZ, add2(vz_x, vx_z)));
    const float2 tr = mul2(L, add2(vx_x, vz_z));
    sxx = add2(sxx, fma2(M2, vx_x, tr));
    szz = add2(szz, fma2(M2, vz_z, tr));
    if (!inb((long long)c + 1, FWI_NFIELD(D), 35)) return;
    if constexpr (INTERIOR) {
        *reinterpret_cast<float2*>(D.ux + c) = ux;
        *reinterpret_cast<float2*>(D.uz + c) = uz;
        *reinterpret_cast<float2*>(D.sxx + c) = sxx;
        *reinterpret_cast<float2*>(D.szx + c) = szx;
        *reinterpret_cast<float2*>(D.szz + c) = szz;
    } else {
        const bool fsurf = D.fsurf != 0;
        if (fsurf && iz == FP) {
            szz = make_float2(0.f, 0.f);
            szx = make_float2(0.f, 0.f);
            sxx.x = fsurf_sxx(vx_x.x, L.x, M2.x);
            sxx.y = fsurf_sxx(vx_x.y, L.y, M2.y);
        }
        st2(D.ux + c, ux, pc.on0, pc.on1);
        st2(D.uz + c, uz, pc.on0, pc.on1);
        st2(D.sxx + c, sxx, pc.on0, pc.on1);
        st2(D.szx + c, szx, pc.on0, pc.on1);
        st2(D.szz + c, szz, pc.on0, pc.on1);
        if (fsurf && iz > FP && iz <= 2 * FP) {
            const size_t cm = (size_t)(2 * FP - iz) * P + ix;
            st2(D.szx + cm, make_float2(-szx.x, -szx.y), pc.on0, pc.on1);
            st2(D.szz + cm, make_float2(-szz.x, -szz.y), pc.on0, pc.on1);
        }
    }
}

template <int FP>
__global__ void __launch_bounds__(kAdjThreads, 1)
    adjoint_tma_kernel(const __grid_constant__ AdjMaps maps, const ItemDesc* __restrict__ items, const TmaGrid g,
                       int it, unsigned flags, int* err) {
    using G = AdjGeom<FP>;
    const bool grad = (flags & FL_GRAD) != 0;
    float2 hx[FP], hz[FP];
    load_weights<FP>(items, hx, hz);
    // gradient window origin and row length (the same for every slot)
    const int wx1 = __ldg(&items[0].wx1), wz1 = __ldg(&items[0].wz1), nfx = __ldg(&items[0].nfx);
    GradAhead ga;
    ga.valid = false;
    tma_pipeline<FP, G::STAGE, true>(
        g.ntiles, err, [&](int t, int* b, int* x0, int* z0) { tile_coords(g, t, b, x0, z0, FP, kAdjTZ); },
        [&](int b, int x0, int z0, float* st, uint64_t* bar) {
            adjoint_issue<FP>(maps, items + b, b, x0, z0, st, bar, grad);
        },
        [&](int4 c, int4 n, const float* st, int k) {
            const ItemDesc& D = *reinterpret_cast<const ItemDesc*>(st + G::DESC);
            const int lt = rotated_thread<kAdjThreads>(k);
            const bool in = interior_warp_adj(g, c.y, c.z, grad, lt);
            if (grad) {
                if (in) adjoint_rows<FP, true, true>(D, st, c.y, c.z, hx, hz, ga, lt);
                else adjoint_rows<FP, false, true>(D, st, c.y, c.z, hx, hz, ga, lt);
            } else {
                if (in) adjoint_rows<FP, true, false>(D, st, c.y, c.z, hx, hz, ga, lt);
                else adjoint_rows<FP, false, false>(D, st, c.y, c.z, hx, hz, ga, lt);
            }
            ga.valid = false;
            // gradient samples of this thread's cells in the CTA's next tile
            // (its role there is that of rotation k + 1)
            const int ln = rotated_thread<kAdjThreads>(k + 1);
            if (grad && n.x >= 0 && interior_warp_adj(g, n.y, n.z, true, ln)) {
                const ItemDesc* In = items + n.x;
                const int gi = (n.z + ln / (kTmaTX / 2) - wz1) * nfx + (n.y + (ln & (kTmaTX / 2 - 1)) * 2 - wx1);
                if (!inb((long long)gi + 1, (long long)__ldg(&In->nfz) * nfx, 36)) return;
                const float* gl = ldg_ptr(&In->glam);
                const float* gm = ldg_ptr(&In->gmu);
                const float* gr = ldg_ptr(&In->grho);
                ga.g[0] = gl[gi];
                ga.g[1] = gl[gi + 1];
                ga.g[2] = gm[gi];
                ga.g[3] = gm[gi + 1];
                ga.g[4] = gr[gi];
                ga.g[5] = gr[gi + 1];
                ga.valid = true;
            }
        },
        g.wait_ns);
}

// ---------------------------------------------------------------------------
// independent models of uneven size in one launch (multi-model engine)
// ---------------------------------------------------------------------------
// Per model, the tensor maps of its states (one slot each) live in device
// memory, written by the host before the launches, and the TMA copies take
// them by address.  The tile work-list gives (model, x0, z0); the stencil
// weights and the plain-stencil ranges come from the model's staged
// descriptor.  Models of one half order share a launch.
struct MultiMaps {
    StressMaps sf;  // forward state, stress pass
    VelMaps vf;     // forward state, velocity pass (energy Ws)
    VelMaps va;     // adjoint state, velocity pass (energy Wr)
    AdjMaps a;      // adjoint stress pass: adjoint state, ux/uz, forward fields
};

// Plain-stencil ranges of one model: the rule the single-model engine applies
// on the host for its TmaGrid.
__device__ __forceinline__ TmaGrid model_ranges(const ItemDesc& D) {
    TmaGrid g{};
    const int fp = D.fpad;
    g.cxl = fp;
    g.cxh = D.nxt - fp - 1;
    g.czl = fp;
    g.czh = D.nzt - fp - 1;
    if (D.npml > 0) {
        g.cxl = max(g.cxl, D.ppad + 1);
        g.cxh = min(g.cxh, D.nxt - D.ppad - 2);
        g.czh = min(g.czh, D.nzt - D.ppad - 2);
        if (!D.fsurf) g.czl = max(g.czl, D.ppad + 1);
    }
    if (D.fsurf) g.czl = max(g.czl, 2 * fp + 1);
    g.gxl = g.gzl = 0;
    g.gxh = g.gzh = -1;
    if (D.fwi_dx == 1 && D.fwi_dz == 1) {
        g.gxl = D.wx1;
        g.gxh = D.wx2 - 1;
        g.gzl = D.wz1;
        g.gzh = D.wz2 - 1;
    }
    return g;
}

template <int FP>
__device__ __forceinline__ void staged_weights(const ItemDesc& D, float2 (&hx)[FP], float2 (&hz)[FP]) {
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = bc2(D.hx[k]);
        hz[k] = bc2(D.hz[k]);
    }
}

// Launch arguments: mx = the maps of the buffer the state is read from, my =
// of the buffer it is written to, items = the descriptors writing to my's
// buffer, msrc = (source - destination) in floats for the CPML memories
// (mx == my and msrc == 0 in place).
template <int FP>
__global__ void __launch_bounds__(kFwdThreads, 1)
    stress_tma_multi_kernel(const MultiMaps* __restrict__ mx, const MultiMaps* __restrict__ my,
                            const ItemDesc* __restrict__ items, const Tile* __restrict__ tiles, int ntiles, int it,
                            unsigned flags, long long msrc, int* err) {
    const MultiMaps* maps = mx;
    using G = TmaGeom<FP>;
    tma_pipeline<FP, G::S_STAGE>(
        ntiles, err,
        [&](int t, int* b, int* x0, int* z0) {
            const Tile T = tiles[t];
            *b = T.item;
            *x0 = T.x0;
            *z0 = T.z0;
        },
        [&](int b, int x0, int z0, float* st, uint64_t* bar) {
            stress_issue<FP>(maps[b].sf, items + b, 0, x0, z0, st, bar);
        },
        [&](int4 c, int4, const float* st, int k) {
            const ItemDesc& D = *reinterpret_cast<const ItemDesc*>(st + G::S_DESC);
            float2 hx[FP], hz[FP];
            staged_weights<FP>(D, hx, hz);
            TmaGrid gg = model_ranges(D);
            gg.msrc = msrc;
            stress_compute<FP>(D, gg, st, c.y, c.z, it, flags, hx, hz, rotated_thread(k));
        });
}

template <int FP>
__global__ void __launch_bounds__(kFwdThreads, 1)
    velocity_tma_multi_kernel(const MultiMaps* __restrict__ mx, const MultiMaps* __restrict__ my,
                              const ItemDesc* __restrict__ items, const Tile* __restrict__ tiles, int ntiles, int it,
                              unsigned flags, int adj, long long msrc, int* err) {
    using G = TmaGeom<FP>;
    const bool we = (flags & FL_WE) != 0;
    tma_pipeline<FP, G::V_STAGE>(
        ntiles, err,
        [&](int t, int* b, int* x0, int* z0) {
            const Tile T = tiles[t];
            *b = T.item;
            *x0 = T.x0;
            *z0 = T.z0;
        },
        [&](int b, int x0, int z0, float* st, uint64_t* bar) {
            if (adj) velocity_issue<FP>(mx[b].va, items + b, 0, x0, z0, st, bar, we);
            else velocity_issue2<FP>(my[b].vf, mx[b].vf, items + b, 0, x0, z0, st, bar, we);
        },
        [&](int4 c, int4, const float* st, int k) {
            const ItemDesc& D = *reinterpret_cast<const ItemDesc*>(st + G::V_DESC);
            float2 hx[FP], hz[FP];
            staged_weights<FP>(D, hx, hz);
            TmaGrid gg = model_ranges(D);
            gg.msrc = msrc;
            velocity_compute<FP>(D, gg, st, c.y, c.z, flags, hx, hz, rotated_thread(k));
        });
}

// mx: the maps whose forward fields (AdjMaps::fv*) name the buffer holding
// the forward state.
template <int FP>
__global__ void __launch_bounds__(kAdjThreads, 1)
    adjoint_tma_multi_kernel(const MultiMaps* __restrict__ mx, const ItemDesc* __restrict__ items,
                             const Tile* __restrict__ tiles, int ntiles, int it, unsigned flags, int* err) {
    const MultiMaps* maps = mx;
    using G = AdjGeom<FP>;
    const bool grad = (flags & FL_GRAD) != 0;
    GradAhead none;
    none.valid = false;
    tma_pipeline<FP, G::STAGE>(
        ntiles, err,
        [&](int t, int* b, int* x0, int* z0) {
            const Tile T = tiles[t];
            *b = T.item;
            *x0 = T.x0;
            *z0 = T.z0;
        },
        [&](int b, int x0, int z0, float* st, uint64_t* bar) {
            adjoint_issue<FP>(maps[b].a, items + b, 0, x0, z0, st, bar, grad);
        },
        [&](int4 c, int4, const float* st, int k) {
            const ItemDesc& D = *reinterpret_cast<const ItemDesc*>(st + G::DESC);
            float2 hx[FP], hz[FP];
            staged_weights<FP>(D, hx, hz);
            const int lt = rotated_thread<kAdjThreads>(k);
            const bool in = interior_warp_adj(model_ranges(D), c.y, c.z, grad, lt);
            if (grad) {
                if (in) adjoint_rows<FP, true, true>(D, st, c.y, c.z, hx, hz, none, lt);
                else adjoint_rows<FP, false, true>(D, st, c.y, c.z, hx, hz, none, lt);
            } else {
                if (in) adjoint_rows<FP, true, false>(D, st, c.y, c.z, hx, hz, none, lt);
                else adjoint_rows<FP, false, false>(D, st, c.y, c.z, hx, hz, none, lt);
            }
        });
}

}  // namespace fwi
