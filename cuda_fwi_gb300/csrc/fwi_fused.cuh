// fwi_fused.cuh -- one launch per forward time step: the stress update and the
// velocity update of a batch of shots fused into a single pass over HBM.
//
// Same arithmetic as the two TMA passes of fwi_tma.cuh (stress_rows and
// velocity_rows: forward_kernel_PSV_GPU.cu:830-1023 generalised to fdorder
// 2..8), statement for statement, so the results are bit-identical to the
// two-pass step; what changes is the traffic.  The two-pass step reads v,
// reads and writes s (stress pass), then reads s again, reads and writes v
// (velocity pass): 60 B per cell and shot.  Here each cell's five fields are
// read once and written once: 40 B.
//
// Work decomposition.  A unit is one shot's column strip of W owned columns
// (W = 128 - 2 HX, HX = FP rounded up to 4: 120 columns up to order 8).  A
// persistent CTA (512 threads, one per SM) marches each of its units down the
// grid in chunks of TZ = 16 rows.  For a chunk whose stress rows are
// [z, z+16), one TMA stage brings
//   vx, vz   rows [z-FP, z+16+FP), columns [x0-2HX, x0+W+2HX)
//   sxx, szx, szz and L, M2, MZ   rows [z, z+16), columns [x0-HX, x0+W+HX)
//   BX, BZ   rows [z-FP, z+16-FP), columns [x0, x0+W)
// The new stresses are computed on all 128 columns (the strip and HX halo
// columns each side -- the halo columns are recomputed, identically, by the
// neighbouring strip, which owns them) into a ring in shared memory that also
// keeps the previous chunk's last 2 FP rows; the velocity update of rows
// [z-FP, z+16-FP) then reads its x- and z-taps from that ring.  Only owned
// columns are written to HBM.
//
// Because a strip's halo columns are read while the neighbouring strip may
// already be writing its step, the state is double-buffered: the step reads
// buffer X (state n) and writes buffer Y (state n+1), X != Y.  Cells no step
// updates (border columns and rows) are zero in every buffer.
//
// Per chunk: one bounded mbarrier wait by one thread and a CTA barrier (which
// also releases the previous chunk's stage for its refill), the stress
// phase, a barrier, the velocity phase.  Source injection and receiver
// recording run in the engine's small events kernel after the launch.
#pragma once

#include "fwi_tma.cuh"

namespace fwi {

constexpr int kFusedTZ = 16;        // rows per chunk
constexpr int kFusedThreads = 512;  // 64 column pairs x 8 row pairs
constexpr int kFusedMaxHalf = 4;    // fdorder <= 8 (the stages of higher orders exceed shared memory)

template <int FP>
struct FusedGeom {
    static_assert(FP >= 1 && FP <= kFusedMaxHalf, "fused step: fdorder 2..8");
    static constexpr int TZ = kFusedTZ;
    static constexpr int HX = 4;                   // halo columns of the stress region (>= FP, 16-byte rule)
    static constexpr int SX = 128;                 // stress columns per strip
    static constexpr int W = SX - 2 * HX;          // owned (velocity) columns per strip
    static constexpr int VX = SX + 2 * HX;         // velocity box width
    static constexpr int VZ = TZ + 2 * FP;         // velocity box height
    static constexpr int pad(int n) { return (n + 31) / 32 * 32; }  // 128-byte sub-buffers
    static constexpr int VB = pad(VX * VZ);
    static constexpr int SB = SX * TZ;
    static constexpr int BB = pad(W * TZ);
    static constexpr int O_S = 2 * VB;             // old sxx, szx, szz
    static constexpr int O_M = O_S + 3 * SB;       // L, M2, MZ
    static constexpr int O_B = O_M + 3 * SB;       // BX, BZ
    static constexpr int O_D = O_B + 2 * BB;       // slot descriptor (of the destination buffer)
    static constexpr int STAGE = O_D + kDescFloats;
    static constexpr int NR = TZ + 2 * FP;         // ring rows: [z - 2FP, z + TZ)
    static constexpr int NSF = NR * SX;
    static constexpr int NS = 3 * NSF;
    static_assert(TZ >= 2 * FP, "the ring's head rows are the previous chunk's last rows");
    static constexpr unsigned BYTES = 4u * (2 * VX * VZ + 6 * SB + 2 * W * TZ) + (unsigned)sizeof(ItemDesc);
};
template <int FP>
constexpr size_t fused_smem() {
    return sizeof(float) * (2 * FusedGeom<FP>::STAGE + FusedGeom<FP>::NS) + 2 * sizeof(uint64_t) + 16;
}
static_assert(fused_smem<4>() <= 232448, "shared memory per CTA");

// Tensor maps of one source buffer (the state fields) and of the materials.
struct FusedMaps {
    CUtensorMap vx, vz, sxx, szx, szz, L, M2, MZ, BX, BZ;
};

// Launch description: units are (shot, strip), shot-minor; chunks of a unit
// run top to bottom.  [cxl, cxh] x [czl, czh]: plain-stencil cells (as in
// TmaGrid).  msrc: source - destination buffer offset (floats) for the CPML
// memories.  wait_ns: limit of each bounded wait.  stall: a test hook -- the
// first chunk of CTA 0 expects 16 bytes more than its copies deliver, so its
// wait runs out (the failure path of a copy that never completes).
struct FusedGrid {
    int nb, nunits, nch, stall;
    int cxl, cxh, czl, czh;
    long long msrc;
    unsigned long long wait_ns;
};

template <int FP>
__device__ __forceinline__ void fused_issue(const FusedMaps& m, const ItemDesc* desc, int b, int x0, int z,
                                            float* st, uint64_t* bar) {
    using G = FusedGeom<FP>;
    mbar_expect_tx(bar, G::BYTES);
    bulk_load(st + G::O_D, desc, (unsigned)sizeof(ItemDesc), bar);
    tma_load_3d(st, &m.vx, x0 - 2 * G::HX, z - FP, b, bar);
    tma_load_3d(st + G::VB, &m.vz, x0 - 2 * G::HX, z - FP, b, bar);
    float* s = st + G::O_S;
    tma_load_3d(s, &m.sxx, x0 - G::HX, z, b, bar);
    tma_load_3d(s + G::SB, &m.szx, x0 - G::HX, z, b, bar);
    tma_load_3d(s + 2 * G::SB, &m.szz, x0 - G::HX, z, b, bar);
    float* c = st + G::O_M;
    tma_load_2d(c, &m.L, x0 - G::HX, z, bar);
    tma_load_2d(c + G::SB, &m.M2, x0 - G::HX, z, bar);
    tma_load_2d(c + 2 * G::SB, &m.MZ, x0 - G::HX, z, bar);
    tma_load_2d(st + G::O_B, &m.BX, x0, z - FP, bar);
    tma_load_2d(st + G::O_B + G::BB, &m.BZ, x0, z - FP, bar);
}

// x-strip CPML of both lanes of a pair; the memories are stored only for the
// strip's own columns (a halo column's memory belongs to the neighbour).
__device__ __forceinline__ void cpml_x_pair_own(const PairCols& pc, const float* __restrict__ cpml, int iz, int tp,
                                                const float (&o1)[2], const float (&o2)[2], float* __restrict__ a1,
                                                float* __restrict__ a2, float2& d1, float2& d2, bool own) {
#pragma unroll
    for (int l = 0; l < 2; l++)
        if (pc.px[l] >= 0 && inb(pc.px[l], tp, 41))
            cpml_x_lane(load_cpml6(cpml, tp, pc.px[l]), (size_t)iz * tp + pc.px[l], o1[l], o2[l], a1, a2,
                        l ? d1.y : d1.x, l ? d2.y : d2.x, own);
}

// A pair with the lanes outside the updated columns zeroed (the ring holds
// zero there, as HBM does for cells no step updates).
__device__ __forceinline__ float2 masked(float2 v, const PairCols& pc) {
    return make_float2(pc.on0 ? v.x : 0.f, pc.on1 ? v.y : 0.f);
}

// ---------------------------------------------------------------------------
// stress phase: rows [z, z+TZ) of the 128 stress columns, into the ring
// ---------------------------------------------------------------------------
template <int FP, bool INTERIOR>
__device__ __forceinline__ void fused_stress(const ItemDesc& D, const float* st, float* ns, int x0, int z, bool first,
                                             int it, unsigned flags, const float2 (&hx)[FP], const float2 (&hz)[FP],
                                             long long msrc) {
    using G = FusedGeom<FP>;
    constexpr int R = 2;
    constexpr int WIN = R + 2 * FP - 1;
    const int cs = (threadIdx.x & 63) * 2;  // stress column of the pair within the strip's 128
    const int r0 = (threadIdx.x >> 6) * R;  // chunk row of the pair's first row
    const int ix = x0 - G::HX + cs;
    const bool own = cs >= G::HX && cs < G::HX + G::W;  // both lanes (W and HX are even)
    const int nzt = D.nzt, P = D.pitch, tp = D.tp;
    const bool fsurf = D.fsurf != 0;
    PairCols pc = {true, true, {-1, -1}};
    if constexpr (!INTERIOR) pc = pair_cols<FP>(D, ix, true);
    const bool any = pc.on0 || pc.on1;
    float* nsxx = ns;
    float* nszx = ns + G::NSF;
    float* nszz = ns + 2 * G::NSF;
    // Ring head rows [0, 2FP) = stress rows [z-2FP, z): the previous chunk's ring
    // rows [TZ, TZ+2FP), which are exactly the rows this thread overwrites below
    // (chunk rows [TZ-2FP, TZ)), so it moves them itself before writing.  The
    // first chunk of a unit has no previous rows: zero (rows above the grid and
    // the unupdated border rows), except the free-surface mirror rows of
    // interior columns, which the rows below write.
    if (r0 >= G::TZ - 2 * FP) {
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int src = 2 * FP + r0 + rr, dst = src - G::TZ;
            const int os = src * G::SX + cs, od = dst * G::SX + cs;
            if (!first) {
                *reinterpret_cast<float2*>(nsxx + od) = ld2(nsxx + os);
                *reinterpret_cast<float2*>(nszx + od) = ld2(nszx + os);
                *reinterpret_cast<float2*>(nszz + od) = ld2(nszz + os);
            } else {
                const int y = z - 2 * FP + dst;
                const bool mirror = fsurf && y >= 0 && y < FP && any;
                *reinterpret_cast<float2*>(nsxx + od) = make_float2(0.f, 0.f);
                if (!mirror) {
                    *reinterpret_cast<float2*>(nszx + od) = make_float2(0.f, 0.f);
                    *reinterpret_cast<float2*>(nszz + od) = make_float2(0.f, 0.f);
                }
            }
        }
    }
    if (!any) {  // border or beyond-grid columns: the ring holds zero
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int o = (2 * FP + r0 + rr) * G::SX + cs;
            *reinterpret_cast<float2*>(nsxx + o) = make_float2(0.f, 0.f);
            *reinterpret_cast<float2*>(nszx + o) = make_float2(0.f, 0.f);
            *reinterpret_cast<float2*>(nszz + o) = make_float2(0.f, 0.f);
        }
        return;
    }
    const float* svx = st;
    const float* svz = st + G::VB;
    const float* sold = st + G::O_S;
    const float* mat = st + G::O_M;
    const int col = cs + G::HX;  // column in the velocity boxes
    // z-windows: wvx[j] = vx pair of row r0 + j - FP + 1, wvz[j] = vz pair of row r0 + j - FP
    float2 wvx[WIN], wvz[WIN];
#pragma unroll
    for (int j = 0; j < WIN; j++) {
        wvx[j] = ld2(svx + (r0 + j + 1) * G::VX + col);
        wvz[j] = ld2(svz + (r0 + j) * G::VX + col);
    }
    float* __restrict__ gsxx = D.sxx;
    float* __restrict__ gszx = D.szx;
    float* __restrict__ gszz = D.szz;
    float* __restrict__ mvx_x = D.mvx_x;
    float* __restrict__ mvz_x = D.mvz_x;
    float* __restrict__ mvx_z = D.mvx_z;
    float* __restrict__ mvz_z = D.mvz_z;
    float mx1[R][2], mx2[R][2];
    float2 mz1[R], mz2[R];
    int pzr[R];
    int xf[2] = {-1, -1};
    if constexpr (!INTERIOR) {
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int iz = z + r0 + rr;
            mz1[rr] = mz2[rr] = make_float2(0.f, 0.f);
#pragma unroll
            for (int l = 0; l < 2; l++) {
                mx1[rr][l] = mx2[rr][l] = 0.f;
                if (pc.px[l] >= 0 && iz < nzt - FP && inb((long long)iz * tp + pc.px[l], FWI_NXS(D), 42)) {
                    mx1[rr][l] = (mvx_x + msrc)[(size_t)iz * tp + pc.px[l]];
                    mx2[rr][l] = (mvz_x + msrc)[(size_t)iz * tp + pc.px[l]];
                }
            }
            pzr[rr] = strip_z<FP>(D, iz, true);
            if (pzr[rr] >= 0 && !(inb(pzr[rr], tp, 43) && inb((long long)pzr[rr] * P + ix + 1, FWI_NZS(D), 43)))
                pzr[rr] = -1;
            if (pzr[rr] >= 0) {
                mz1[rr] = ld2(mvz_z + msrc + (size_t)pzr[rr] * P + ix);
                mz2[rr] = ld2(mvx_z + msrc + (size_t)pzr[rr] * P + ix);
            }
        }
        if ((flags & FL_STORE) && D.store && own) {
#pragma unroll
            for (int l = 0; l < 2; l++) {
                const int i = ix + l;
                if ((l ? pc.on1 : pc.on0) && i >= D.wx1 && i < D.wx2 && (i - D.wx1) % D.fwi_dx == 0)
                    xf[l] = (i - D.wx1) / D.fwi_dx;
            }
        }
    }
    // the increments are added with a runtime unit factor, as the two-pass
    // kernels do (a constant 1 lets the compiler emit a plain add, whose
    // handling of subnormal values can differ)
    const float2 sg = bc2((flags & FL_REVERSE) ? -1.f : 1.f);
    size_t c = (size_t)(z + r0) * P + ix;
#pragma unroll
    for (int rr = 0; rr < R; rr++, c += P) {
        const int r = r0 + rr;
        const int iz = z + r;
        const int o = (2 * FP + r) * G::SX + cs;  // ring offset of the pair
        if constexpr (!INTERIOR) {
            if (iz >= nzt - FP) {  // below the updated rows: zero, as in HBM
                *reinterpret_cast<float2*>(nsxx + o) = make_float2(0.f, 0.f);
                *reinterpret_cast<float2*>(nszx + o) = make_float2(0.f, 0.f);
                *reinterpret_cast<float2*>(nszz + o) = make_float2(0.f, 0.f);
                continue;
            }
        }
        const int row = r + FP;
        RowPairs<FP> tvx, tvz;
        tvx.load(svx + row * G::VX + col, wvx[rr + FP - 1]);
        tvz.load(svz + row * G::VX + col, wvz[rr + FP]);
        float2 vx_x = tvx.dminus(hx);
        float2 vz_x = tvz.dplus(hx);
        float2 vx_z = make_float2(0.f, 0.f), vz_z = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_z = fma2(hz[k - 1], sub2(wvx[rr + k + FP - 1], wvx[rr - k + FP]), vx_z);
            vz_z = fma2(hz[k - 1], sub2(wvz[rr + k - 1 + FP], wvz[rr - k + FP]), vz_z);
        }
        if constexpr (!INTERIOR) {
            cpml_x_pair_own(pc, D.cpml, iz, tp, mx1[rr], mx2[rr], mvx_x, mvz_x, vx_x, vz_x, own);
            if (pzr[rr] >= 0) {
                const Cpml cz = load_cpml6(D.cpml, tp, pzr[rr]);
                const size_t m = (size_t)pzr[rr] * P + ix;
                const float2 m1 = fma2(bc2(cz.b), mz1[rr], mul2(bc2(cz.a), vz_z));
                const float2 m2 = fma2(bc2(cz.bh), mz2[rr], mul2(bc2(cz.ah), vx_z));
                st2(mvz_z + m, m1, pc.on0 && own, pc.on1 && own);
                st2(mvx_z + m, m2, pc.on0 && own, pc.on1 && own);
                vz_z = fma2(vz_z, bc2(cz.iK), m1);
                vx_z = fma2(vx_z, bc2(cz.iKh), m2);
            }
        }
        const int ci = r * G::SX + cs;
        const float2 L = ld2(mat + ci), M2 = ld2(mat + G::SB + ci), MZ = ld2(mat + 2 * G::SB + ci);
        float2 sxx = ld2(sold + ci), szx = ld2(sold + G::SB + ci), szz = ld2(sold + 2 * G::SB + ci);
        if constexpr (!INTERIOR) {
            if ((xf[0] >= 0 || xf[1] >= 0) && iz >= D.wz1 && iz < D.wz2 && (iz - D.wz1) % D.fwi_dz == 0) {
                const size_t fs = (size_t)D.nfz * D.nfx;
                const size_t so = (size_t)(it / D.fwi_dt) * 5 * fs + (size_t)((iz - D.wz1) / D.fwi_dz) * D.nfx;
                float* s = D.store + so;
#pragma unroll
                for (int l = 0; l < 2; l++) {
                    if (xf[l] < 0 ||
                        !inb((long long)(so + xf[l] + 4 * fs), (long long)(1 + (D.nt - 1) / D.fwi_dt) * 5 * fs, 44))
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
        // global stores only where the index is in range (the ring below always)
        const bool gok = inb((long long)c + 1, FWI_NFIELD(D), 45);
        if constexpr (INTERIOR) {
            if (own && gok) {
                *reinterpret_cast<float2*>(gsxx + c) = sxx;
                *reinterpret_cast<float2*>(gszx + c) = szx;
                *reinterpret_cast<float2*>(gszz + c) = szz;
            }
            *reinterpret_cast<float2*>(nsxx + o) = sxx;
            *reinterpret_cast<float2*>(nszx + o) = szx;
            *reinterpret_cast<float2*>(nszz + o) = szz;
        } else {
            if (fsurf && iz == FP) {
                szz = make_float2(0.f, 0.f);
                szx = make_float2(0.f, 0.f);
                sxx.x = fsurf_sxx(vx_x.x, L.x, M2.x);
                sxx.y = fsurf_sxx(vx_x.y, L.y, M2.y);
            }
            st2(gsxx + c, sxx, pc.on0 && own && gok, pc.on1 && own && gok);
            st2(gszx + c, szx, pc.on0 && own && gok, pc.on1 && own && gok);
            st2(gszz + c, szz, pc.on0 && own && gok, pc.on1 && own && gok);
            *reinterpret_cast<float2*>(nsxx + o) = masked(sxx, pc);
            *reinterpret_cast<float2*>(nszx + o) = masked(szx, pc);
            *reinterpret_cast<float2*>(nszz + o) = masked(szz, pc);
            if (fsurf && iz > FP && iz <= 2 * FP) {
                const size_t cm = (size_t)(2 * FP - iz) * P + ix;
                const float2 mx = make_float2(-szx.x, -szx.y), mzz = make_float2(-szz.x, -szz.y);
                const bool mok = inb((long long)cm + 1, FWI_NFIELD(D), 46);
                st2(gszx + cm, mx, pc.on0 && own && mok, pc.on1 && own && mok);
                st2(gszz + cm, mzz, pc.on0 && own && mok, pc.on1 && own && mok);
                // ring row of the mirror row 2FP - iz (head rows of a unit's first chunk)
                const int om = (2 * FP - iz - (z - 2 * FP)) * G::SX + cs;
                *reinterpret_cast<float2*>(nszx + om) = masked(mx, pc);
                *reinterpret_cast<float2*>(nszz + om) = masked(mzz, pc);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// velocity phase: rows [z-FP, z-FP+TZ) of the W owned columns, from the ring
// ---------------------------------------------------------------------------
template <int FP, bool INTERIOR>
__device__ __forceinline__ void fused_velocity(const ItemDesc& D, const float* st, const float* ns, int x0, int q_base,
                                               unsigned flags, const float2 (&hx)[FP], const float2 (&hz)[FP],
                                               long long msrc) {
    using G = FusedGeom<FP>;
    constexpr int R = 2;
    constexpr int WIN = R + 2 * FP - 1;
    const int cv = (threadIdx.x & 63) * 2 - G::HX;  // owned column of the pair
    if (cv < 0 || cv >= G::W) return;
    const int q0 = (threadIdx.x >> 6) * R;
    const int ix = x0 + cv;
    PairCols pc = {true, true, {-1, -1}};
    if constexpr (!INTERIOR) {
        pc = pair_cols<FP>(D, ix, false);
        if (!pc.on0 && !pc.on1) return;
    }
    const int nzt = D.nzt, P = D.pitch, tp = D.tp;
    const float* nsxx = ns;
    const float* nszx = ns + G::NSF;
    const float* nszz = ns + 2 * G::NSF;
    const int ncol = cv + G::HX;  // column in the ring
    // ring row of stress row (q_base + q) is q + FP; z-windows:
    // wsx[j] = szx pair of row q0 + j - FP, wsz[j] = szz pair of row q0 + j - FP + 1
    float2 wsx[WIN], wsz[WIN];
#pragma unroll
    for (int j = 0; j < WIN; j++) {
        wsx[j] = ld2(nszx + (q0 + j) * G::SX + ncol);
        wsz[j] = ld2(nszz + (q0 + j + 1) * G::SX + ncol);
    }
    const float* svx = st;
    const float* svz = st + G::VB;
    const float* sbx = st + G::O_B;
    const float* sbz = st + G::O_B + G::BB;
    const int vcol = cv + 2 * G::HX;  // column in the velocity boxes (box row = q)
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
    constexpr bool kHoistCx = FP <= 4;
    Cpml cx[2];
    if constexpr (!INTERIOR) {
        if constexpr (kHoistCx) load_cpml_x(pc, D.cpml, tp, cx);
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int iz = q_base + q0 + rr;
            mz1[rr] = mz2[rr] = make_float2(0.f, 0.f);
#pragma unroll
            for (int l = 0; l < 2; l++) {
                mx1[rr][l] = mx2[rr][l] = 0.f;
                if (pc.px[l] >= 0 && iz >= FP && iz < nzt - FP &&
                    inb((long long)iz * tp + pc.px[l], FWI_NXS(D), 47)) {
                    mx1[rr][l] = (msxx_x + msrc)[(size_t)iz * tp + pc.px[l]];
                    mx2[rr][l] = (mszx_x + msrc)[(size_t)iz * tp + pc.px[l]];
                }
            }
            pzr[rr] = iz >= FP ? strip_z<FP>(D, iz, false) : -1;
            if (pzr[rr] >= 0 && !(inb(pzr[rr], tp, 48) && inb((long long)pzr[rr] * P + ix + 1, FWI_NZS(D), 48)))
                pzr[rr] = -1;
            if (pzr[rr] >= 0) {
                mz1[rr] = ld2(mszz_z + msrc + (size_t)pzr[rr] * P + ix);
                mz2[rr] = ld2(mszx_z + msrc + (size_t)pzr[rr] * P + ix);
            }
        }
    }
    const bool we = (flags & FL_WE) != 0;
    const float2 sg = bc2((flags & FL_REVERSE) ? -1.f : 1.f);  // as in fused_stress
    size_t c = (size_t)(q_base + q0) * P + ix;
#pragma unroll
    for (int rr = 0; rr < R; rr++, c += P) {
        const int q = q0 + rr;
        const int iz = q_base + q;
        if constexpr (!INTERIOR) {
            if (iz < FP) continue;
            if (iz >= nzt - FP) break;
        }
        RowPairs<FP> tsx, tzx;
        const int nrow = (q + FP) * G::SX + ncol;
        tsx.load(nsxx + nrow, ld2(nsxx + nrow));
        tzx.load(nszx + nrow, wsx[rr + FP]);
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
                const Cpml cz = load_cpml6(D.cpml, tp, pzr[rr]);
                const size_t m = (size_t)pzr[rr] * P + ix;
                const float2 m1 = fma2(bc2(cz.b), mz1[rr], mul2(bc2(cz.a), szz_z));
                const float2 m2 = fma2(bc2(cz.bh), mz2[rr], mul2(bc2(cz.ah), szx_z));
                st2(mszz_z + m, m1, pc.on0, pc.on1);
                st2(mszx_z + m, m2, pc.on0, pc.on1);
                szz_z = fma2(szz_z, bc2(cz.iK), m1);
                szx_z = fma2(szx_z, bc2(cz.iKh), m2);
            }
        }
        const int bi = q * G::W + cv;
        const float2 vxo = ld2(svx + q * G::VX + vcol), vzo = ld2(svz + q * G::VX + vcol);
        const float2 vxn = fma2(sg, mul2(ld2(sbx + bi), add2(sxx_x, szx_z)), vxo);
        const float2 vzn = fma2(sg, mul2(ld2(sbz + bi), add2(szx_x, szz_z)), vzo);
        if (!inb((long long)c + 1, FWI_NFIELD(D), 49)) continue;
        if constexpr (INTERIOR) {
            if (we) *reinterpret_cast<float2*>(gwe + c) = add2(ld2(gwe + c), fma2(vxn, vxn, mul2(vzn, vzn)));
            *reinterpret_cast<float2*>(gvx + c) = vxn;
            *reinterpret_cast<float2*>(gvz + c) = vzn;
        } else {
            if (we) st2(gwe + c, add2(ld2(gwe + c), fma2(vxn, vxn, mul2(vzn, vzn))), pc.on0, pc.on1);
            st2(gvx + c, vxn, pc.on0, pc.on1);
            st2(gvz + c, vzn, pc.on0, pc.on1);
        }
    }
}

// The warp's 64 columns starting at wx0 and its 2 rows starting at wz0 are
// plain-stencil cells (and no storage sample is taken).
__device__ __forceinline__ bool fused_interior(const FusedGrid& g, int wx0, int wz0, unsigned flags) {
    return !(flags & FL_STORE) && wx0 >= g.cxl && wx0 + 63 <= g.cxh && wz0 >= g.czl && wz0 + 1 <= g.czh;
}

template <int FP>
__global__ void __launch_bounds__(kFusedThreads, 1)
    step_fused_kernel(const __grid_constant__ FusedMaps maps, const ItemDesc* __restrict__ items, const FusedGrid g,
                      int it, unsigned flags, int* err) {
    using G = FusedGeom<FP>;
    extern __shared__ __align__(128) float fsm[];
    float* ns = fsm + 2 * G::STAGE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(ns + G::NS);
    volatile int* sflag = reinterpret_cast<volatile int*>(bar + 2);
    const int tid = threadIdx.x;
    // an earlier launch gave up: return at once (CTA-uniform)
    if (__syncthreads_or(*(volatile int*)err != 0)) return;
    if (smem_u32(fsm) & 127u) {
        if (tid == 0) atomicOr(err, 8);
        return;
    }
    float2 hx[FP], hz[FP];
    load_weights<FP>(items, hx, hz);
    const int nch = g.nch;
    auto unit_of = [&](int j) { return (int)blockIdx.x + (j / nch) * (int)gridDim.x; };
    auto exists = [&](int j) { return unit_of(j) < g.nunits; };
    auto issue = [&](int j) {
        const int u = unit_of(j), c = j % nch;
        const int b = u % g.nb;
        fused_issue<FP>(maps, items + b, b, (u / g.nb) * G::W, FP + c * G::TZ, fsm + (j & 1) * G::STAGE,
                        &bar[j & 1]);
    };
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // test hook: 16 more bytes than chunk 0's copies deliver, raised before
        // they are issued, so that phase cannot complete
        if (g.stall && blockIdx.x == 0) mbar_expect_tx_only(&bar[0], 16u);
        if (exists(0)) issue(0);
        if (exists(1)) issue(1);
    }
    __syncthreads();
    const int w = tid >> 5;
    for (int j = 0; exists(j); j++) {
        const int s = j & 1;
        if (tid == 0) *sflag = mbar_wait_bounded(&bar[s], (unsigned)((j >> 1) & 1), g.wait_ns) ? 0 : 1;
        // every thread has finished chunk j-1 (its stage may be refilled) and
        // sees whether chunk j arrived
        __syncthreads();
        if (*sflag) {
            if (tid == 0) {
                atomicOr(err, 4);
                // drain the copies issued and not consumed: chunk j, and chunk 1 when j == 0
                mbar_wait_bounded(&bar[s], (unsigned)((j >> 1) & 1), g.wait_ns);
                if (j == 0 && exists(1)) mbar_wait_bounded(&bar[1], 0u, g.wait_ns);
            }
            return;
        }
        if (tid == 0 && j >= 1 && exists(j + 1)) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(j + 1);
        }
        const float* st = fsm + s * G::STAGE;
        const ItemDesc& D = *reinterpret_cast<const ItemDesc*>(st + G::O_D);
        const int u = unit_of(j), c = j % nch;
        const int x0 = (u / g.nb) * G::W, z = FP + c * G::TZ;
        const int wx0 = x0 - G::HX + (w & 1) * 64;
        if (fused_interior(g, wx0, z + (w >> 1) * 2, flags))
            fused_stress<FP, true>(D, st, ns, x0, z, c == 0, it, flags, hx, hz, g.msrc);
        else
            fused_stress<FP, false>(D, st, ns, x0, z, c == 0, it, flags, hx, hz, g.msrc);
        __syncthreads();  // the ring is complete
        const int qb = z - FP;
        if (fused_interior(g, wx0, qb + (w >> 1) * 2, flags))
            fused_velocity<FP, true>(D, st, ns, x0, qb, flags, hx, hz, g.msrc);
        else
            fused_velocity<FP, false>(D, st, ns, x0, qb, flags, hx, hz, g.msrc);
    }
}

}  // namespace fwi
