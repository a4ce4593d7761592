// fwi_kernels.cuh -- sm_103a stencil kernels of the elastic P-SV FWI hot path.
//
// Reference semantics (Mohammad-debug/CUDA_FWI, paths relative to its root):
//   stress update + CPML on velocity derivatives + free surface
//       CUDA_week2/forward_kernel_PSV_GPU.cu:830-931, mirror :934-942
//   velocity update + CPML on stress derivatives + energy
//       CUDA_week2/forward_kernel_PSV_GPU.cu:946-1023
//   source injection :1033-1047, receiver recording :1049-1063
//   FWI storage (sampled forward wavefield) :803-821
//   adjoint ux/uz integration CUDA_week2/adjoint_kernel_PSV_GPU.cu:818-825,
//   gradient :830-863, residual injection :1077-1087
// The reference implements fdorder 2 only; FP (= fdorder/2) generalises each
// one-sided difference to sum_k hc[k] * (f[i+k] - f[i-k+1]) (D+) and
// sum_k hc[k] * (f[i+k-1] - f[i-k]) (D-).
//
// Layout in HBM (per shot, FP32): every field is [nzt][pitch] with pitch = nxt
// rounded up to 32 floats; the five state fields of one shot are contiguous
// (vx, vz, sxx, szx, szz) and followed by the eight CPML memory arrays
// (x-strips [nzt][tp], z-strips [tp][pitch], tp = 2(npml+1)), so a checkpoint
// of a batch is one contiguous copy.  Materials are stored pre-multiplied by dt:
// L = dt*lam, M2 = 2*dt*mu, MZX = dt*mu_zx, BX = dt*rho_xp, BZ = dt*rho_zp.
//
// Thread mapping: one thread per grid column ix, marching down the rows of a
// z-tile.  The z-taps of the stencil live in a register window that advances
// one row per iteration (each row of vx/vz or szx/szz is loaded once per
// thread); the x-taps are read from the same row (L1 hits).  One launch covers
// a work-list of tiles from every shot of a batch, ordered tile-major so that
// consecutive blocks share the material tile in L2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fwi {

constexpr int kMaxHalf = 6;  // fdorder <= 12

// Rows whose loads are issued ahead of the row being computed (software
// pipelining in registers: each thread keeps PF rows of loads in flight).
#ifndef FWI_PF
#define FWI_PF 1
#endif
constexpr int kPF = FWI_PF;
constexpr int kTileX = 128;  // columns per tile = threads per block

enum Field { F_VX = 0, F_VZ = 1, F_SXX = 2, F_SZX = 3, F_SZZ = 4 };

enum Flags : unsigned {
    FL_STORE = 1u << 0,   // forward: write the sampled window to storage (before the update)
    FL_GRAD = 1u << 1,    // adjoint: accumulate the gradient at this step
    FL_WE = 1u << 2,      // accumulate the energy sum We += vx^2 + vz^2
    FL_INJECT = 1u << 3,  // add the injection signal at source positions
    FL_RECORD = 1u << 4,  // record vz at receiver positions
    FL_REVERSE = 1u << 5, // undo a step: subtract the increments / the injection (TMA mapping)
};

struct __align__(16) ItemDesc {
    int nzt, nxt, pitch, fpad;
    int ppad, npml, tp, pnx;
    int pnz, fsurf, nt, fwi_dt;
    int fwi_dx, fwi_dz, wx1, wx2;
    int wz1, wz2, nfz, nfx;
    int fwd_kind, fwd_xs, pad0, pad1;  // fwd_kind: 0 = storage, 1 = forward state
    long long fwd_fs, fwd_zs;
    float dt, inv_dt, gscale, pad2;    // gscale = fwi_dt * dt
    float hx[kMaxHalf], hz[kMaxHalf];  // dxi*hc[k], dzi*hc[k]
    const float* cpml;                 // [6][tp]: a, b, 1/K, a_half, b_half, 1/K_half
    const float *L, *M2, *MZX, *BX, *BZ;
    float *vx, *vz, *sxx, *szx, *szz, *We;
    float *mvx_x, *mvz_x, *msxx_x, *mszx_x;  // [nzt][tp]
    float *mvx_z, *mvz_z, *mszz_z, *mszx_z;  // [tp][pitch]
    const int* ev_col;                       // [nxt+1] offsets into ev, by column
    const int2* ev;                          // (z, code): code >= 0 inject row, < 0 record row ~code
    const int* ev_x;                         // column of each ev entry (same indexing as ev)
    const float* inj;                        // [rows][nt]
    float* rec;                              // [rows][nt]
    float* store;                            // [nft][5][nfz][nfx]
    float *ux, *uz;                          // adjoint displacement integrals
    float *glam, *gmu, *grho;                // [nfz][nfx]
    const float* fwd;                        // gradient source (see fwd_kind)
};

struct Tile {
    int item, x0, z0, z1;
};

// CPML coefficient bundle of one strip index.
struct Cpml {
    float a, b, iK, ah, bh, iKh;
};

// Bounds-checked debug build (-DFWI_BOUNDS_CHECK=1; compute-sanitizer is not
// available on every GPU host).  inb(i, n, site) guards an access to element i
// of an n-element array: in the checked build an index outside [0, n) records
// the first offending (site, index) in g_fwi_oob and the access is skipped, no
// trap; in the normal build it is true and compiles away.  The engine reads
// the record after each call (FWI_ERR_CUDA "out-of-range index").  Sites of
// the TMA-staged kernels: 1-2 x-strip CPML of a pair, 11-14 forward stress
// pass, 21-24 forward velocity pass, 31-36 adjoint stress pass, 41-49 fused
// forward step.  The cell mappings and the exact adjoint are not guarded.
#ifndef FWI_BOUNDS_CHECK
#define FWI_BOUNDS_CHECK 0
#endif
#if FWI_BOUNDS_CHECK
static __device__ unsigned long long g_fwi_oob;  // site << 48 | index (low 48 bits)
#endif
__device__ __forceinline__ bool inb(long long i, long long n, int site) {
#if FWI_BOUNDS_CHECK
    if (i >= 0 && i < n) return true;
    atomicCAS(&g_fwi_oob, 0ull, ((unsigned long long)site << 48) | ((unsigned long long)i & 0xFFFFFFFFFFFFull));
    return false;
#else
    (void)i, (void)n, (void)site;
    return true;
#endif
}
// Element counts of a slot's arrays: fields [nzt][pitch], x-strip memories
// [nzt][tp], z-strip memories [tp][pitch], gradients [nfz][nfx].
#define FWI_NFIELD(D) ((long long)(D).nzt * (D).pitch)
#define FWI_NXS(D) ((long long)(D).nzt * (D).tp)
#define FWI_NZS(D) ((long long)(D).tp * (D).pitch)
#define FWI_NGRAD(D) ((long long)(D).nfz * (D).nfx)

__device__ __forceinline__ Cpml load_cpml(const float* __restrict__ c, int tp, int p) {
    Cpml r;
    r.a = __ldg(c + p);
    r.b = __ldg(c + tp + p);
    r.iK = __ldg(c + 2 * tp + p);
    r.ah = __ldg(c + 3 * tp + p);
    r.bh = __ldg(c + 4 * tp + p);
    r.iKh = __ldg(c + 5 * tp + p);
    return r;
}

// The engines store a grid's coefficient table as [6][tp] (a, b, 1/K, a_half,
// b_half, 1/K_half per strip index) followed by the same values per index,
// [tp][6]: the TMA-staged kernels read one index with three 8-byte loads.
inline void interleave_cpml(float* t, int tp) {
    for (int i = 0; i < tp; i++)
        for (int k = 0; k < 6; k++) t[6 * tp + 6 * i + k] = t[k * tp + i];
}
__device__ __forceinline__ Cpml load_cpml6(const float* __restrict__ c, int tp, int p) {
    const float2* q = reinterpret_cast<const float2*>(c + 6 * tp) + 3 * p;
    const float2 u = __ldg(q), v = __ldg(q + 1), w = __ldg(q + 2);
    Cpml r;
    r.a = u.x;
    r.b = u.y;
    r.iK = v.x;
    r.ah = v.y;
    r.bh = w.x;
    r.iKh = w.y;
    return r;
}

// Stress pass over one tile (forward or adjoint; the reference uses the same
// operator for both).  One thread per column marches down the rows.  All
// descriptor fields are copied into registers first; the per-row loads that
// go to L2/HBM (the next row of the z-window, materials, stresses and, for the
// adjoint, ux/uz, the forward wavefield and the gradients) are issued kPF rows
// ahead and held in small register queues, so kPF+1 rows of loads are in
// flight per thread.  x-taps read lines the z-window brought into L1.
template <int FP, bool ADJ>
__device__ __forceinline__ void stress_tile(const ItemDesc& D, const Tile t, int it, unsigned flags) {
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    const int ix = t.x0 + (int)threadIdx.x;
    if (ix < FP || ix >= nxt - FP) return;
    const int zb = max(t.z0, FP), ze = min(t.z1, nzt - FP);
    if (zb >= ze) return;

    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const float dt = D.dt, inv_dt = D.inv_dt, gs = D.gscale;
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    const float* __restrict__ vx = D.vx;
    const float* __restrict__ vz = D.vz;
    const float* __restrict__ Lp = D.L;
    const float* __restrict__ M2p = D.M2;
    const float* __restrict__ MZp = D.MZX;
    float* __restrict__ sxxp = D.sxx;
    float* __restrict__ szxp = D.szx;
    float* __restrict__ szzp = D.szz;
    float* __restrict__ mvx_x = D.mvx_x;
    float* __restrict__ mvz_x = D.mvz_x;
    float* __restrict__ mvx_z = D.mvx_z;
    float* __restrict__ mvz_z = D.mvz_z;

    // x-strip CPML index of this column (stress: left strip includes ix == ppad).
    int px = -1;
    if (npml > 0) {
        if (ix <= ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;  // shared identity slot (checked on the host)
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(cpml, tp, px);

    // FWI window (storage / gradient).
    int xf = -1;
    const int wz1 = D.wz1, wz2 = D.wz2, fdz = D.fwi_dz, nfx = D.nfx;
    if (flags & (FL_STORE | FL_GRAD)) {
        if (ix >= D.wx1 && ix < D.wx2 && (ix - D.wx1) % D.fwi_dx == 0) xf = (ix - D.wx1) / D.fwi_dx;
    }
    const size_t fs = (size_t)D.nfz * nfx;
    const int tf = it / D.fwi_dt;
    float* __restrict__ store = (D.store && xf >= 0) ? D.store + (size_t)tf * 5 * fs + xf : nullptr;
    const bool grad = ADJ && (flags & FL_GRAD) && xf >= 0 && D.fwd;
    const bool grad_state = grad && D.fwd_kind == 1;  // forward fields from the forward state rows
    const float* __restrict__ fwd_st = (grad && !grad_state) ? D.fwd + (size_t)tf * 5 * fs + xf : nullptr;
    const float* __restrict__ fwd_rows = grad_state ? D.fwd + ix : nullptr;
    const size_t ffs = (size_t)D.fwd_fs;
    float* __restrict__ uxp = ADJ ? D.ux : nullptr;
    float* __restrict__ uzp = ADJ ? D.uz : nullptr;
    float* __restrict__ glam = grad ? D.glam + xf : nullptr;
    float* __restrict__ gmu = grad ? D.gmu + xf : nullptr;
    float* __restrict__ grho = grad ? D.grho + xf : nullptr;
    auto is_sample = [&](int z) { return xf >= 0 && z >= wz1 && z < wz2 && (z - wz1) % fdz == 0; };

    // Register windows: wvx holds vx rows iz-FP+1 .. iz+FP, wvz holds vz rows iz-FP .. iz+FP-1.
    float wvx[2 * FP], wvz[2 * FP];
#pragma unroll
    for (int r = 0; r < 2 * FP - 1; r++) {
        wvx[r] = __ldg(vx + (size_t)(zb - FP + 1 + r) * P + ix);
        wvz[r] = __ldg(vz + (size_t)(zb - FP + r) * P + ix);
    }
    // Prefetch queues: slot j holds the loads of row iz + j.
    constexpr int NQ = kPF + 1;
    float qwx[NQ], qwz[NQ], qL[NQ], qM2[NQ], qMZ[NQ], qsxx[NQ], qszx[NQ], qszz[NQ];
    float qux[NQ], quz[NQ], qf[5][NQ], qg[3][NQ];
    auto fetch = [&](int j, int z) {
        const int zc = min(z, ze - 1);  // rows past the tile are never used; stay in bounds
        const size_t c = (size_t)zc * P + ix;
        qwx[j] = __ldg(vx + (size_t)(zc + FP) * P + ix);
        qwz[j] = __ldg(vz + (size_t)(zc + FP - 1) * P + ix);
        qL[j] = __ldg(Lp + c);
        qM2[j] = __ldg(M2p + c);
        qMZ[j] = __ldg(MZp + c);
        qsxx[j] = sxxp[c];
        qszx[j] = szxp[c];
        qszz[j] = szzp[c];
        if (ADJ) {
            qux[j] = uxp[c];
            quz[j] = uzp[c];
            if (grad_state) {
#pragma unroll
                for (int f = 0; f < 5; f++) qf[f][j] = fwd_rows[(size_t)zc * P + f * ffs];
            }
            if (grad && z < ze && is_sample(z)) {
                const size_t g = (size_t)((z - wz1) / fdz) * nfx;
                qg[0][j] = glam[g];
                qg[1][j] = gmu[g];
                qg[2][j] = grho[g];
            }
        }
    };
#pragma unroll
    for (int j = 0; j < kPF; j++) fetch(j, zb + j);

    for (int iz = zb; iz < ze; iz++) {
        fetch(kPF, iz + kPF);
        wvx[2 * FP - 1] = qwx[0];
        wvz[2 * FP - 1] = qwz[0];
        const size_t c = (size_t)iz * P + ix;
        const float* vxr = vx + c;
        const float* vzr = vz + c;
        float vx_x = 0.f, vz_x = 0.f, vx_z = 0.f, vz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            const float xa = k == 1 ? wvx[FP - 1] : __ldg(vxr + k - 1);
            vx_x += hx[k - 1] * (xa - __ldg(vxr - k));
            const float za = k == 1 ? wvz[FP] : __ldg(vzr - k + 1);
            vz_x += hx[k - 1] * (__ldg(vzr + k) - za);
            vx_z += hz[k - 1] * (wvx[FP - 1 + k] - wvx[FP - k]);
            vz_z += hz[k - 1] * (wvz[FP + k - 1] - wvz[FP - k]);
        }
        const float L = qL[0], M2 = qM2[0], MZ = qMZ[0];
        float sxx = qsxx[0], szx = qszx[0], szz = qszz[0];
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * mvx_x[m] + cx.a * vx_x;
            const float m2 = cx.bh * mvz_x[m] + cx.ah * vz_x;
            mvx_x[m] = m1;
            mvz_x[m] = m2;
            vx_x = vx_x * cx.iK + m1;
            vz_x = vz_x * cx.iKh + m2;
        }
        if (npml > 0) {
            int pz = -1;
            if (!fsurf && iz <= ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz >= 0 && pz != npml) {
                const Cpml cz = load_cpml(cpml, tp, pz);
                const size_t m = (size_t)pz * P + ix;
                const float m1 = cz.b * mvz_z[m] + cz.a * vz_z;
                const float m2 = cz.bh * mvx_z[m] + cz.ah * vx_z;
                mvz_z[m] = m1;
                mvx_z[m] = m2;
                vz_z = vz_z * cz.iK + m1;
                vx_z = vx_z * cz.iKh + m2;
            }
        }
        const float vxc = wvx[FP - 1], vzc = wvz[FP];
        const bool sample = is_sample(iz);
        if (!ADJ && (flags & FL_STORE) && sample && store) {
            float* s = store + (size_t)((iz - wz1) / fdz) * nfx;
            s[F_VX * fs] = vxc / dt;
            s[F_VZ * fs] = vzc / dt;
            s[F_SXX * fs] = sxx;
            s[F_SZX * fs] = szx;
            s[F_SZZ * fs] = szz;
        }
        if (ADJ) {
            const float ux = qux[0] + dt * vxc;
            const float uz = quz[0] + dt * vzc;
            uxp[c] = ux;
            uzp[c] = uz;
            if (grad && sample) {
                const size_t g = (size_t)((iz - wz1) / fdz) * nfx;
                float fvx, fvz, fsxx, fszx, fszz;
                if (grad_state) {
                    fvx = qf[F_VX][0] / dt;
                    fvz = qf[F_VZ][0] / dt;
                    fsxx = qf[F_SXX][0];
                    fszx = qf[F_SZX][0];
                    fszz = qf[F_SZZ][0];
                } else {
                    const float* s = fwd_st + g;
                    fvx = s[F_VX * fs];
                    fvz = s[F_VZ * fs];
                    fsxx = s[F_SXX * fs];
                    fszx = s[F_SZX * fs];
                    fszz = s[F_SZZ * fs];
                }
                // lam + mu and mu recovered from the dt-scaled materials.
                const float lpm = (L + 0.5f * M2) * inv_dt;
                const float mu = 0.5f * M2 * inv_dt;
                const float s1 = (fsxx + fszz) * (sxx + szz) * 0.25f / (lpm * lpm);
                const float s2 = (fsxx - fszz) * (sxx - szz) / (mu * mu);
                const float s3 = (fszx * szx) / (mu * mu);
                const float s4 = ux * fvx + uz * fvz;
                glam[g] = qg[0][0] + gs * s1;
                gmu[g] = qg[1][0] + gs * (s3 + s1 + s2);
                grho[g] = qg[2][0] - gs * s4;
            }
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
        sxxp[c] = sxx;
        szxp[c] = szx;
        szzp[c] = szz;
        if (fsurf && iz > FP && iz <= 2 * FP) {  // stress mirroring above the free surface
            const size_t cm = (size_t)(2 * FP - iz) * P + ix;
            szxp[cm] = -szx;
            szzp[cm] = -szz;
        }
#pragma unroll
        for (int r = 0; r < 2 * FP - 1; r++) {
            wvx[r] = wvx[r + 1];
            wvz[r] = wvz[r + 1];
        }
#pragma unroll
        for (int j = 0; j < kPF; j++) {
            qwx[j] = qwx[j + 1]; qwz[j] = qwz[j + 1];
            qL[j] = qL[j + 1]; qM2[j] = qM2[j + 1]; qMZ[j] = qMZ[j + 1];
            qsxx[j] = qsxx[j + 1]; qszx[j] = qszx[j + 1]; qszz[j] = qszz[j + 1];
            if (ADJ) {
                qux[j] = qux[j + 1]; quz[j] = quz[j + 1];
#pragma unroll
                for (int f = 0; f < 5; f++) qf[f][j] = qf[f][j + 1];
#pragma unroll
                for (int f = 0; f < 3; f++) qg[f][j] = qg[f][j + 1];
            }
        }
    }
}

// Velocity pass over one tile + energy + source injection / receiver recording,
// with the same kPF-row register prefetch.
template <int FP>
__device__ __forceinline__ void velocity_tile(const ItemDesc& D, const Tile t, int it, unsigned flags) {
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    const int ix = t.x0 + (int)threadIdx.x;
    if (ix < FP || ix >= nxt - FP) return;
    const int zb = max(t.z0, FP), ze = min(t.z1, nzt - FP);
    if (zb >= ze) return;

    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz, nt = D.nt;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    const float* __restrict__ sxxp = D.sxx;
    const float* __restrict__ szxp = D.szx;
    const float* __restrict__ szzp = D.szz;
    const float* __restrict__ BXp = D.BX;
    const float* __restrict__ BZp = D.BZ;
    float* __restrict__ vxp = D.vx;
    float* __restrict__ vzp = D.vz;
    float* __restrict__ Wep = D.We;
    float* __restrict__ msxx_x = D.msxx_x;
    float* __restrict__ mszx_x = D.mszx_x;
    float* __restrict__ mszz_z = D.mszz_z;
    float* __restrict__ mszx_z = D.mszx_z;
    const int2* __restrict__ ev = D.ev;
    const float* __restrict__ inj = D.inj;
    float* __restrict__ rec = D.rec;

    // velocity: left strip is ix < ppad.
    int px = -1;
    if (npml > 0) {
        if (ix < ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(cpml, tp, px);

    // events of this column from row zb on (sorted by z)
    int e = 0, ee = 0, ez = 0x7fffffff;
    if (flags & (FL_INJECT | FL_RECORD)) {
        e = D.ev_col[ix];
        ee = D.ev_col[ix + 1];
        while (e < ee && ev[e].x < zb) e++;
        if (e < ee) ez = ev[e].x;
    }
    const bool we = (flags & FL_WE) != 0;

    // wsx: szx rows iz-FP .. iz+FP-1 ; wsz: szz rows iz-FP+1 .. iz+FP
    float wsx[2 * FP], wsz[2 * FP];
#pragma unroll
    for (int r = 0; r < 2 * FP - 1; r++) {
        wsx[r] = __ldg(szxp + (size_t)(zb - FP + r) * P + ix);
        wsz[r] = __ldg(szzp + (size_t)(zb - FP + 1 + r) * P + ix);
    }
    constexpr int NQ = kPF + 1;
    float qwx[NQ], qwz[NQ], qsxx[NQ], qbx[NQ], qbz[NQ], qvx[NQ], qvz[NQ], qwe[NQ];
    auto fetch = [&](int j, int z) {
        const int zc = min(z, ze - 1);
        const size_t c = (size_t)zc * P + ix;
        qwx[j] = __ldg(szxp + (size_t)(zc + FP - 1) * P + ix);
        qwz[j] = __ldg(szzp + (size_t)(zc + FP) * P + ix);
        qsxx[j] = __ldg(sxxp + c);  // also brings the x-taps' line into L1
        qbx[j] = __ldg(BXp + c);
        qbz[j] = __ldg(BZp + c);
        qvx[j] = vxp[c];
        qvz[j] = vzp[c];
        if (we) qwe[j] = Wep[c];
    };
#pragma unroll
    for (int j = 0; j < kPF; j++) fetch(j, zb + j);

    for (int iz = zb; iz < ze; iz++) {
        fetch(kPF, iz + kPF);
        wsx[2 * FP - 1] = qwx[0];
        wsz[2 * FP - 1] = qwz[0];
        const size_t c = (size_t)iz * P + ix;
        const float* sxr = sxxp + c;
        const float* szr = szxp + c;
        float sxx_x = 0.f, szx_x = 0.f, szx_z = 0.f, szz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            const float xa = k == 1 ? qsxx[0] : __ldg(sxr - k + 1);
            sxx_x += hx[k - 1] * (__ldg(sxr + k) - xa);
            const float za = k == 1 ? wsx[FP] : __ldg(szr + k - 1);
            szx_x += hx[k - 1] * (za - __ldg(szr - k));
            szx_z += hz[k - 1] * (wsx[FP + k - 1] - wsx[FP - k]);
            szz_z += hz[k - 1] * (wsz[FP - 1 + k] - wsz[FP - k]);
        }
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * msxx_x[m] + cx.a * sxx_x;
            const float m2 = cx.bh * mszx_x[m] + cx.ah * szx_x;
            msxx_x[m] = m1;
            mszx_x[m] = m2;
            sxx_x = sxx_x * cx.iK + m1;
            szx_x = szx_x * cx.iKh + m2;
        }
        if (npml > 0) {
            int pz = -1;
            if (!fsurf && iz < ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz >= 0 && pz != npml) {
                const Cpml cz = load_cpml(cpml, tp, pz);
                const size_t m = (size_t)pz * P + ix;
                const float m1 = cz.b * mszz_z[m] + cz.a * szz_z;
                const float m2 = cz.bh * mszx_z[m] + cz.ah * szx_z;
                mszz_z[m] = m1;
                mszx_z[m] = m2;
                szz_z = szz_z * cz.iK + m1;
                szx_z = szx_z * cz.iKh + m2;
            }
        }
        float vxn = qvx[0] + qbx[0] * (sxx_x + szx_z);
        float vzn = qvz[0] + qbz[0] * (szx_x + szz_z);
        if (we) Wep[c] = qwe[0] + (vxn * vxn + vzn * vzn);
        while (iz == ez) {
            const int code = ev[e].y;
            if (code >= 0) {
                if (flags & FL_INJECT) vzn += __ldg(inj + (size_t)code * nt + it);
            } else if (flags & FL_RECORD) {
                rec[(size_t)(~code) * nt + it] = vzn;
            }
            e++;
            ez = (e < ee) ? ev[e].x : 0x7fffffff;
        }
        vxp[c] = vxn;
        vzp[c] = vzn;
#pragma unroll
        for (int r = 0; r < 2 * FP - 1; r++) {
            wsx[r] = wsx[r + 1];
            wsz[r] = wsz[r + 1];
        }
#pragma unroll
        for (int j = 0; j < kPF; j++) {
            qwx[j] = qwx[j + 1]; qwz[j] = qwz[j + 1]; qsxx[j] = qsxx[j + 1];
            qbx[j] = qbx[j + 1]; qbz[j] = qbz[j + 1]; qvx[j] = qvx[j + 1]; qvz[j] = qvz[j + 1];
            qwe[j] = qwe[j + 1];
        }
    }
}

// ---------------------------------------------------------------------------
// Cell-parallel mapping.  A block of kTileX x kCellY threads covers a tile of
// kTileX columns and any number of rows; each thread computes the cells of
// one column, rows kCellY apart.  Every tap is an independent load (the
// z-taps of neighbouring rows hit L1/L2), so many warps hide the latency that
// limits a thread-serial z-march.
// ---------------------------------------------------------------------------
#ifndef FWI_CELL_Y
#define FWI_CELL_Y 4
#endif
#ifndef FWI_CELL_R
#define FWI_CELL_R 1
#endif
#ifndef FWI_CELL_MINB
#define FWI_CELL_MINB 2
#endif
constexpr int kCellY = FWI_CELL_Y;
constexpr int kCellR = FWI_CELL_R;
constexpr int kCellRows = kCellY * kCellR;

template <int FP, bool ADJ>
__device__ __forceinline__ void stress_cells(const ItemDesc& D, const Tile t, int it, unsigned flags) {
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    const int ix = t.x0 + (int)threadIdx.x;
    if (ix < FP || ix >= nxt - FP) return;
    const int zb = max(t.z0, FP), ze = min(t.z1, nzt - FP);
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const float dt = D.dt, inv_dt = D.inv_dt, gs = D.gscale;
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    const float* __restrict__ vx = D.vx;
    const float* __restrict__ vz = D.vz;
    int px = -1;
    if (npml > 0) {
        if (ix <= ppad) px = ix - FP;  // stress: the left strip includes ix == ppad
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;  // shared identity slot (checked on the host)
    }
    int xf = -1;
    const int wz1 = D.wz1, wz2 = D.wz2, fdz = D.fwi_dz, nfx = D.nfx;
    if (flags & (FL_STORE | FL_GRAD)) {
        if (ix >= D.wx1 && ix < D.wx2 && (ix - D.wx1) % D.fwi_dx == 0) xf = (ix - D.wx1) / D.fwi_dx;
    }
    const size_t fs = (size_t)D.nfz * nfx;
    const int tf = it / D.fwi_dt;
    for (int iz = zb + (int)threadIdx.y; iz < ze; iz += kCellY) {
        const size_t c = (size_t)iz * P + ix;
        const float* vxr = vx + c;
        const float* vzr = vz + c;
        float vx_x = 0.f, vz_x = 0.f, vx_z = 0.f, vz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_x += hx[k - 1] * (__ldg(vxr + k - 1) - __ldg(vxr - k));
            vz_x += hx[k - 1] * (__ldg(vzr + k) - __ldg(vzr - k + 1));
            vx_z += hz[k - 1] * (__ldg(vxr + (size_t)k * P) - __ldg(vxr - (ptrdiff_t)(k - 1) * P));
            vz_z += hz[k - 1] * (__ldg(vzr + (ptrdiff_t)(k - 1) * P) - __ldg(vzr - (ptrdiff_t)k * P));
        }
        const float L = __ldg(D.L + c), M2 = __ldg(D.M2 + c), MZ = __ldg(D.MZX + c);
        float sxx = D.sxx[c], szx = D.szx[c], szz = D.szz[c];
        if (px >= 0) {
            const Cpml cx = load_cpml(cpml, tp, px);
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * D.mvx_x[m] + cx.a * vx_x;
            const float m2 = cx.bh * D.mvz_x[m] + cx.ah * vz_x;
            D.mvx_x[m] = m1;
            D.mvz_x[m] = m2;
            vx_x = vx_x * cx.iK + m1;
            vz_x = vz_x * cx.iKh + m2;
        }
        if (npml > 0) {
            int pz = -1;
            if (!fsurf && iz <= ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz >= 0 && pz != npml) {
                const Cpml cz = load_cpml(cpml, tp, pz);
                const size_t m = (size_t)pz * P + ix;
                const float m1 = cz.b * D.mvz_z[m] + cz.a * vz_z;
                const float m2 = cz.bh * D.mvx_z[m] + cz.ah * vx_z;
                D.mvz_z[m] = m1;
                D.mvx_z[m] = m2;
                vz_z = vz_z * cz.iK + m1;
                vx_z = vx_z * cz.iKh + m2;
            }
        }
        const float vxc = __ldg(vxr), vzc = __ldg(vzr);
        const bool sample = xf >= 0 && iz >= wz1 && iz < wz2 && (iz - wz1) % fdz == 0;
        if (!ADJ && (flags & FL_STORE) && sample && D.store) {
            float* sp = D.store + (size_t)tf * 5 * fs + (size_t)((iz - wz1) / fdz) * nfx + xf;
            sp[F_VX * fs] = vxc / dt;
            sp[F_VZ * fs] = vzc / dt;
            sp[F_SXX * fs] = sxx;
            sp[F_SZX * fs] = szx;
            sp[F_SZZ * fs] = szz;
        }
        if (ADJ) {
            const float ux = D.ux[c] + dt * vxc;
            const float uz = D.uz[c] + dt * vzc;
            D.ux[c] = ux;
            D.uz[c] = uz;
            if ((flags & FL_GRAD) && sample && D.fwd) {
                const size_t g = (size_t)((iz - wz1) / fdz) * nfx + xf;
                float fvx, fvz, fsxx, fszx, fszz;
                if (D.fwd_kind == 0) {
                    const float* sp = D.fwd + (size_t)tf * 5 * fs + g;
                    fvx = sp[F_VX * fs];
                    fvz = sp[F_VZ * fs];
                    fsxx = sp[F_SXX * fs];
                    fszx = sp[F_SZX * fs];
                    fszz = sp[F_SZZ * fs];
                } else {
                    const float* sp = D.fwd + c;
                    const size_t ffs = (size_t)D.fwd_fs;
                    fvx = sp[F_VX * ffs] / dt;
                    fvz = sp[F_VZ * ffs] / dt;
                    fsxx = sp[F_SXX * ffs];
                    fszx = sp[F_SZX * ffs];
                    fszz = sp[F_SZZ * ffs];
                }
                // lam + mu and mu recovered from the dt-scaled materials.
                const float lpm = (L + 0.5f * M2) * inv_dt;
                const float mu = 0.5f * M2 * inv_dt;
                const float s1 = (fsxx + fszz) * (sxx + szz) * 0.25f / (lpm * lpm);
                const float s2 = (fsxx - fszz) * (sxx - szz) / (mu * mu);
                const float s3 = (fszx * szx) / (mu * mu);
                const float s4 = ux * fvx + uz * fvz;
                D.glam[g] += gs * s1;
                D.gmu[g] += gs * (s3 + s1 + s2);
                D.grho[g] -= gs * s4;
            }
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
        D.sxx[c] = sxx;
        D.szx[c] = szx;
        D.szz[c] = szz;
        if (fsurf && iz > FP && iz <= 2 * FP) {  // stress mirroring above the free surface
            const size_t cm = (size_t)(2 * FP - iz) * P + ix;
            D.szx[cm] = -szx;
            D.szz[cm] = -szz;
        }
    }
}

template <int FP>
__device__ __forceinline__ void velocity_cells(const ItemDesc& D, const Tile t, int it, unsigned flags) {
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    const int ix = t.x0 + (int)threadIdx.x;
    if (ix < FP || ix >= nxt - FP) return;
    const int zb = max(t.z0, FP), ze = min(t.z1, nzt - FP);
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz, nt = D.nt;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    const float* __restrict__ sxxp = D.sxx;
    const float* __restrict__ szxp = D.szx;
    const float* __restrict__ szzp = D.szz;
    int px = -1;
    if (npml > 0) {
        if (ix < ppad) px = ix - FP;  // velocity: the left strip is ix < ppad
        else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
        if (px == npml) px = -1;
    }
    const bool we = (flags & FL_WE) != 0;
    int e0 = 0, e1 = 0;
    if (flags & (FL_INJECT | FL_RECORD)) {
        e0 = D.ev_col[ix];
        e1 = D.ev_col[ix + 1];
    }
    for (int iz = zb + (int)threadIdx.y; iz < ze; iz += kCellY) {
        const size_t c = (size_t)iz * P + ix;
        const float* sxr = sxxp + c;
        const float* szr = szxp + c;
        const float* zzr = szzp + c;
        float sxx_x = 0.f, szx_x = 0.f, szx_z = 0.f, szz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            sxx_x += hx[k - 1] * (__ldg(sxr + k) - __ldg(sxr - k + 1));
            szx_x += hx[k - 1] * (__ldg(szr + k - 1) - __ldg(szr - k));
            szx_z += hz[k - 1] * (__ldg(szr + (ptrdiff_t)(k - 1) * P) - __ldg(szr - (ptrdiff_t)k * P));
            szz_z += hz[k - 1] * (__ldg(zzr + (ptrdiff_t)k * P) - __ldg(zzr - (ptrdiff_t)(k - 1) * P));
        }
        if (px >= 0) {
            const Cpml cx = load_cpml(cpml, tp, px);
            const size_t m = (size_t)iz * tp + px;
            const float m1 = cx.b * D.msxx_x[m] + cx.a * sxx_x;
            const float m2 = cx.bh * D.mszx_x[m] + cx.ah * szx_x;
            D.msxx_x[m] = m1;
            D.mszx_x[m] = m2;
            sxx_x = sxx_x * cx.iK + m1;
            szx_x = szx_x * cx.iKh + m2;
        }
        if (npml > 0) {
            int pz = -1;
            if (!fsurf && iz < ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - pnz;
            if (pz >= 0 && pz != npml) {
                const Cpml cz = load_cpml(cpml, tp, pz);
                const size_t m = (size_t)pz * P + ix;
                const float m1 = cz.b * D.mszz_z[m] + cz.a * szz_z;
                const float m2 = cz.bh * D.mszx_z[m] + cz.ah * szx_z;
                D.mszz_z[m] = m1;
                D.mszx_z[m] = m2;
                szz_z = szz_z * cz.iK + m1;
                szx_z = szx_z * cz.iKh + m2;
            }
        }
        float vxn = D.vx[c] + __ldg(D.BX + c) * (sxx_x + szx_z);
        float vzn = D.vz[c] + __ldg(D.BZ + c) * (szx_x + szz_z);
        if (we) D.We[c] += vxn * vxn + vzn * vzn;
        for (int e = e0; e < e1; e++) {
            const int2 ev = D.ev[e];
            if (ev.x != iz) continue;
            if (ev.y >= 0) {
                if (flags & FL_INJECT) vzn += __ldg(D.inj + (size_t)ev.y * nt + it);
            } else if (flags & FL_RECORD) {
                D.rec[(size_t)(~ev.y) * nt + it] = vzn;
            }
        }
        D.vx[c] = vxn;
        D.vz[c] = vzn;
    }
}

// ---------------------------------------------------------------------------
// Vectorised cell mapping (fdorder <= 8).  A thread computes 4 adjacent
// columns of one row from aligned 16-byte loads: the x-taps of a field come
// from three float4 loads (left, centre, right: the neighbours' centres, so
// L1 hits), the z-taps from one float4 per row offset.  A block of 32 x kV4Y
// threads covers 128 columns x kV4Y rows.  Per 4 cells this issues ~26 vector
// loads instead of ~144 scalar ones.
// ---------------------------------------------------------------------------
#ifndef FWI_V4_Y
#define FWI_V4_Y 8
#endif
#ifndef FWI_V4_MINB
#define FWI_V4_MINB 2
#endif
constexpr int kV4Y = FWI_V4_Y;

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ld4rw(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float get(const float4& v, int j) {
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set(float4& v, int j, float a) {
    if (j == 0) v.x = a; else if (j == 1) v.y = a; else if (j == 2) v.z = a; else v.w = a;
}

// x-taps of a row: values of columns c-4 .. c+7 (index 4+j = column c+j).
struct Row12 {
    float v[12];
};
__device__ __forceinline__ Row12 load_row12(const float* rowp, int c, int nxt, bool readonly) {
    Row12 r;
    const float4 m = readonly ? ld4(rowp + c) : ld4rw(rowp + c);
    const float4 l = c >= 4 ? (readonly ? ld4(rowp + c - 4) : ld4rw(rowp + c - 4)) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 h = c + 4 < nxt ? (readonly ? ld4(rowp + c + 4) : ld4rw(rowp + c + 4)) : make_float4(0.f, 0.f, 0.f, 0.f);
    r.v[0] = l.x; r.v[1] = l.y; r.v[2] = l.z; r.v[3] = l.w;
    r.v[4] = m.x; r.v[5] = m.y; r.v[6] = m.z; r.v[7] = m.w;
    r.v[8] = h.x; r.v[9] = h.y; r.v[10] = h.z; r.v[11] = h.w;
    return r;
}

template <int FP, bool ADJ>
__device__ __forceinline__ void stress_v4(const ItemDesc& D, const Tile t, int it, unsigned flags) {
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    const int c = t.x0 + 4 * (int)threadIdx.x;  // first of this thread's 4 columns
    const int iz = t.z0 + (int)threadIdx.y;
    if (iz < FP || iz >= nzt - FP || iz >= t.z1 || c >= nxt - FP || c + 3 < FP) return;
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const float dt = D.dt;
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    const size_t rc = (size_t)iz * P;
    const float* __restrict__ vxrow = D.vx + rc;
    const float* __restrict__ vzrow = D.vz + rc;
    const Row12 X = load_row12(vxrow, c, nxt, true);
    const Row12 Z = load_row12(vzrow, c, nxt, true);
    // z-derivatives of the 4 columns, accumulated as each row arrives:
    // vx_z = sum_k hz (vx[iz+k] - vx[iz-k+1]), vz_z = sum_k hz (vz[iz+k-1] - vz[iz-k])
    float dvxz[4] = {0.f, 0.f, 0.f, 0.f}, dvzz[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 1; k <= FP; k++) {
        const float4 a = ld4(D.vx + (size_t)(iz + k) * P + c);
        const float4 b = k == 1 ? make_float4(X.v[4], X.v[5], X.v[6], X.v[7])
                                : ld4(D.vx + (size_t)(iz - k + 1) * P + c);
        const float4 e = k == 1 ? make_float4(Z.v[4], Z.v[5], Z.v[6], Z.v[7])
                                : ld4(D.vz + (size_t)(iz + k - 1) * P + c);
        const float4 f = ld4(D.vz + (size_t)(iz - k) * P + c);
        dvxz[0] += hz[k - 1] * (a.x - b.x); dvxz[1] += hz[k - 1] * (a.y - b.y);
        dvxz[2] += hz[k - 1] * (a.z - b.z); dvxz[3] += hz[k - 1] * (a.w - b.w);
        dvzz[0] += hz[k - 1] * (e.x - f.x); dvzz[1] += hz[k - 1] * (e.y - f.y);
        dvzz[2] += hz[k - 1] * (e.z - f.z); dvzz[3] += hz[k - 1] * (e.w - f.w);
    }
    const size_t cc = rc + c;
    const float4 L4 = ld4(D.L + cc), M24 = ld4(D.M2 + cc), MZ4 = ld4(D.MZX + cc);
    float4 sxx4 = ld4rw(D.sxx + cc), szx4 = ld4rw(D.szx + cc), szz4 = ld4rw(D.szz + cc);
    float4 ux4, uz4;
    if (ADJ) {
        ux4 = ld4rw(D.ux + cc);
        uz4 = ld4rw(D.uz + cc);
    }
    // z-strip CPML row of this thread (uniform over the 4 columns)
    int pz = -1;
    if (npml > 0) {
        if (!fsurf && iz <= ppad) pz = iz - FP;
        else if (iz >= nzt - ppad - 1) pz = iz - pnz;
        if (pz == npml) pz = -1;
    }
    float4 mvz4, mvx4;
    Cpml cz = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (pz >= 0) {
        cz = load_cpml(cpml, tp, pz);
        mvz4 = ld4rw(D.mvz_z + (size_t)pz * P + c);
        mvx4 = ld4rw(D.mvx_z + (size_t)pz * P + c);
    }
    const int wz1 = D.wz1, wz2 = D.wz2, fdz = D.fwi_dz, nfx = D.nfx;
    const bool row_sample = (flags & (FL_STORE | FL_GRAD)) && iz >= wz1 && iz < wz2 && (iz - wz1) % fdz == 0;
    const size_t fs = (size_t)D.nfz * nfx;
    const int tf = it / D.fwi_dt;
    float4 fw[5];
    const bool grad_state = ADJ && (flags & FL_GRAD) && row_sample && D.fwd && D.fwd_kind == 1;
    if (grad_state) {
#pragma unroll
        for (int f = 0; f < 5; f++) fw[f] = ld4(D.fwd + cc + (size_t)f * D.fwd_fs);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int ix = c + j;
        if (ix < FP || ix >= nxt - FP) continue;
        float vx_x = 0.f, vz_x = 0.f, vx_z = dvxz[j], vz_z = dvzz[j];
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_x += hx[k - 1] * (X.v[4 + j + k - 1] - X.v[4 + j - k]);
            vz_x += hx[k - 1] * (Z.v[4 + j + k] - Z.v[4 + j - k + 1]);
        }
        if (npml > 0) {
            int px = -1;
            if (ix <= ppad) px = ix - FP;  // stress: the left strip includes ix == ppad
            else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
            if (px >= 0 && px != npml) {
                const Cpml cx = load_cpml(cpml, tp, px);
                const size_t m = (size_t)iz * tp + px;
                const float m1 = cx.b * D.mvx_x[m] + cx.a * vx_x;
                const float m2 = cx.bh * D.mvz_x[m] + cx.ah * vz_x;
                D.mvx_x[m] = m1;
                D.mvz_x[m] = m2;
                vx_x = vx_x * cx.iK + m1;
                vz_x = vz_x * cx.iKh + m2;
            }
        }
        if (pz >= 0) {
            const float m1 = cz.b * get(mvz4, j) + cz.a * vz_z;
            const float m2 = cz.bh * get(mvx4, j) + cz.ah * vx_z;
            set(mvz4, j, m1);
            set(mvx4, j, m2);
            vz_z = vz_z * cz.iK + m1;
            vx_z = vx_z * cz.iKh + m2;
        }
        const float L = get(L4, j), M2 = get(M24, j), MZ = get(MZ4, j);
        float sxx = get(sxx4, j), szx = get(szx4, j), szz = get(szz4, j);
        const float vxc = X.v[4 + j], vzc = Z.v[4 + j];
        const bool sample = row_sample && ix >= D.wx1 && ix < D.wx2 && (ix - D.wx1) % D.fwi_dx == 0;
        const size_t g = sample ? (size_t)((iz - wz1) / fdz) * nfx + (ix - D.wx1) / D.fwi_dx : 0;
        if (!ADJ && (flags & FL_STORE) && sample && D.store) {
            float* sp = D.store + (size_t)tf * 5 * fs + g;
            sp[F_VX * fs] = vxc / dt;
            sp[F_VZ * fs] = vzc / dt;
            sp[F_SXX * fs] = sxx;
            sp[F_SZX * fs] = szx;
            sp[F_SZZ * fs] = szz;
        }
        if (ADJ) {
            const float ux = get(ux4, j) + dt * vxc;
            const float uz = get(uz4, j) + dt * vzc;
            set(ux4, j, ux);
            set(uz4, j, uz);
            if ((flags & FL_GRAD) && sample && D.fwd) {
                float fvx, fvz, fsxx, fszx, fszz;
                if (D.fwd_kind == 0) {
                    const float* sp = D.fwd + (size_t)tf * 5 * fs + g;
                    fvx = sp[F_VX * fs];
                    fvz = sp[F_VZ * fs];
                    fsxx = sp[F_SXX * fs];
                    fszx = sp[F_SZX * fs];
                    fszz = sp[F_SZZ * fs];
                } else {
                    fvx = get(fw[F_VX], j) / dt;
                    fvz = get(fw[F_VZ], j) / dt;
                    fsxx = get(fw[F_SXX], j);
                    fszx = get(fw[F_SZX], j);
                    fszz = get(fw[F_SZZ], j);
                }
                // lam + mu and mu recovered from the dt-scaled materials.
                const float lpm = (L + 0.5f * M2) * D.inv_dt;
                const float mu = 0.5f * M2 * D.inv_dt;
                const float s1 = (fsxx + fszz) * (sxx + szz) * 0.25f / (lpm * lpm);
                const float s2 = (fsxx - fszz) * (sxx - szz) / (mu * mu);
                const float s3 = (fszx * szx) / (mu * mu);
                const float s4 = ux * fvx + uz * fvz;
                const float gsc = D.gscale;
                D.glam[g] += gsc * s1;
                D.gmu[g] += gsc * (s3 + s1 + s2);
                D.grho[g] -= gsc * s4;
            }
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
        set(sxx4, j, sxx);
        set(szx4, j, szx);
        set(szz4, j, szz);
    }
    // write back: whole vectors when all 4 columns are interior, else per column
    const bool full = c >= FP && c + 3 < nxt - FP;
    if (full) {
        st4(D.sxx + cc, sxx4);
        st4(D.szx + cc, szx4);
        st4(D.szz + cc, szz4);
        if (ADJ) {
            st4(D.ux + cc, ux4);
            st4(D.uz + cc, uz4);
        }
        if (pz >= 0) {
            st4(D.mvz_z + (size_t)pz * P + c, mvz4);
            st4(D.mvx_z + (size_t)pz * P + c, mvx4);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ix = c + j;
            if (ix < FP || ix >= nxt - FP) continue;
            D.sxx[cc + j] = get(sxx4, j);
            D.szx[cc + j] = get(szx4, j);
            D.szz[cc + j] = get(szz4, j);
            if (ADJ) {
                D.ux[cc + j] = get(ux4, j);
                D.uz[cc + j] = get(uz4, j);
            }
            if (pz >= 0) {
                D.mvz_z[(size_t)pz * P + ix] = get(mvz4, j);
                D.mvx_z[(size_t)pz * P + ix] = get(mvx4, j);
            }
        }
    }
    if (fsurf && iz > FP && iz <= 2 * FP) {  // stress mirroring above the free surface
        const size_t cm = (size_t)(2 * FP - iz) * P;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ix = c + j;
            if (ix < FP || ix >= nxt - FP) continue;
            D.szx[cm + ix] = -get(szx4, j);
            D.szz[cm + ix] = -get(szz4, j);
        }
    }
}

template <int FP>
__device__ __forceinline__ void velocity_v4(const ItemDesc& D, const Tile t, int it, unsigned flags) {
    const int nxt = D.nxt, nzt = D.nzt, P = D.pitch;
    const int c = t.x0 + 4 * (int)threadIdx.x;
    const int iz = t.z0 + (int)threadIdx.y;
    if (iz < FP || iz >= nzt - FP || iz >= t.z1 || c >= nxt - FP || c + 3 < FP) return;
    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = D.hx[k];
        hz[k] = D.hz[k];
    }
    const int ppad = D.ppad, npml = D.npml, tp = D.tp, pnz = D.pnz, nt = D.nt;
    const bool fsurf = D.fsurf != 0;
    const float* __restrict__ cpml = D.cpml;
    const size_t rc = (size_t)iz * P;
    const Row12 SX = load_row12(D.sxx + rc, c, nxt, true);
    const Row12 SZ = load_row12(D.szx + rc, c, nxt, true);
    // szx_z = sum_k hz (szx[iz+k-1] - szx[iz-k]), szz_z = sum_k hz (szz[iz+k] - szz[iz-k+1])
    float dsxz[4] = {0.f, 0.f, 0.f, 0.f}, dszz[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 1; k <= FP; k++) {
        const float4 a = k == 1 ? make_float4(SZ.v[4], SZ.v[5], SZ.v[6], SZ.v[7])
                                : ld4(D.szx + (size_t)(iz + k - 1) * P + c);
        const float4 b = ld4(D.szx + (size_t)(iz - k) * P + c);
        const float4 e = ld4(D.szz + (size_t)(iz + k) * P + c);
        const float4 f = ld4(D.szz + (size_t)(iz - k + 1) * P + c);
        dsxz[0] += hz[k - 1] * (a.x - b.x); dsxz[1] += hz[k - 1] * (a.y - b.y);
        dsxz[2] += hz[k - 1] * (a.z - b.z); dsxz[3] += hz[k - 1] * (a.w - b.w);
        dszz[0] += hz[k - 1] * (e.x - f.x); dszz[1] += hz[k - 1] * (e.y - f.y);
        dszz[2] += hz[k - 1] * (e.z - f.z); dszz[3] += hz[k - 1] * (e.w - f.w);
    }
    const size_t cc = rc + c;
    const float4 BX4 = ld4(D.BX + cc), BZ4 = ld4(D.BZ + cc);
    float4 vx4 = ld4rw(D.vx + cc), vz4 = ld4rw(D.vz + cc);
    const bool we = (flags & FL_WE) != 0;
    float4 we4;
    if (we) we4 = ld4rw(D.We + cc);
    int pz = -1;
    if (npml > 0) {
        if (!fsurf && iz < ppad) pz = iz - FP;
        else if (iz >= nzt - ppad - 1) pz = iz - pnz;
        if (pz == npml) pz = -1;
    }
    float4 msz4, msx4;
    Cpml cz = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (pz >= 0) {
        cz = load_cpml(cpml, tp, pz);
        msz4 = ld4rw(D.mszz_z + (size_t)pz * P + c);
        msx4 = ld4rw(D.mszx_z + (size_t)pz * P + c);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int ix = c + j;
        if (ix < FP || ix >= nxt - FP) continue;
        float sxx_x = 0.f, szx_x = 0.f, szx_z = dsxz[j], szz_z = dszz[j];
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            sxx_x += hx[k - 1] * (SX.v[4 + j + k] - SX.v[4 + j - k + 1]);
            szx_x += hx[k - 1] * (SZ.v[4 + j + k - 1] - SZ.v[4 + j - k]);
        }
        if (npml > 0) {
            int px = -1;
            if (ix < ppad) px = ix - FP;  // velocity: the left strip is ix < ppad
            else if (ix >= nxt - ppad - 1) px = ix - D.pnx;
            if (px >= 0 && px != npml) {
                const Cpml cx = load_cpml(cpml, tp, px);
                const size_t m = (size_t)iz * tp + px;
                const float m1 = cx.b * D.msxx_x[m] + cx.a * sxx_x;
                const float m2 = cx.bh * D.mszx_x[m] + cx.ah * szx_x;
                D.msxx_x[m] = m1;
                D.mszx_x[m] = m2;
                sxx_x = sxx_x * cx.iK + m1;
                szx_x = szx_x * cx.iKh + m2;
            }
        }
        if (pz >= 0) {
            const float m1 = cz.b * get(msz4, j) + cz.a * szz_z;
            const float m2 = cz.bh * get(msx4, j) + cz.ah * szx_z;
            set(msz4, j, m1);
            set(msx4, j, m2);
            szz_z = szz_z * cz.iK + m1;
            szx_z = szx_z * cz.iKh + m2;
        }
        const float vxn = get(vx4, j) + get(BX4, j) * (sxx_x + szx_z);
        float vzn = get(vz4, j) + get(BZ4, j) * (szx_x + szz_z);
        if (we) set(we4, j, get(we4, j) + (vxn * vxn + vzn * vzn));
        if (flags & (FL_INJECT | FL_RECORD)) {
            const int e1 = D.ev_col[ix + 1];
            for (int e = D.ev_col[ix]; e < e1; e++) {
                const int2 ev = D.ev[e];
                if (ev.x != iz) continue;
                if (ev.y >= 0) {
                    if (flags & FL_INJECT) vzn += __ldg(D.inj + (size_t)ev.y * nt + it);
                } else if (flags & FL_RECORD) {
                    D.rec[(size_t)(~ev.y) * nt + it] = vzn;
                }
            }
        }
        set(vx4, j, vxn);
        set(vz4, j, vzn);
    }
    const bool full = c >= FP && c + 3 < nxt - FP;
    if (full) {
        st4(D.vx + cc, vx4);
        st4(D.vz + cc, vz4);
        if (we) st4(D.We + cc, we4);
        if (pz >= 0) {
            st4(D.mszz_z + (size_t)pz * P + c, msz4);
            st4(D.mszx_z + (size_t)pz * P + c, msx4);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ix = c + j;
            if (ix < FP || ix >= nxt - FP) continue;
            D.vx[cc + j] = get(vx4, j);
            D.vz[cc + j] = get(vz4, j);
            if (we) D.We[cc + j] = get(we4, j);
            if (pz >= 0) {
                D.mszz_z[(size_t)pz * P + ix] = get(msz4, j);
                D.mszx_z[(size_t)pz * P + ix] = get(msx4, j);
            }
        }
    }
}

// Launch entry points.  MAP 0: thread-serial z-march (blockDim kTileX x 1);
// MAP 1: cell-parallel (blockDim kTileX x kCellY); MAP 2: vectorised cells
// (blockDim 32 x kV4Y, fdorder <= 8).  Blocks walk the tile work-list with a
// grid stride (persistent grid, no partial last wave).  `err` is unused by
// these kernels (they hold no waits); kept for the launch ABI.
template <int MAP>
struct MapDims {
    static constexpr int x = MAP == 2 ? 32 : kTileX;
    static constexpr int y = MAP == 0 ? 1 : (MAP == 1 ? kCellY : kV4Y);
    static constexpr int minb = MAP == 0 ? 1 : (MAP == 1 ? FWI_CELL_MINB : FWI_V4_MINB);
    static constexpr int rows = kV4Y;  // tile height of the cell mappings
};

template <int FP, bool ADJ, int MAP>
__global__ void __launch_bounds__(MapDims<MAP>::x * MapDims<MAP>::y,
                                  (ADJ && MAP == 2) ? 1 : MapDims<MAP>::minb) stress_kernel(
    const ItemDesc* __restrict__ items, const Tile* __restrict__ tiles, int ntiles, int it,
    unsigned flags, int* err) {
    (void)err;
    for (int i = blockIdx.x; i < ntiles; i += gridDim.x) {
        const Tile t = tiles[i];
        if (MAP == 2) {
            if constexpr (FP <= 4) stress_v4<FP, ADJ>(items[t.item], t, it, flags);
        } else if (MAP == 1) {
            stress_cells<FP, ADJ>(items[t.item], t, it, flags);
        } else {
            stress_tile<FP, ADJ>(items[t.item], t, it, flags);
        }
    }
}

template <int FP, int MAP>
__global__ void __launch_bounds__(MapDims<MAP>::x * MapDims<MAP>::y, MapDims<MAP>::minb) velocity_kernel(
    const ItemDesc* __restrict__ items, const Tile* __restrict__ tiles, int ntiles, int it,
    unsigned flags, int* err) {
    (void)err;
    for (int i = blockIdx.x; i < ntiles; i += gridDim.x) {
        const Tile t = tiles[i];
        if (MAP == 2) {
            if constexpr (FP <= 4) velocity_v4<FP>(items[t.item], t, it, flags);
        } else if (MAP == 1) {
            velocity_cells<FP>(items[t.item], t, it, flags);
        } else {
            velocity_tile<FP>(items[t.item], t, it, flags);
        }
    }
}

}  // namespace fwi
