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

// Minimum resident blocks per SM requested from the register allocator.
#ifndef FWI_MIN_BLOCKS
#define FWI_MIN_BLOCKS 1
#endif

enum Field { F_VX = 0, F_VZ = 1, F_SXX = 2, F_SZX = 3, F_SZZ = 4 };

enum Flags : unsigned {
    FL_STORE = 1u << 0,   // forward: write the sampled window to storage (before the update)
    FL_GRAD = 1u << 1,    // adjoint: accumulate the gradient at this step
    FL_WE = 1u << 2,      // accumulate the energy sum We += vx^2 + vz^2
    FL_INJECT = 1u << 3,  // add the injection signal at source positions
    FL_RECORD = 1u << 4,  // record vz at receiver positions
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

// Stress pass over one tile (forward or adjoint; the reference uses the same
// operator for both).  Every descriptor field is copied into a register before
// the row loop so that no load in the loop depends on another load.
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
    float* __restrict__ store = D.store ? D.store + (size_t)tf * 5 * fs + xf : nullptr;
    const float* __restrict__ fwd = nullptr;
    const int fwd_kind = D.fwd_kind;
    const size_t ffs = fwd_kind == 0 ? fs : (size_t)D.fwd_fs;
    if (ADJ && D.fwd) fwd = fwd_kind == 0 ? D.fwd + (size_t)tf * 5 * fs + xf : D.fwd + ix;
    float* __restrict__ uxp = ADJ ? D.ux : nullptr;
    float* __restrict__ uzp = ADJ ? D.uz : nullptr;
    float* __restrict__ glam = ADJ ? D.glam + xf : nullptr;
    float* __restrict__ gmu = ADJ ? D.gmu + xf : nullptr;
    float* __restrict__ grho = ADJ ? D.grho + xf : nullptr;
    // next sampled row of the window at or below zb
    int zwin = 0x7fffffff;
    if (xf >= 0) {
        int z = max(zb, wz1);
        z = wz1 + ((z - wz1 + fdz - 1) / fdz) * fdz;
        if (z < wz2) zwin = z;
    }

    // Register windows: wvx holds vx rows iz-FP+1 .. iz+FP, wvz holds vz rows iz-FP .. iz+FP-1.
    float wvx[2 * FP], wvz[2 * FP];
#pragma unroll
    for (int r = 0; r < 2 * FP - 1; r++) {
        wvx[r] = __ldg(vx + (size_t)(zb - FP + 1 + r) * P + ix);
        wvz[r] = __ldg(vz + (size_t)(zb - FP + r) * P + ix);
    }

    for (int iz = zb; iz < ze; iz++) {
        wvx[2 * FP - 1] = __ldg(vx + (size_t)(iz + FP) * P + ix);
        wvz[2 * FP - 1] = __ldg(vz + (size_t)(iz + FP - 1) * P + ix);
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
        const float L = __ldg(Lp + c), M2 = __ldg(M2p + c), MZ = __ldg(MZp + c);
        float sxx = sxxp[c], szx = szxp[c], szz = szzp[c];
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
        const bool sample = iz == zwin;
        if (sample) zwin = (zwin + fdz < wz2) ? zwin + fdz : 0x7fffffff;
        if (!ADJ && (flags & FL_STORE) && sample) {
            float* s = store + (size_t)((iz - wz1) / fdz) * nfx;
            s[F_VX * fs] = vxc / dt;
            s[F_VZ * fs] = vzc / dt;
            s[F_SXX * fs] = sxx;
            s[F_SZX * fs] = szx;
            s[F_SZZ * fs] = szz;
        }
        if (ADJ) {
            const float ux = uxp[c] + dt * vxc;
            const float uz = uzp[c] + dt * vzc;
            uxp[c] = ux;
            uzp[c] = uz;
            if ((flags & FL_GRAD) && sample) {
                const size_t g = (size_t)((iz - wz1) / fdz) * nfx;
                float fvx, fvz, fsxx, fszx, fszz;
                if (fwd_kind == 0) {
                    const float* s = fwd + g;
                    fvx = s[F_VX * ffs];
                    fvz = s[F_VZ * ffs];
                    fsxx = s[F_SXX * ffs];
                    fszx = s[F_SZX * ffs];
                    fszz = s[F_SZZ * ffs];
                } else {
                    const float* s = fwd + (size_t)iz * P;
                    fvx = s[F_VX * ffs] / dt;
                    fvz = s[F_VZ * ffs] / dt;
                    fsxx = s[F_SXX * ffs];
                    fszx = s[F_SZX * ffs];
                    fszz = s[F_SZZ * ffs];
                }
                // lam + mu and mu recovered from the dt-scaled materials.
                const float lpm = (L + 0.5f * M2) * inv_dt;
                const float mu = 0.5f * M2 * inv_dt;
                const float s1 = (fsxx + fszz) * (sxx + szz) * 0.25f / (lpm * lpm);
                const float s2 = (fsxx - fszz) * (sxx - szz) / (mu * mu);
                const float s3 = (fszx * szx) / (mu * mu);
                const float s4 = ux * fvx + uz * fvz;
                glam[g] += gs * s1;
                gmu[g] += gs * (s3 + s1 + s2);
                grho[g] -= gs * s4;
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
    }
}

// Velocity pass over one tile + energy + source injection / receiver recording.
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
    for (int iz = zb; iz < ze; iz++) {
        wsx[2 * FP - 1] = __ldg(szxp + (size_t)(iz + FP - 1) * P + ix);
        wsz[2 * FP - 1] = __ldg(szzp + (size_t)(iz + FP) * P + ix);
        const size_t c = (size_t)iz * P + ix;
        const float* sxr = sxxp + c;
        const float* szr = szxp + c;
        float sxx_x = 0.f, szx_x = 0.f, szx_z = 0.f, szz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            sxx_x += hx[k - 1] * (__ldg(sxr + k) - __ldg(sxr - k + 1));
            const float za = k == 1 ? wsx[FP] : __ldg(szr + k - 1);
            szx_x += hx[k - 1] * (za - __ldg(szr - k));
            szx_z += hz[k - 1] * (wsx[FP + k - 1] - wsx[FP - k]);
            szz_z += hz[k - 1] * (wsz[FP - 1 + k] - wsz[FP - k]);
        }
        const float bxv = __ldg(BXp + c), bzv = __ldg(BZp + c);
        float vxn = vxp[c], vzn = vzp[c];
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
        vxn += bxv * (sxx_x + szx_z);
        vzn += bzv * (szx_x + szz_z);
        if (we) Wep[c] += vxn * vxn + vzn * vzn;
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
    }
}

// Persistent launches: each block walks the tile work-list with a grid stride,
// so a launch sized to the resident capacity has no partial last wave.
template <int FP, bool ADJ>
__global__ void __launch_bounds__(128, FWI_MIN_BLOCKS) stress_kernel(const ItemDesc* __restrict__ items,
                                                     const Tile* __restrict__ tiles, int ntiles,
                                                     int it, unsigned flags) {
    for (int i = blockIdx.x; i < ntiles; i += gridDim.x) {
        const Tile t = tiles[i];
        stress_tile<FP, ADJ>(items[t.item], t, it, flags);
    }
}

template <int FP>
__global__ void __launch_bounds__(128, FWI_MIN_BLOCKS) velocity_kernel(const ItemDesc* __restrict__ items,
                                                       const Tile* __restrict__ tiles, int ntiles,
                                                       int it, unsigned flags) {
    for (int i = blockIdx.x; i < ntiles; i += gridDim.x) {
        const Tile t = tiles[i];
        velocity_tile<FP>(items[t.item], t, it, flags);
    }
}

}  // namespace fwi
