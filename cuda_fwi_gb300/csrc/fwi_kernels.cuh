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

// Stress pass (forward or adjoint; the reference uses the same operator for both).
template <int FP, bool ADJ>
__global__ void __launch_bounds__(256) stress_kernel(const ItemDesc* __restrict__ items,
                                                     const Tile* __restrict__ tiles, int it,
                                                     unsigned flags) {
    const Tile t = tiles[blockIdx.x];
    const ItemDesc& d = items[t.item];
    const int nxt = d.nxt, nzt = d.nzt, P = d.pitch;
    const int ix = t.x0 + (int)threadIdx.x;
    if (ix < FP || ix >= nxt - FP) return;
    const int zb = max(t.z0, FP), ze = min(t.z1, nzt - FP);
    if (zb >= ze) return;

    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = d.hx[k];
        hz[k] = d.hz[k];
    }
    const float dt = d.dt;
    const int ppad = d.ppad, npml = d.npml, tp = d.tp;

    // x-strip CPML index of this column (stress: left strip includes ix == ppad).
    int px = -1;
    if (npml > 0) {
        if (ix <= ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - d.pnx;
        if (px == npml) px = -1;  // shared identity slot (checked on the host)
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(d.cpml, tp, px);

    // FWI window column (storage / gradient).
    int xf = -1;
    if (flags & (FL_STORE | FL_GRAD)) {
        if (ix >= d.wx1 && ix < d.wx2 && (ix - d.wx1) % d.fwi_dx == 0) xf = (ix - d.wx1) / d.fwi_dx;
    }
    const int tf = it / d.fwi_dt;

    const float* __restrict__ vx = d.vx;
    const float* __restrict__ vz = d.vz;

    // Register windows: wvx holds vx rows iz-FP+1 .. iz+FP, wvz holds vz rows iz-FP .. iz+FP-1.
    float wvx[2 * FP], wvz[2 * FP];
#pragma unroll
    for (int r = 0; r < 2 * FP - 1; r++) {
        wvx[r] = vx[(size_t)(zb - FP + 1 + r) * P + ix];
        wvz[r] = vz[(size_t)(zb - FP + r) * P + ix];
    }

    for (int iz = zb; iz < ze; iz++) {
        wvx[2 * FP - 1] = vx[(size_t)(iz + FP) * P + ix];
        wvz[2 * FP - 1] = vz[(size_t)(iz + FP - 1) * P + ix];
        const size_t c = (size_t)iz * P + ix;
        const float* vxr = vx + c;
        const float* vzr = vz + c;
        float vx_x = 0.f, vz_x = 0.f, vx_z = 0.f, vz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            vx_x += hx[k - 1] * (vxr[k - 1] - vxr[-k]);
            vz_x += hx[k - 1] * (vzr[k] - vzr[-k + 1]);
            vx_z += hz[k - 1] * (wvx[FP - 1 + k] - wvx[FP - k]);
            vz_z += hz[k - 1] * (wvz[FP + k - 1] - wvz[FP - k]);
        }
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            float m1 = cx.b * d.mvx_x[m] + cx.a * vx_x;
            float m2 = cx.bh * d.mvz_x[m] + cx.ah * vz_x;
            d.mvx_x[m] = m1;
            d.mvz_x[m] = m2;
            vx_x = vx_x * cx.iK + m1;
            vz_x = vz_x * cx.iKh + m2;
        }
        if (npml > 0) {
            int pz = -1;
            if (!d.fsurf && iz <= ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - d.pnz;
            if (pz >= 0 && pz != npml) {
                const Cpml cz = load_cpml(d.cpml, tp, pz);
                const size_t m = (size_t)pz * P + ix;
                float m1 = cz.b * d.mvz_z[m] + cz.a * vz_z;
                float m2 = cz.bh * d.mvx_z[m] + cz.ah * vx_z;
                d.mvz_z[m] = m1;
                d.mvx_z[m] = m2;
                vz_z = vz_z * cz.iK + m1;
                vx_z = vx_z * cz.iKh + m2;
            }
        }
        const float L = d.L[c], M2 = d.M2[c], MZ = d.MZX[c];
        float sxx = d.sxx[c], szx = d.szx[c], szz = d.szz[c];
        const float vxc = wvx[FP - 1], vzc = wvz[FP];

        const bool in_win = xf >= 0 && iz >= d.wz1 && iz < d.wz2 && (iz - d.wz1) % d.fwi_dz == 0;
        if (!ADJ && (flags & FL_STORE) && in_win) {
            const int zf = (iz - d.wz1) / d.fwi_dz;
            const size_t fs = (size_t)d.nfz * d.nfx;
            float* s = d.store + (size_t)tf * 5 * fs + (size_t)zf * d.nfx + xf;
            s[F_VX * fs] = vxc / dt;
            s[F_VZ * fs] = vzc / dt;
            s[F_SXX * fs] = sxx;
            s[F_SZX * fs] = szx;
            s[F_SZZ * fs] = szz;
        }
        if (ADJ) {
            const float ux = d.ux[c] + dt * vxc;
            const float uz = d.uz[c] + dt * vzc;
            d.ux[c] = ux;
            d.uz[c] = uz;
            if ((flags & FL_GRAD) && in_win) {
                const int zf = (iz - d.wz1) / d.fwi_dz;
                float fvx, fvz, fsxx, fszx, fszz;
                if (d.fwd_kind == 0) {
                    const size_t fs = (size_t)d.nfz * d.nfx;
                    const float* s = d.fwd + (size_t)tf * 5 * fs + (size_t)zf * d.nfx + xf;
                    fvx = s[F_VX * fs];
                    fvz = s[F_VZ * fs];
                    fsxx = s[F_SXX * fs];
                    fszx = s[F_SZX * fs];
                    fszz = s[F_SZZ * fs];
                } else {
                    const float* s = d.fwd + c;
                    fvx = s[F_VX * d.fwd_fs] / dt;
                    fvz = s[F_VZ * d.fwd_fs] / dt;
                    fsxx = s[F_SXX * d.fwd_fs];
                    fszx = s[F_SZX * d.fwd_fs];
                    fszz = s[F_SZZ * d.fwd_fs];
                }
                // lam + mu and mu recovered from the dt-scaled materials.
                const float lpm = (L + 0.5f * M2) * d.inv_dt;
                const float mu = 0.5f * M2 * d.inv_dt;
                const float s1 = (fsxx + fszz) * (sxx + szz) * 0.25f / (lpm * lpm);
                const float s2 = (fsxx - fszz) * (sxx - szz) / (mu * mu);
                const float s3 = (fszx * szx) / (mu * mu);
                const float s4 = ux * fvx + uz * fvz;
                const size_t g = (size_t)zf * d.nfx + xf;
                const float gs = d.gscale;
                d.glam[g] += gs * s1;
                d.gmu[g] += gs * (s3 + s1 + s2);
                d.grho[g] -= gs * s4;
            }
        }
        szx += MZ * (vz_x + vx_z);
        const float tr = L * (vx_x + vz_z);
        sxx += tr + M2 * vx_x;
        szz += tr + M2 * vz_z;
        if (d.fsurf && iz == FP) {
            szz = 0.f;
            szx = 0.f;
            sxx = vx_x * (2.f * M2 * (L + 0.5f * M2)) / (L + M2);
        }
        d.sxx[c] = sxx;
        d.szx[c] = szx;
        d.szz[c] = szz;
        if (d.fsurf && iz > FP && iz <= 2 * FP) {  // stress mirroring above the free surface
            const size_t cm = (size_t)(2 * FP - iz) * P + ix;
            d.szx[cm] = -szx;
            d.szz[cm] = -szz;
        }
#pragma unroll
        for (int r = 0; r < 2 * FP - 1; r++) {
            wvx[r] = wvx[r + 1];
            wvz[r] = wvz[r + 1];
        }
    }
}

// Velocity pass + energy + source injection / receiver recording.
template <int FP>
__global__ void __launch_bounds__(256) velocity_kernel(const ItemDesc* __restrict__ items,
                                                       const Tile* __restrict__ tiles, int it,
                                                       unsigned flags) {
    const Tile t = tiles[blockIdx.x];
    const ItemDesc& d = items[t.item];
    const int nxt = d.nxt, nzt = d.nzt, P = d.pitch;
    const int ix = t.x0 + (int)threadIdx.x;
    if (ix < FP || ix >= nxt - FP) return;
    const int zb = max(t.z0, FP), ze = min(t.z1, nzt - FP);
    if (zb >= ze) return;

    float hx[FP], hz[FP];
#pragma unroll
    for (int k = 0; k < FP; k++) {
        hx[k] = d.hx[k];
        hz[k] = d.hz[k];
    }
    const int ppad = d.ppad, npml = d.npml, tp = d.tp;

    // velocity: left strip is ix < ppad.
    int px = -1;
    if (npml > 0) {
        if (ix < ppad) px = ix - FP;
        else if (ix >= nxt - ppad - 1) px = ix - d.pnx;
        if (px == npml) px = -1;
    }
    Cpml cx = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (px >= 0) cx = load_cpml(d.cpml, tp, px);

    // events of this column from row zb on (sorted by z)
    int e = 0, ee = 0, ez = 0x7fffffff;
    if (flags & (FL_INJECT | FL_RECORD)) {
        e = d.ev_col[ix];
        ee = d.ev_col[ix + 1];
        while (e < ee && d.ev[e].x < zb) e++;
        if (e < ee) ez = d.ev[e].x;
    }
    const bool we = (flags & FL_WE) != 0;

    const float* __restrict__ szxp = d.szx;
    const float* __restrict__ szzp = d.szz;
    const float* __restrict__ sxxp = d.sxx;
    // wsx: szx rows iz-FP .. iz+FP-1 ; wsz: szz rows iz-FP+1 .. iz+FP
    float wsx[2 * FP], wsz[2 * FP];
#pragma unroll
    for (int r = 0; r < 2 * FP - 1; r++) {
        wsx[r] = szxp[(size_t)(zb - FP + r) * P + ix];
        wsz[r] = szzp[(size_t)(zb - FP + 1 + r) * P + ix];
    }
    for (int iz = zb; iz < ze; iz++) {
        wsx[2 * FP - 1] = szxp[(size_t)(iz + FP - 1) * P + ix];
        wsz[2 * FP - 1] = szzp[(size_t)(iz + FP) * P + ix];
        const size_t c = (size_t)iz * P + ix;
        const float* sxr = sxxp + c;
        const float* szr = szxp + c;
        float sxx_x = 0.f, szx_x = 0.f, szx_z = 0.f, szz_z = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            sxx_x += hx[k - 1] * (sxr[k] - sxr[-k + 1]);
            szx_x += hx[k - 1] * (szr[k - 1] - szr[-k]);
            szx_z += hz[k - 1] * (wsx[FP + k - 1] - wsx[FP - k]);
            szz_z += hz[k - 1] * (wsz[FP - 1 + k] - wsz[FP - k]);
        }
        if (px >= 0) {
            const size_t m = (size_t)iz * tp + px;
            float m1 = cx.b * d.msxx_x[m] + cx.a * sxx_x;
            float m2 = cx.bh * d.mszx_x[m] + cx.ah * szx_x;
            d.msxx_x[m] = m1;
            d.mszx_x[m] = m2;
            sxx_x = sxx_x * cx.iK + m1;
            szx_x = szx_x * cx.iKh + m2;
        }
        if (npml > 0) {
            int pz = -1;
            if (!d.fsurf && iz < ppad) pz = iz - FP;
            else if (iz >= nzt - ppad - 1) pz = iz - d.pnz;
            if (pz >= 0 && pz != npml) {
                const Cpml cz = load_cpml(d.cpml, tp, pz);
                const size_t m = (size_t)pz * P + ix;
                float m1 = cz.b * d.mszz_z[m] + cz.a * szz_z;
                float m2 = cz.bh * d.mszx_z[m] + cz.ah * szx_z;
                d.mszz_z[m] = m1;
                d.mszx_z[m] = m2;
                szz_z = szz_z * cz.iK + m1;
                szx_z = szx_z * cz.iKh + m2;
            }
        }
        float vxn = d.vx[c] + d.BX[c] * (sxx_x + szx_z);
        float vzn = d.vz[c] + d.BZ[c] * (szx_x + szz_z);
        if (we) d.We[c] += vxn * vxn + vzn * vzn;
        while (iz == ez) {
            const int code = d.ev[e].y;
            if (code >= 0) {
                if (flags & FL_INJECT) vzn += d.inj[(size_t)code * d.nt + it];
            } else if (flags & FL_RECORD) {
                d.rec[(size_t)(~code) * d.nt + it] = vzn;
            }
            e++;
            ez = (e < ee) ? d.ev[e].x : 0x7fffffff;
        }
        d.vx[c] = vxn;
        d.vz[c] = vzn;
#pragma unroll
        for (int r = 0; r < 2 * FP - 1; r++) {
            wsx[r] = wsx[r + 1];
            wsz[r] = wsz[r + 1];
        }
    }
}

}  // namespace fwi
