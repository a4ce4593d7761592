// fwi_exact.cuh -- discrete adjoint of the FP32 time stepping (FWI_GRAD_EXACT).
//
// The reference's gradient (CUDA_week2/adjoint_kernel_PSV_GPU.cu:830-863) runs
// the forward operator backwards in time and correlates fields: a
// continuous-adjoint approximation that does not match finite differences of
// the discrete misfit.  This file transposes the discrete scheme instead, so
// the result is dJ/dm of J = sum_n sum_r 0.5 dt (vz^{n+1}[r] - obs_n[r])^2.
//
// Forward step n (interior cells, as in fwi_kernels.cuh):
//   stress:   a_x = Dx- vx, b_x = Dx+ vz, a_z = Dz+ vx, b_z = Dz- vz
//             u' = u/K + psi', psi' = b psi + a u   (CPML on each derivative u)
//             sxx += L (a_x'+b_z') + M2 a_x';  szz += L (a_x'+b_z') + M2 b_z';
//             szx += MZ (b_x' + a_z')
//   velocity: c_x = Dx+ sxx, d_x = Dx- szx, d_z = Dz- szx, e_z = Dz+ szz (+ CPML)
//             vx += BX (c_x' + d_z');  vz += BZ (d_x' + e_z') [+ source]
// Reverse step n, given the adjoints of level n+1 (one kernel each):
//   1. vel_adj_local: vz^-[rec] += dt (d_n - obs_n); w1 = BX vx^-, w2 = BZ vz^-;
//      CPML transposes give the derivative adjoints G (4 fields); the
//      sensitivities R += vx^- dvx, T += vz^- (dvz - src) accumulate.
//   2. vel_adj_stencil: s^- += (D)^T G.
//   3. str_adj_local: stress derivative adjoints + CPML transposes -> H (4
//      fields); P += (sxx^- + szz^-)(dsxx + dszz), A += sxx^- dsxx + szz^- dszz,
//      Q += szx^- dszx.
//   4. str_adj_stencil: v^- += (D)^T H.
// Free surface (row fpad): the forward assigns sxx = c a_x' with
// c = M2 (2L + M2)/(L + M2) and zeroes szx, szz there, then mirrors szx, szz of
// rows fpad+1..2fpad onto rows fpad-1..0 with a minus sign.  The transpose
// zeroes the old stress adjoint on that row and folds the pad-row adjoints of
// the velocity z-stencils back onto the mirrored rows.
// The forward increments d* = field^{n+1} - field^n come from the forward
// states n and n+1 (binomial checkpointing at one-step granularity keeps them);
// the increment form needs mu > 0 (in a fluid cell the two normal-stress
// increments cannot be split into their lam and mu parts).
// With (D+)^T g(j) = sum_k h_k (g[j-k] - g[j+k-1]) and
//      (D-)^T g(j) = sum_k h_k (g[j-k+1] - g[j+k]), g = 0 off the interior.
// Finally chain_rule maps P, A, Q, R, T through the dt scaling and the
// staggered averages (fd_medium.cu:128-159) to lam, mu, rho on the window.
#pragma once

#include "fwi_kernels.cuh"

namespace fwi {

// Adjoint-only buffers of one shot, reached through ExactDesc.
struct ExactDesc {
    float* tmp;            // [4][field] G or H derivative adjoints
    float* acc;            // [5][field] P, A, Q, R, T
    const float* next;     // forward state n+1: [5][field] (vx, vz, sxx, szx, szz)
    const int* src_col;    // forward source events by column (inject codes only)
    const int2* src_ev;
    const float* src_sig;  // [nsrc][nt]
    long long field;       // floats per field
};

__device__ __forceinline__ bool cell_of(const ItemDesc& D, long long idx, int FPv, int* iz, int* ix) {
    const int nxi = D.nxt - 2 * FPv;
    const int nzi = D.nzt - 2 * FPv;
    if (idx >= (long long)nxi * nzi) return false;
    *iz = FPv + (int)(idx / nxi);
    *ix = FPv + (int)(idx % nxi);
    return true;
}

// x / z strip indices of the two passes (same rules as the forward kernels).
__device__ __forceinline__ int stress_px(const ItemDesc& D, int ix, int FPv) {
    if (D.npml <= 0) return -1;
    int px = -1;
    if (ix <= D.ppad) px = ix - FPv;
    else if (ix >= D.nxt - D.ppad - 1) px = ix - D.pnx;
    return px == D.npml ? -1 : px;
}
__device__ __forceinline__ int velocity_px(const ItemDesc& D, int ix, int FPv) {
    if (D.npml <= 0) return -1;
    int px = -1;
    if (ix < D.ppad) px = ix - FPv;
    else if (ix >= D.nxt - D.ppad - 1) px = ix - D.pnx;
    return px == D.npml ? -1 : px;
}
__device__ __forceinline__ int stress_pz(const ItemDesc& D, int iz, int FPv) {
    if (D.npml <= 0) return -1;
    int pz = -1;
    if (!D.fsurf && iz <= D.ppad) pz = iz - FPv;
    else if (iz >= D.nzt - D.ppad - 1) pz = iz - D.pnz;
    return pz == D.npml ? -1 : pz;
}
__device__ __forceinline__ int velocity_pz(const ItemDesc& D, int iz, int FPv) {
    if (D.npml <= 0) return -1;
    int pz = -1;
    if (!D.fsurf && iz < D.ppad) pz = iz - FPv;
    else if (iz >= D.nzt - D.ppad - 1) pz = iz - D.pnz;
    return pz == D.npml ? -1 : pz;
}

// CPML transpose: u' = u iK + psi', psi' = b psi + a u.  Given ubar' and the
// stored adjoint memory m (= b * psibar'' of the later step), returns ubar and
// updates m to b * (m + ubar').
__device__ __forceinline__ float cpml_adj(float ubar, float* m, float a, float b, float iK) {
    const float tot = *m + ubar;
    *m = b * tot;
    return ubar * iK + a * tot;
}

template <int FP>
__global__ void vel_adj_local(const ItemDesc* __restrict__ items, const ExactDesc* __restrict__ ex, int nb,
                              int it, long long cells) {
    const int b = blockIdx.y;
    if (b >= nb) return;
    const ItemDesc& D = items[b];
    const ExactDesc& E = ex[b];
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int iz, ix;
    if (idx >= cells || !cell_of(D, idx, FP, &iz, &ix)) return;
    const int P = D.pitch, tp = D.tp;
    const size_t c = (size_t)iz * P + ix;
    float vzb = D.vz[c];
    const float vxb = D.vx[c];
    // receivers record vz^{n+1} after the source: their adjoint source comes first
    const int e1 = D.ev_col[ix + 1];
    bool touched = false;
    for (int e = D.ev_col[ix]; e < e1; e++) {
        const int2 ev = D.ev[e];
        if (ev.x == iz && ev.y >= 0) {
            vzb += D.dt * D.inj[(size_t)ev.y * D.nt + it];
            touched = true;
        }
    }
    if (touched) D.vz[c] = vzb;
    // sensitivities to BX, BZ: adjoint times the forward increment (minus the source)
    const float* nx = E.next;
    const float* fw = D.fwd;  // forward state n
    const long long F = E.field;
    const float dvx = nx[F_VX * F + c] - fw[F_VX * F + c];
    float dvz = nx[F_VZ * F + c] - fw[F_VZ * F + c];
    const int s1 = E.src_col[ix + 1];
    for (int e = E.src_col[ix]; e < s1; e++) {
        const int2 ev = E.src_ev[e];
        if (ev.x == iz && ev.y >= 0) dvz -= E.src_sig[(size_t)ev.y * D.nt + it];
    }
    E.acc[3 * F + c] += vxb * dvx;
    E.acc[4 * F + c] += vzb * dvz;
    const float w1 = D.BX[c] * vxb, w2 = D.BZ[c] * vzb;
    // c_x (full, psi5 = msxx_x), d_x (half, psi6 = mszx_x) from w1 / w2; d_z (half, psi8), e_z (full, psi7)
    float gcx = w1, gdx = w2, gdz = w1, gez = w2;
    const float* cp = D.cpml;
    const int px = velocity_px(D, ix, FP);
    if (px >= 0) {
        const size_t m = (size_t)iz * tp + px;
        gcx = cpml_adj(w1, D.msxx_x + m, cp[px], cp[tp + px], cp[2 * tp + px]);
        gdx = cpml_adj(w2, D.mszx_x + m, cp[3 * tp + px], cp[4 * tp + px], cp[5 * tp + px]);
    }
    const int pz = velocity_pz(D, iz, FP);
    if (pz >= 0) {
        const size_t m = (size_t)pz * P + ix;
        gez = cpml_adj(w2, D.mszz_z + m, cp[pz], cp[tp + pz], cp[2 * tp + pz]);
        gdz = cpml_adj(w1, D.mszx_z + m, cp[3 * tp + pz], cp[4 * tp + pz], cp[5 * tp + pz]);
    }
    E.tmp[0 * F + c] = gcx;
    E.tmp[1 * F + c] = gdx;
    E.tmp[2 * F + c] = gdz;
    E.tmp[3 * F + c] = gez;
}

template <int FP>
__device__ __forceinline__ float tmp_at(const ItemDesc& D, const float* t, int iz, int ix) {
    // derivative adjoints live on interior cells only
    if (iz < FP || iz >= D.nzt - FP || ix < FP || ix >= D.nxt - FP) return 0.f;
    return t[(size_t)iz * D.pitch + ix];
}

template <int FP>
__global__ void vel_adj_stencil(const ItemDesc* __restrict__ items, const ExactDesc* __restrict__ ex,
                                int nb, long long cells) {
    const int b = blockIdx.y;
    if (b >= nb) return;
    const ItemDesc& D = items[b];
    const ExactDesc& E = ex[b];
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int iz, ix;
    if (idx >= cells || !cell_of(D, idx, FP, &iz, &ix)) return;
    const long long F = E.field;
    const float *gcx = E.tmp, *gdx = E.tmp + F, *gdz = E.tmp + 2 * F, *gez = E.tmp + 3 * F;
    float sxx = 0.f, szx = 0.f, szz = 0.f;
#pragma unroll
    for (int k = 1; k <= FP; k++) {
        const float hx = D.hx[k - 1], hz = D.hz[k - 1];
        sxx += hx * (tmp_at<FP>(D, gcx, iz, ix - k) - tmp_at<FP>(D, gcx, iz, ix + k - 1));       // (Dx+)^T
        szx += hx * (tmp_at<FP>(D, gdx, iz, ix - k + 1) - tmp_at<FP>(D, gdx, iz, ix + k));       // (Dx-)^T
        szx += hz * (tmp_at<FP>(D, gdz, iz - k + 1, ix) - tmp_at<FP>(D, gdz, iz + k, ix));       // (Dz-)^T
        szz += hz * (tmp_at<FP>(D, gez, iz - k, ix) - tmp_at<FP>(D, gez, iz + k - 1, ix));       // (Dz+)^T
    }
    if (D.fsurf && iz > FP && iz <= 2 * FP) {
        // rows fpad-1..0 hold -szx, -szz of rows fpad+1..2fpad: their adjoints
        // (z-stencil taps of the interior rows only) fold back with a minus sign
        const int r = 2 * FP - iz;
        float px = 0.f, pz = 0.f;
#pragma unroll
        for (int k = 1; k <= FP; k++) {
            const float hz = D.hz[k - 1];
            px += hz * (tmp_at<FP>(D, gdz, r - k + 1, ix) - tmp_at<FP>(D, gdz, r + k, ix));
            pz += hz * (tmp_at<FP>(D, gez, r - k, ix) - tmp_at<FP>(D, gez, r + k - 1, ix));
        }
        szx -= px;
        szz -= pz;
    }
    const size_t c = (size_t)iz * D.pitch + ix;
    D.sxx[c] += sxx;
    D.szx[c] += szx;
    D.szz[c] += szz;
}

template <int FP>
__global__ void str_adj_local(const ItemDesc* __restrict__ items, const ExactDesc* __restrict__ ex, int nb,
                              long long cells) {
    const int b = blockIdx.y;
    if (b >= nb) return;
    const ItemDesc& D = items[b];
    const ExactDesc& E = ex[b];
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int iz, ix;
    if (idx >= cells || !cell_of(D, idx, FP, &iz, &ix)) return;
    const int P = D.pitch, tp = D.tp;
    const size_t c = (size_t)iz * P + ix;
    const long long F = E.field;
    const float sxxb = D.sxx[c], szxb = D.szx[c], szzb = D.szz[c];
    const float* nx = E.next;
    const float* fw = D.fwd;
    const float L = D.L[c], M2 = D.M2[c], MZ = D.MZX[c];
    float ax, bz, bx, az;  // adjoints of a_x' (vx_x), b_z' (vz_z), b_x' (vz_x), a_z' (vx_z)
    if (D.fsurf && iz == FP) {
        // sxx^{n+1} = c a_x', c = M2 (2L + M2)/(L + M2): dJ/dL = X M2/((2L+M2)(L+M2)) and
        // dJ/dM2 = X/M2 - L X/((2L+M2)(L+M2)) with X = sxx_bar sxx^{n+1}, which the
        // interior formulas of chain_rule return for P = X M2/(L+M2), A = X.
        const float X = sxxb * nx[F_SXX * F + c];
        if (L + M2 != 0.f) E.acc[0 * F + c] += X * M2 / (L + M2);
        E.acc[1 * F + c] += X;
        ax = sxxb * ((2.f * M2 * (L + 0.5f * M2)) / (L + M2));
        bz = bx = az = 0.f;
        D.sxx[c] = 0.f;  // the old stress of this row is overwritten by the step
        D.szx[c] = 0.f;
        D.szz[c] = 0.f;
    } else {
        const float dxx = nx[F_SXX * F + c] - fw[F_SXX * F + c];
        const float dzx = nx[F_SZX * F + c] - fw[F_SZX * F + c];
        const float dzz = nx[F_SZZ * F + c] - fw[F_SZZ * F + c];
        E.acc[0 * F + c] += (sxxb + szzb) * (dxx + dzz);
        E.acc[1 * F + c] += sxxb * dxx + szzb * dzz;
        E.acc[2 * F + c] += szxb * dzx;
        ax = (L + M2) * sxxb + L * szzb;
        bz = L * sxxb + (L + M2) * szzb;
        bx = MZ * szxb;
        az = MZ * szxb;
    }
    float hax = ax, hbx = bx, haz = az, hbz = bz;
    const float* cp = D.cpml;
    const int px = stress_px(D, ix, FP);
    if (px >= 0) {
        const size_t m = (size_t)iz * tp + px;
        hax = cpml_adj(ax, D.mvx_x + m, cp[px], cp[tp + px], cp[2 * tp + px]);
        hbx = cpml_adj(bx, D.mvz_x + m, cp[3 * tp + px], cp[4 * tp + px], cp[5 * tp + px]);
    }
    const int pz = stress_pz(D, iz, FP);
    if (pz >= 0) {
        const size_t m = (size_t)pz * P + ix;
        hbz = cpml_adj(bz, D.mvz_z + m, cp[pz], cp[tp + pz], cp[2 * tp + pz]);
        haz = cpml_adj(az, D.mvx_z + m, cp[3 * tp + pz], cp[4 * tp + pz], cp[5 * tp + pz]);
    }
    E.tmp[0 * F + c] = hax;
    E.tmp[1 * F + c] = hbx;
    E.tmp[2 * F + c] = haz;
    E.tmp[3 * F + c] = hbz;
}

template <int FP>
__global__ void str_adj_stencil(const ItemDesc* __restrict__ items, const ExactDesc* __restrict__ ex,
                                int nb, long long cells) {
    const int b = blockIdx.y;
    if (b >= nb) return;
    const ItemDesc& D = items[b];
    const ExactDesc& E = ex[b];
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int iz, ix;
    if (idx >= cells || !cell_of(D, idx, FP, &iz, &ix)) return;
    const long long F = E.field;
    const float *hax = E.tmp, *hbx = E.tmp + F, *haz = E.tmp + 2 * F, *hbz = E.tmp + 3 * F;
    float vx = 0.f, vz = 0.f;
#pragma unroll
    for (int k = 1; k <= FP; k++) {
        const float hx = D.hx[k - 1], hz = D.hz[k - 1];
        vx += hx * (tmp_at<FP>(D, hax, iz, ix - k + 1) - tmp_at<FP>(D, hax, iz, ix + k));   // (Dx-)^T
        vx += hz * (tmp_at<FP>(D, haz, iz - k, ix) - tmp_at<FP>(D, haz, iz + k - 1, ix));   // (Dz+)^T
        vz += hx * (tmp_at<FP>(D, hbx, iz, ix - k) - tmp_at<FP>(D, hbx, iz, ix + k - 1));   // (Dx+)^T
        vz += hz * (tmp_at<FP>(D, hbz, iz - k + 1, ix) - tmp_at<FP>(D, hbz, iz + k, ix));   // (Dz-)^T
    }
    const size_t c = (size_t)iz * D.pitch + ix;
    D.vx[c] += vx;
    D.vz[c] += vz;
}

// Sensitivities to the dt-scaled materials -> gradients of lam, mu, rho on the
// raw grid, sampled on the FWI window ([nfz][nfx]):
//   dJ/dlam = dt P/(2L+M2)                               (L = dt lam, M2 = 2 dt mu)
//   dJ/dmu  = 2 dt (A - L P/(2L+M2))/M2 + sum over the 4 mu_zx cells using mu:
//             Q MZ / (4 dt mu^2)                        (mu_zx = 4/sum(1/mu))
//   dJ/drho = - sum over the 2 rho_xp cells R BX/(2 dt) - sum over the 2 rho_zp cells T BZ/(2 dt)
__global__ void chain_rule(const ItemDesc* __restrict__ items, const ExactDesc* __restrict__ ex, int nb) {
    const int b = blockIdx.y;
    if (b >= nb) return;
    const ItemDesc& D = items[b];
    const ExactDesc& E = ex[b];
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)D.nfz * D.nfx;
    if (idx >= n) return;
    const int zf = (int)(idx / D.nfx), xf = (int)(idx % D.nfx);
    const int iz = D.wz1 + zf * D.fwi_dz, ix = D.wx1 + xf * D.fwi_dx;
    float gl = 0.f, gm = 0.f, gr = 0.f;
    if (iz < D.wz2 && ix < D.wx2) {
        const int FPv = D.fpad, P = D.pitch;
        const long long F = E.field;
        const float dt = D.dt;
        auto interior = [&](int z, int x) {
            return z >= FPv && z < D.nzt - FPv && x >= FPv && x < D.nxt - FPv;
        };
        const size_t c = (size_t)iz * P + ix;
        const float L = D.L[c], M2 = D.M2[c];
        if (interior(iz, ix)) {
            const float Pv = E.acc[c], Av = E.acc[F + c];
            const float gL = (2.f * L + M2) != 0.f ? Pv / (2.f * L + M2) : 0.f;
            gl = dt * gL;
            if (M2 != 0.f) gm = 2.f * dt * (Av - L * gL) / M2;
        }
        const float mu = 0.5f * M2 / dt;
        const int dz[4] = {0, 0, -1, -1}, dx[4] = {0, -1, 0, -1};
        if (mu != 0.f)
            for (int q = 0; q < 4; q++) {
                const int z = iz + dz[q], x = ix + dx[q];
                if (z < 0 || x < 0 || !interior(z, x)) continue;
                const size_t cq = (size_t)z * P + x;
                const float MZ = D.MZX[cq];
                gm += E.acc[2 * F + cq] * MZ / (4.f * dt * mu * mu);
            }
        for (int q = 0; q < 2; q++) {
            const int x = ix - q;  // rho_xp[iz][x] averages rho[iz][x], rho[iz][x+1]
            if (x >= 0 && interior(iz, x)) {
                const size_t cq = (size_t)iz * P + x;
                gr -= E.acc[3 * F + cq] * D.BX[cq] / (2.f * dt);
            }
            const int z = iz - q;  // rho_zp[z][ix] averages rho[z][ix], rho[z+1][ix]
            if (z >= 0 && interior(z, ix)) {
                const size_t cq = (size_t)z * P + ix;
                gr -= E.acc[4 * F + cq] * D.BZ[cq] / (2.f * dt);
            }
        }
    }
    D.glam[idx] = gl;
    D.gmu[idx] = gm;
    D.grho[idx] = gr;
}

}  // namespace fwi
