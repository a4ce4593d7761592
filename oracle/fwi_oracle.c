/*
 * fwi_oracle.c -- FP64 CPU restatement of the reference's FWI hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle); see fwi_oracle.h for the
 * scope, the generalisation to orders 4..12 and the reference line map.
 * Compile with -ffp-contract=off so that x86-64 and aarch64 round alike and
 * fdorder-2 results match the reference's own CPU functions bit for bit.
 */
#include "fwi_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IX2(p, iz, ix, pitch) (p)[(size_t)(iz) * (size_t)(pitch) + (size_t)(ix)]

/* Grids below this many cells run their cell loops on one thread (a parallel
 * region per pass costs more than it saves there). */
#define ORC_PAR(g) ((size_t)(g)->nzt * (size_t)(g)->nxt >= 65536)

/* Threads of the cell loops (OpenMP builds; every cell of a pass is computed
 * by one thread from values no thread of that pass writes, so the results do
 * not depend on the thread count).  n <= 0: the OpenMP default. */
int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int orc_nft(int nt, int fwi_dt) { return 1 + (nt - 1) / fwi_dt; }
int orc_nfz(const orc_fwi* f) { return 1 + (f->z2 - f->z1) / f->fwi_dz; }
int orc_nfx(const orc_fwi* f) { return 1 + (f->x2 - f->x1) / f->fwi_dx; }

/* Holberg (1987) optimised staggered-grid coefficients, rows = maximum relative
 * group-velocity error index 0..4 (0 = Taylor), columns = order 2..12; entry 0
 * of each row is the table's accuracy figure, entries 1..6 the coefficients.
 * Same table as CUDA_week2/holbergcoeff.cu:10-52 (published values). */
static const double k_holberg[5][6][7] = {
    {{23.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0},
     {8.0, 9.0 / 8.0, -1.0 / 24.0, 0.0, 0.0, 0.0, 0.0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0.0, 0.0, 0.0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0.0, 0.0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0,
      35.0 / 294912.0, 0.0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0,
      -5445.0 / 1835008.0, 847.0 / 2359296.0, -63.0 / 2883584.0}},
    {{49.7, 1.0010, 0.0, 0.0, 0.0, 0.0, 0.0},
     {8.32, 1.1382, -0.046414, 0.0, 0.0, 0.0, 0.0},
     {4.77, 1.1965, -0.078804, 0.0081781, 0.0, 0.0, 0.0},
     {3.69, 1.2257, -0.099537, 0.018063, -0.0026274, 0.0, 0.0},
     {3.19, 1.2415, -0.11231, 0.026191, -0.0064682, 0.001191, 0.0},
     {2.91, 1.2508, -0.12034, 0.032131, -0.010142, 0.0029857, -0.00066667}},
    {{22.2, 1.0050, 0.0, 0.0, 0.0, 0.0, 0.0},
     {5.65, 1.1534, -0.052806, 0.0, 0.0, 0.0, 0.0},
     {3.74, 1.2111, -0.088313, 0.011768, 0.0, 0.0, 0.0},
     {3.11, 1.2367, -0.10815, 0.023113, -0.0046905, 0.0, 0.0},
     {2.80, 1.2496, -0.11921, 0.031130, -0.0093272, 0.0025161, 0.0},
     {2.62, 1.2568, -0.12573, 0.036423, -0.013132, 0.0047484, -0.0015979}},
    {{15.8, 1.0100, 0.0, 0.0, 0.0, 0.0, 0.0},
     {4.80, 1.1640, -0.057991, 0.0, 0.0, 0.0, 0.0},
     {3.39, 1.2192, -0.094070, 0.014608, 0.0, 0.0, 0.0},
     {2.90, 1.2422, -0.11269, 0.026140, -0.0064054, 0.0, 0.0},
     {2.65, 1.2534, -0.12257, 0.033755, -0.011081, 0.0036784, 0.0},
     {2.51, 1.2596, -0.12825, 0.038550, -0.014763, 0.0058619, -0.0024538}},
    {{9.16, 1.0300, 0.0, 0.0, 0.0, 0.0, 0.0},
     {3.47, 1.1876, -0.072518, 0.0, 0.0, 0.0, 0.0},
     {2.91, 1.2341, -0.10569, 0.022589, 0.0, 0.0, 0.0},
     {2.61, 1.2516, -0.12085, 0.032236, -0.011459, 0.0, 0.0},
     {2.45, 1.2596, -0.12829, 0.038533, -0.014681, 0.0072580, 0.0},
     {2.36, 1.2640, -0.13239, 0.042217, -0.017803, 0.0081959, -0.0051848}},
};

int orc_holberg(int fdorder, int max_rel_err, double hc[7]) {
    int nl = fdorder / 2 - 1;
    if (fdorder < 2 || fdorder > 12 || (fdorder & 1) || max_rel_err < 0 || max_rel_err > 4)
        return -1;
    for (int i = 0; i < 7; i++) hc[i] = k_holberg[max_rel_err][nl][i];
    return 0;
}

/* One side of the CPML profile at abscissa `dist` (metres into the layer, <0 = outside).
 * Writes d, K, alpha following the formulas of fd_cpml.cu:95-110. */
static void cpml_point(double dist, double thickness, double d0, double npower, double kmax,
                       double alpha_max, double* d, double* K, double* alpha) {
    *d = 0.0;
    *alpha = 0.0;
    if (dist >= 0) {
        double xn = dist / thickness;
        *d = d0 * pow(xn, npower);
        *K = 1.0 + (kmax - 1.0) * pow(xn, npower);
        *alpha = alpha_max * (1.0 - xn);
    }
    if (*alpha < 0.0) *alpha = 0.0;
}

static void cpml_ab(double d, double K, double alpha, double dt, double* a, double* b) {
    *b = exp(-(d / K + alpha) * dt);
    if (fabs(d) > 1.0e-6) *a = d * (*b - 1.0) / (K * (d + K * alpha));
}

void orc_cpml(int npml, double dh, double fpml, double npower, double k_max_pml, double rcoef,
              double damp_v_pml, double dt, double* a, double* b, double* K, double* a_half,
              double* b_half, double* K_half) {
    const double alpha_max = 2.0 * ORC_PI * (fpml / 2.0);
    const double thick = npml * dh;
    const double d0 = -(npower + 1) * damp_v_pml * log(rcoef) / (2.0 * thick);
    const int n = 2 * (npml + 1);
    for (int i = 0; i < n; i++) {
        a[i] = 0.0; a_half[i] = 0.0;
        b[i] = 1.0; b_half[i] = 1.0;
        K[i] = 1.0; K_half[i] = 1.0;
    }
    for (int i = 0; i < n; i++) {
        double x = dh * (double)i, dist, dist_h;
        if (i <= npml) { /* left: measured from the outer edge inwards */
            dist = thick - x;
            dist_h = thick - (x + dh / 2.0);
        } else { /* right: measured from dh*(npml+1) outwards */
            dist = x - dh * (npml + 1);
            dist_h = (x + dh / 2.0) - dh * (npml + 1);
        }
        double d, al, dhf, alh;
        cpml_point(dist, thick, d0, npower, k_max_pml, alpha_max, &d, &K[i], &al);
        cpml_point(dist_h, thick, d0, npower, k_max_pml, alpha_max, &dhf, &K_half[i], &alh);
        cpml_ab(d, K[i], al, dt, &a[i], &b[i]);
        cpml_ab(dhf, K_half[i], alh, dt, &a_half[i], &b_half[i]);
    }
}

void orc_average(int nzt, int nxt, const double* lam, const double* mu, const double* rho,
                 double* mu_zx, double* rho_zp, double* rho_xp) {
    (void)lam;
    const int dz = nzt - 1, dx = nxt - 1;
    for (int ix = 0; ix < dx; ix++) {
        for (int iz = 0; iz < dz; iz++) {
            double m00 = IX2(mu, iz, ix, nxt), m01 = IX2(mu, iz, ix + 1, nxt);
            double m10 = IX2(mu, iz + 1, ix, nxt), m11 = IX2(mu, iz + 1, ix + 1, nxt);
            double h = 4.0 / ((1.0 / m00) + (1.0 / m01) + (1.0 / m10) + (1.0 / m11));
            if (m00 == 0.0 || m01 == 0.0 || m10 == 0.0 || m11 == 0.0) h = 0.0;
            IX2(mu_zx, iz, ix, dx) = h;
            double r00 = IX2(rho, iz, ix, nxt), r10 = IX2(rho, iz + 1, ix, nxt);
            double r01 = IX2(rho, iz, ix + 1, nxt);
            IX2(rho_zp, iz, ix, dx) = 1.0 / (0.5 * (r00 + r10));
            IX2(rho_xp, iz, ix, dx) = 1.0 / (0.5 * (r00 + r01));
            if (r00 < 1e-4 && r10 < 1e-4) IX2(rho_zp, iz, ix, dx) = 0.0;
            /* the reference's second guard also writes rho_zp (fd_medium.cu:152-154) */
            if (r00 < 1e-4 && r01 < 1e-4) IX2(rho_zp, iz, ix, dx) = 0.0;
        }
    }
}

void orc_wavelet(double* signal, int nt, double dt, double amp, double fc, double ts, int shape) {
    const double fci = 1.0 / fc;
    if (shape != 1) return;
    for (int it = 0; it < nt; it++) {
        double t = it * dt;
        double tau = ORC_PI * (t - 1.5 * fci - ts) / (1.5 * fci);
        signal[it] = amp * (1.0 - 2.0 * tau * tau) * exp(-2.0 * tau * tau);
    }
}

void orc_total_grid(int nx, int nz, int fdorder, int npml, int fsurf, int* fpad, int* ppad,
                    int* nxt, int* nzt) {
    *fpad = fdorder / 2;
    *ppad = npml + *fpad;
    *nxt = nx + 2 * *ppad;
    *nzt = fsurf ? nz + *ppad + *fpad : nz + 2 * *ppad;
}

/* ---------------------------------------------------------------------------
 * Stencils.  Evaluation order mirrors the reference at fdorder 2:
 *   d = (dxi*hc[1]) * (f[i] - f[i-1]).
 * ------------------------------------------------------------------------- */
static inline double dminus(const double* f, ptrdiff_t c, ptrdiff_t s, int fpad, const double* hd) {
    double acc = 0.0;
    for (int k = 1; k <= fpad; k++) acc += hd[k] * (f[c + (k - 1) * s] - f[c - k * s]);
    return acc;
}
static inline double dplus(const double* f, ptrdiff_t c, ptrdiff_t s, int fpad, const double* hd) {
    double acc = 0.0;
    for (int k = 1; k <= fpad; k++) acc += hd[k] * (f[c + k * s] - f[c - (k - 1) * s]);
    return acc;
}

/* Bottom CPML index offset.  fdorder 2 is the reference's (forward_kernel_PSV_GPU.cu:749-755);
 * with a free surface at higher orders the reference's formula would index past
 * 2(npml+1), so the offset is chosen to keep the same layer cells on indices npml+1..2npml+1. */
static int bottom_offset(const orc_grid* g) {
    if (g->fsurf) return g->nzt - 2 * g->ppad + g->fpad - 2;
    return g->nzt - 2 * g->ppad + g->fpad - 1;
}

/* One stress update (forward_kernel_PSV_GPU.cu:830-931) and the mirror (:934-942). */
static void stress_pass(const orc_grid* g, const orc_medium* m, orc_wave* w) {
    const int nxt = g->nxt, nzt = g->nzt, fpad = g->fpad, ppad = g->ppad, npml = g->npml;
    const int tp = 2 * (npml + 1);
    const int pnx = nxt - 2 * ppad + fpad - 1, pnz = bottom_offset(g);
    const double dxi = 1.0 / g->dx, dzi = 1.0 / g->dz, dt = g->dt;
    double hx[7], hz[7];
    for (int k = 1; k <= fpad; k++) { hx[k] = dxi * g->hc[k]; hz[k] = dzi * g->hc[k]; }
    const int nz1 = fpad, nz2 = nzt - fpad, nx1 = fpad, nx2 = nxt - fpad;
#pragma omp parallel for schedule(static) if (ORC_PAR(g))
    for (int iz = nz1; iz < nz2; iz++) {
        for (int ix = nx1; ix < nx2; ix++) {
            size_t c = (size_t)iz * nxt + ix;
            double vx_x = dminus(w->vx, c, 1, fpad, hx);
            double vz_x = dplus(w->vz, c, 1, fpad, hx);
            double vx_z = dplus(w->vx, c, nxt, fpad, hz);
            double vz_z = dminus(w->vz, c, nxt, fpad, hz);
            if (npml > 0) {
                int px = -1;
                if (ix >= fpad && ix <= ppad) px = ix - fpad;
                if (px >= 0) {
                    double* mx = &IX2(w->mem_vx_x, iz, px, tp);
                    double* mz = &IX2(w->mem_vz_x, iz, px, tp);
                    *mx = g->b[px] * *mx + g->a[px] * vx_x;
                    *mz = g->b_half[px] * *mz + g->a_half[px] * vz_x;
                    vx_x = vx_x / g->K[px] + *mx;
                    vz_x = vz_x / g->K_half[px] + *mz;
                }
                if (ix >= (nxt - ppad - 1) && ix < nxt - fpad) {
                    px = ix - pnx;
                    double* mx = &IX2(w->mem_vx_x, iz, px, tp);
                    double* mz = &IX2(w->mem_vz_x, iz, px, tp);
                    *mx = g->b[px] * *mx + g->a[px] * vx_x;
                    *mz = g->b_half[px] * *mz + g->a_half[px] * vz_x;
                    vx_x = vx_x / g->K[px] + *mx;
                    vz_x = vz_x / g->K_half[px] + *mz;
                }
                if (iz >= fpad && iz <= ppad && !g->fsurf) {
                    int pz = iz - fpad;
                    double* mz = &IX2(w->mem_vz_z, pz, ix, nxt);
                    double* mx = &IX2(w->mem_vx_z, pz, ix, nxt);
                    *mz = g->b[pz] * *mz + g->a[pz] * vz_z;
                    *mx = g->b_half[pz] * *mx + g->a_half[pz] * vx_z;
                    vz_z = vz_z / g->K[pz] + *mz;
                    vx_z = vx_z / g->K_half[pz] + *mx;
                }
                if (iz >= (nzt - ppad - 1) && iz < nzt - fpad) {
                    int pz = iz - pnz;
                    double* mz = &IX2(w->mem_vz_z, pz, ix, nxt);
                    double* mx = &IX2(w->mem_vx_z, pz, ix, nxt);
                    *mz = g->b[pz] * *mz + g->a[pz] * vz_z;
                    *mx = g->b_half[pz] * *mx + g->a_half[pz] * vx_z;
                    vz_z = vz_z / g->K[pz] + *mz;
                    vx_z = vx_z / g->K_half[pz] + *mx;
                }
            }
            const double lam = m->lam[c], mu = m->mu[c];
            const double muzx = IX2(m->mu_zx, iz, ix, nxt - 1);
            w->szx[c] += dt * muzx * (vz_x + vx_z);
            w->sxx[c] += dt * (lam * (vx_x + vz_z) + (2.0 * mu * vx_x));
            w->szz[c] += dt * (lam * (vx_x + vz_z) + (2.0 * mu * vz_z));
            if (g->fsurf && iz == fpad) {
                w->szz[c] = 0.0;
                w->szx[c] = 0.0;
                w->sxx[c] = 4.0 * dt * vx_x * (lam * mu + mu * mu) / (lam + 2.0 * mu);
            }
        }
    }
    if (g->fsurf) {
#pragma omp parallel for schedule(static) if (ORC_PAR(g))
        for (int ix = nx1; ix < nx2; ix++)
            for (int sz = 1; sz <= fpad; sz++) {
                IX2(w->szx, fpad - sz, ix, nxt) = -IX2(w->szx, fpad + sz, ix, nxt);
                IX2(w->szz, fpad - sz, ix, nxt) = -IX2(w->szz, fpad + sz, ix, nxt);
            }
    }
}

/* One velocity update with energy accumulation (forward_kernel_PSV_GPU.cu:946-1023). */
static void velocity_pass(const orc_grid* g, const orc_medium* m, orc_wave* w) {
    const int nxt = g->nxt, nzt = g->nzt, fpad = g->fpad, ppad = g->ppad, npml = g->npml;
    const int tp = 2 * (npml + 1);
    const int pnx = nxt - 2 * ppad + fpad - 1, pnz = bottom_offset(g);
    const double dxi = 1.0 / g->dx, dzi = 1.0 / g->dz, dt = g->dt;
    double hx[7], hz[7];
    for (int k = 1; k <= fpad; k++) { hx[k] = dxi * g->hc[k]; hz[k] = dzi * g->hc[k]; }
    const int nz1 = fpad, nz2 = nzt - fpad, nx1 = fpad, nx2 = nxt - fpad;
#pragma omp parallel for schedule(static) if (ORC_PAR(g))
    for (int iz = nz1; iz < nz2; iz++) {
        for (int ix = nx1; ix < nx2; ix++) {
            size_t c = (size_t)iz * nxt + ix;
            double sxx_x = dplus(w->sxx, c, 1, fpad, hx);
            double szx_x = dminus(w->szx, c, 1, fpad, hx);
            double szx_z = dminus(w->szx, c, nxt, fpad, hz);
            double szz_z = dplus(w->szz, c, nxt, fpad, hz);
            if (npml > 0) {
                if (ix >= fpad && ix < ppad) {
                    int px = ix - fpad;
                    double* mx = &IX2(w->mem_sxx_x, iz, px, tp);
                    double* mz = &IX2(w->mem_szx_x, iz, px, tp);
                    *mx = g->b[px] * *mx + g->a[px] * sxx_x;
                    *mz = g->b_half[px] * *mz + g->a_half[px] * szx_x;
                    sxx_x = sxx_x / g->K[px] + *mx;
                    szx_x = szx_x / g->K_half[px] + *mz;
                }
                if (ix >= (nxt - ppad - 1) && ix < nxt - fpad) {
                    int px = ix - pnx;
                    double* mx = &IX2(w->mem_sxx_x, iz, px, tp);
                    double* mz = &IX2(w->mem_szx_x, iz, px, tp);
                    *mx = g->b[px] * *mx + g->a[px] * sxx_x;
                    *mz = g->b_half[px] * *mz + g->a_half[px] * szx_x;
                    sxx_x = sxx_x / g->K[px] + *mx;
                    szx_x = szx_x / g->K_half[px] + *mz;
                }
                if (iz >= fpad && iz < ppad && !g->fsurf) {
                    int pz = iz - fpad;
                    double* mz = &IX2(w->mem_szz_z, pz, ix, nxt);
                    double* mx = &IX2(w->mem_szx_z, pz, ix, nxt);
                    *mz = g->b[pz] * *mz + g->a[pz] * szz_z;
                    *mx = g->b_half[pz] * *mx + g->a_half[pz] * szx_z;
                    szz_z = szz_z / g->K[pz] + *mz;
                    szx_z = szx_z / g->K_half[pz] + *mx;
                }
                if (iz >= (nzt - ppad - 1) && iz < nzt - fpad) {
                    int pz = iz - pnz;
                    double* mz = &IX2(w->mem_szz_z, pz, ix, nxt);
                    double* mx = &IX2(w->mem_szx_z, pz, ix, nxt);
                    *mz = g->b[pz] * *mz + g->a[pz] * szz_z;
                    *mx = g->b_half[pz] * *mx + g->a_half[pz] * szx_z;
                    szz_z = szz_z / g->K[pz] + *mz;
                    szx_z = szx_z / g->K_half[pz] + *mx;
                }
            }
            const double rxp = IX2(m->rho_xp, iz, ix, nxt - 1);
            const double rzp = IX2(m->rho_zp, iz, ix, nxt - 1);
            w->vx[c] += dt * rxp * (sxx_x + szx_z);
            w->vz[c] += dt * rzp * (szx_x + szz_z);
            w->We[c] += w->vx[c] * w->vx[c] + w->vz[c] * w->vz[c];
        }
    }
}

static void reset_wave(const orc_grid* g, orc_wave* w) {
    size_t n = (size_t)g->nzt * g->nxt;
    size_t nxs = (size_t)g->nzt * 2 * (g->npml + 1), nzs = (size_t)2 * (g->npml + 1) * g->nxt;
    memset(w->vx, 0, n * sizeof(double));
    memset(w->vz, 0, n * sizeof(double));
    memset(w->sxx, 0, n * sizeof(double));
    memset(w->szx, 0, n * sizeof(double));
    memset(w->szz, 0, n * sizeof(double));
    memset(w->We, 0, n * sizeof(double));
    /* the reference's driver resets the CPML memory before every pass
     * (fd_wave_model.cu:781-785, 839-840); the oracle does it here */
    memset(w->mem_vx_x, 0, nxs * sizeof(double));
    memset(w->mem_vz_x, 0, nxs * sizeof(double));
    memset(w->mem_sxx_x, 0, nxs * sizeof(double));
    memset(w->mem_szx_x, 0, nxs * sizeof(double));
    memset(w->mem_vx_z, 0, nzs * sizeof(double));
    memset(w->mem_vz_z, 0, nzs * sizeof(double));
    memset(w->mem_szz_z, 0, nzs * sizeof(double));
    memset(w->mem_szx_z, 0, nzs * sizeof(double));
}

static int check_grid(const orc_grid* g) {
    if (g->fdorder < 2 || g->fdorder > 12 || (g->fdorder & 1)) return -1;
    if (g->fpad != g->fdorder / 2 || g->ppad != g->npml + g->fpad) return -2;
    if (g->nt < 1 || g->nxt <= 2 * g->ppad || g->nzt <= 2 * g->fpad) return -3;
    return 0;
}

int orc_forward(int ishot, const orc_grid* g, const orc_medium* m, orc_wave* w,
                const orc_seis* src, const double* src_signal, const orc_seis* rec,
                double* rec_signal, orc_fwi* f) {
    int rc = check_grid(g);
    if (rc) return rc;
    const int nxt = g->nxt, nt = g->nt;
    reset_wave(g, w);
    int nft = 0, nfz = 0, nfx = 0;
    if (f && f->fwinv) {
        nft = orc_nft(nt, f->fwi_dt); nfz = orc_nfz(f); nfx = orc_nfx(f);
        size_t ns = (size_t)nft * nfz * nfx;
        memset(f->vx, 0, ns * sizeof(double)); memset(f->vz, 0, ns * sizeof(double));
        memset(f->sxx, 0, ns * sizeof(double)); memset(f->szx, 0, ns * sizeof(double));
        memset(f->szz, 0, ns * sizeof(double));
    }
    for (int it = 0; it < nt; it++) {
        if (f && f->fwinv && !(it % f->fwi_dt)) {
            int tf = it / f->fwi_dt;
            for (int iz = f->z1; iz < f->z2; iz += f->fwi_dz) {
                int zf = (iz - f->z1) / f->fwi_dz;
                for (int ix = f->x1; ix < f->x2; ix += f->fwi_dx) {
                    int xf = (ix - f->x1) / f->fwi_dx;
                    size_t o = ((size_t)tf * nfz + zf) * nfx + xf, c = (size_t)iz * nxt + ix;
                    f->sxx[o] = w->sxx[c];
                    f->szx[o] = w->szx[c];
                    f->szz[o] = w->szz[c];
                    f->vx[o] = w->vx[c] / g->dt;
                    f->vz[o] = w->vz[c] / g->dt;
                }
            }
        }
        stress_pass(g, m, w);
        velocity_pass(g, m, w);
        for (int is = 0; src && is < src->n; is++)
            if (src->shot[is] == ishot && src->comp[is] == 2)
                IX2(w->vz, src->z[is], src->x[is], nxt) += src_signal[(size_t)is * nt + it];
        for (int ir = 0; rec && ir < rec->n; ir++)
            if (rec->shot[ir] == ishot && rec->comp[ir] == 2)
                rec_signal[(size_t)ir * nt + it] = IX2(w->vz, rec->z[ir], rec->x[ir], nxt);
    }
    return 0;
}

/* One reverse step of orc_adjoint at time step it (adjoint_kernel_PSV_GPU.cu:818-1087):
 * ux/uz integration, the correlation gradient from the forward fields of frame
 * `frame` of the storage arrays st[5] (vx/dt, vz/dt, sxx, szx, szz; each
 * [frames][nfz][nfx]) when it is a sampled step, the stress and velocity passes
 * and the injection of adj_signal.  Shared by the stored-wavefield and the
 * checkpointed gradients, so both run the same statements. */
static void ref_adjoint_step(int ishot, const orc_grid* g, const orc_medium* m, orc_wave* w, double* ux,
                             double* uz, const orc_seis* adj, const double* adj_signal, const orc_fwi* f,
                             const double* const st[5], int it, int frame, double* grad_lam, double* grad_mu,
                             double* grad_rho) {
    const int nxt = g->nxt, nzt = g->nzt, nt = g->nt, fpad = g->fpad;
    const double dt = g->dt;
    const int nfz = orc_nfz(f), nfx = orc_nfx(f);
#pragma omp parallel for schedule(static) if (ORC_PAR(g))
    for (int iz = fpad; iz < nzt - fpad; iz++)
        for (int ix = fpad; ix < nxt - fpad; ix++) {
            size_t c = (size_t)iz * nxt + ix;
            uz[c] += dt * w->vz[c];
            ux[c] += dt * w->vx[c];
        }
    if (f->fwinv && !(it % f->fwi_dt)) {
        const double *fvx = st[0], *fvz = st[1], *fsxx = st[2], *fszx = st[3], *fszz = st[4];
#pragma omp parallel for schedule(static) if (ORC_PAR(g))
        for (int iz = f->z1; iz < f->z2; iz += f->fwi_dz) {
            int zf = (iz - f->z1) / f->fwi_dz;
            for (int ix = f->x1; ix < f->x2; ix += f->fwi_dx) {
                int xf = (ix - f->x1) / f->fwi_dx;
                size_t o = ((size_t)frame * nfz + zf) * nfx + xf, c = (size_t)iz * nxt + ix;
                size_t gi = (size_t)zf * nfx + xf;
                double lam = m->lam[c], mu = m->mu[c];
                double s1 = (fsxx[o] + fszz[o]) * (w->sxx[c] + w->szz[c]) * 0.25 /
                            ((lam + mu) * (lam + mu));
                double s2 = (fsxx[o] - fszz[o]) * (w->sxx[c] - w->szz[c]) / (mu * mu);
                double s3 = (fszx[o] * w->szx[c]) / (mu * mu);
                double s4 = ux[c] * fvx[o] + uz[c] * fvz[o];
                grad_lam[gi] += f->fwi_dt * dt * s1;
                grad_mu[gi] += f->fwi_dt * dt * (s3 + s1 + s2);
                grad_rho[gi] -= f->fwi_dt * dt * s4;
            }
        }
    }
    stress_pass(g, m, w);
    velocity_pass(g, m, w);
    for (int is = 0; adj && is < adj->n; is++)
        if (adj->shot[is] == ishot && adj->comp[is] == 2)
            IX2(w->vz, adj->z[is], adj->x[is], nxt) += adj_signal[(size_t)is * nt + it];
}

int orc_adjoint(int ishot, const orc_grid* g, const orc_medium* m, orc_wave* w,
                const orc_seis* adj, const double* adj_signal, const orc_fwi* f,
                double* grad_lam, double* grad_mu, double* grad_rho) {
    int rc = check_grid(g);
    if (rc) return rc;
    const int nxt = g->nxt, nzt = g->nzt, nt = g->nt;
    reset_wave(g, w);
    size_t n = (size_t)nzt * nxt;
    double* ux = (double*)calloc(n, sizeof(double));
    double* uz = (double*)calloc(n, sizeof(double));
    if (!ux || !uz) { free(ux); free(uz); return -4; }
    const int nfz = orc_nfz(f), nfx = orc_nfx(f);
    memset(grad_lam, 0, (size_t)nfz * nfx * sizeof(double));
    memset(grad_mu, 0, (size_t)nfz * nfx * sizeof(double));
    memset(grad_rho, 0, (size_t)nfz * nfx * sizeof(double));
    const double* const st[5] = {f->vx, f->vz, f->sxx, f->szx, f->szz};
    for (int it = nt - 1; it >= 0; it--)
        ref_adjoint_step(ishot, g, m, w, ux, uz, adj, adj_signal, f, st, it, it / f->fwi_dt, grad_lam, grad_mu,
                         grad_rho);
    free(ux);
    free(uz);
    return 0;
}

double orc_l2_adjoint_sources(int nr, int nt, double dt, double* signal, const double* signal_meas,
                              int* blowup) {
    double misfit = 0.0;
    if (blowup) *blowup = 0;
    for (int ir = 0; ir < nr; ir++)
        for (int it = 0; it < nt; it++) {
            size_t i = (size_t)ir * nt + it;
            double diff = signal[i] - signal_meas[i];
            misfit += 0.5 * dt * diff * diff;
            signal[i] = diff;
            if (fabs(diff) > 1.0e+10 && blowup) *blowup = 1;
        }
    return misfit;
}

void orc_medium_average(int nzt, int nxt, const double* lam, const double* mu, const double* rho,
                        double* c_lam, double* c_mu, double* c_rho) {
    double sl = 0.0, sm = 0.0, sr = 0.0;
    for (int iz = 0; iz < nzt; iz++)
        for (int ix = 0; ix < nxt; ix++) {
            size_t c = (size_t)iz * nxt + ix;
            sl += lam[c]; sm += mu[c]; sr += rho[c];
        }
    *c_lam = sl / (nzt * nxt);
    *c_mu = sm / (nzt * nxt);
    *c_rho = sr / (nzt * nxt);
}

void orc_scale_gradients(int nxt, const double* Ws, const double* Wr, double c_rho, double c_lam,
                         double c_mu, int nz, int nx, int z1, int x1, int fdz, int fdx,
                         int grad_pitch, double* grad_lam, double* grad_mu, double* grad_rho) {
    const double eps = 0.005;
    double wmax = 0.0;
    for (int iz = z1; iz < nz; iz += fdz)
        for (int ix = x1; ix < nx; ix += fdx) {
            double we = sqrt(IX2(Ws, iz, ix, nxt) * IX2(Wr, iz, ix, nxt));
            if (we > wmax) wmax = we;
        }
    for (int iz = z1; iz < nz; iz += fdz)
        for (int ix = x1; ix < nx; ix += fdx) {
            double we = sqrt(IX2(Ws, iz, ix, nxt) * IX2(Wr, iz, ix, nxt)) + eps * wmax;
            size_t gi = (size_t)iz * grad_pitch + ix;
            grad_lam[gi] = grad_lam[gi] / (we * c_lam * c_lam);
            grad_mu[gi] = grad_mu[gi] / (we * c_mu * c_mu);
            grad_rho[gi] = grad_rho[gi] / (we * c_rho * c_rho);
        }
}

void orc_grad_update(double* mat, double* mat_new, const double* grad, int pitch, int gpitch,
                     double step_length, int dimz, int dimx, int z1, int x1, int fwi_dz,
                     int fwi_dx, int override_, int mat_type) {
    double mat_max = 0.0, grad_max = 0.0, hi = 0.0, lo = 0.0;
    if (mat_type == 1) { hi = 3000; lo = 1.5; }
    else if (mat_type == 2) { hi = 48.0e+9; lo = 0; }
    else if (mat_type == 3) { hi = 27.0e+9; lo = 0; }
    for (int iz = z1; iz < dimz; iz += fwi_dz)
        for (int ix = x1; ix < dimx; ix += fwi_dx) {
            double mv = IX2(mat, iz, ix, pitch), gv = IX2(grad, iz, ix, gpitch);
            if (mv > mat_max) mat_max = mv;
            /* the reference stores the signed value of the largest |grad| */
            if (fabs(gv) > grad_max) grad_max = gv;
        }
    double sn = step_length * (mat_max / grad_max);
    for (int iz = z1; iz < dimz; iz += fwi_dz)
        for (int ix = x1; ix < dimx; ix += fwi_dx) {
            double* nv = &IX2(mat_new, iz, ix, pitch);
            *nv = IX2(mat, iz, ix, pitch) + sn * IX2(grad, iz, ix, gpitch);
            if (*nv < lo) *nv = lo;
            if (*nv > hi) *nv = hi;
            if (*nv < 0.0) *nv = IX2(mat, iz, ix, pitch);
        }
    if (override_)
        for (int iz = z1; iz < dimz; iz += fwi_dz)
            for (int ix = x1; ix < dimx; ix += fwi_dx)
                IX2(mat, iz, ix, pitch) = IX2(mat_new, iz, ix, pitch);
}

double orc_calc_opt_step(const double* L2, const double* sl) {
    /* Gauss elimination with the reference's float multiplier and float
     * back-substitution accumulator (solvelin.cu:10).  The reference starts its
     * back substitution one row past the end (solvelin.cu:29), which reads
     * outside the arrays; this restatement starts at the last row. */
    double A[3][3], b[3], x[3] = {0, 0, 0};
    for (int i = 0; i < 3; i++) { A[i][2] = sl[i] * sl[i]; A[i][1] = sl[i]; A[i][0] = 1.0; b[i] = L2[i]; }
    for (int k = 0; k < 2; k++)
        for (int n = k; n < 2; n++) {
            float a = (float)(A[n + 1][k] / A[k][k]);
            for (int mm = 0; mm < 3; mm++) A[n + 1][mm] = A[n + 1][mm] - a * A[k][mm];
            b[n + 1] = b[n + 1] - a * b[k];
        }
    for (int k = 2; k >= 0; k--) {
        float c = (float)b[k];
        for (int mm = 2; mm > k; mm--) c = (float)(c - A[k][mm] * x[mm]);
        x[k] = c / A[k][k];
    }
    return -x[1] / (2.0 * x[2]);
}

/* ---------------------------------------------------------------------------
 * Exact discrete adjoint (this oracle's own addition; the reference has no
 * such mode).  It differentiates J = sum_it sum_r 0.5 dt (rec_r(it) - obs_r(it))^2
 * of the time stepping above (stress_pass, velocity_pass, source injection,
 * recording) with respect to lam, mu and rho, by transposing every statement
 * of one step in reverse order and scattering each adjoint onto the cells the
 * forward statement read.  Forward states come from sqrt(nt) checkpoints with
 * per-segment recomputation, so memory stays at about 2 sqrt(nt) states.
 * ------------------------------------------------------------------------- */

typedef struct {
    size_t n, nxs, nzs, total;
} st_sizes;

static st_sizes state_sizes(const orc_grid* g) {
    st_sizes s;
    s.n = (size_t)g->nzt * g->nxt;
    s.nxs = (size_t)g->nzt * 2 * (g->npml + 1);
    s.nzs = (size_t)2 * (g->npml + 1) * g->nxt;
    s.total = 5 * s.n + 4 * s.nxs + 4 * s.nzs;
    return s;
}

/* orc_wave view of one contiguous state block (We points to scratch). */
static void wave_view(const orc_grid* g, double* base, double* we, orc_wave* w) {
    st_sizes s = state_sizes(g);
    w->vx = base; w->vz = base + s.n; w->sxx = base + 2 * s.n; w->szx = base + 3 * s.n;
    w->szz = base + 4 * s.n;
    double* x = base + 5 * s.n;
    w->mem_vx_x = x; w->mem_vz_x = x + s.nxs; w->mem_sxx_x = x + 2 * s.nxs; w->mem_szx_x = x + 3 * s.nxs;
    double* z = x + 4 * s.nxs;
    w->mem_vx_z = z; w->mem_vz_z = z + s.nzs; w->mem_szz_z = z + 2 * s.nzs; w->mem_szx_z = z + 3 * s.nzs;
    w->We = we;
}

static void fwd_step(const orc_grid* g, const orc_medium* m, orc_wave* w, int it, int ishot,
                     const orc_seis* src, const double* src_signal) {
    stress_pass(g, m, w);
    velocity_pass(g, m, w);
    for (int is = 0; src && is < src->n; is++)
        if (src->shot[is] == ishot && src->comp[is] == 2)
            IX2(w->vz, src->z[is], src->x[is], g->nxt) += src_signal[(size_t)is * g->nt + it];
}

/* CPML strips touching a cell, in the order the forward applies them.
 * kind 0: stress pass (x: ix <= ppad, z: iz <= ppad); kind 1: velocity pass (<). */
typedef struct {
    int n, p[2];
} strips;

static strips x_strips(const orc_grid* g, int ix, int kind) {
    strips s = {0, {0, 0}};
    if (g->npml <= 0) return s;
    const int pnx = g->nxt - 2 * g->ppad + g->fpad - 1;
    if (ix >= g->fpad && (kind == 0 ? ix <= g->ppad : ix < g->ppad)) s.p[s.n++] = ix - g->fpad;
    if (ix >= g->nxt - g->ppad - 1 && ix < g->nxt - g->fpad) s.p[s.n++] = ix - pnx;
    return s;
}

static strips z_strips(const orc_grid* g, int iz, int kind) {
    strips s = {0, {0, 0}};
    if (g->npml <= 0) return s;
    if (!g->fsurf && iz >= g->fpad && (kind == 0 ? iz <= g->ppad : iz < g->ppad)) s.p[s.n++] = iz - g->fpad;
    if (iz >= g->nzt - g->ppad - 1 && iz < g->nzt - g->fpad) s.p[s.n++] = iz - bottom_offset(g);
    return s;
}

/* Post-CPML derivative u' as the forward computes it from the memory before the step. */
static double cpml_apply(double u, strips s, const double* mem, size_t stride, size_t off,
                         const double* a, const double* b, const double* K) {
    for (int i = 0; i < s.n; i++) {
        const int p = s.p[i];
        const double mn = b[p] * mem[(size_t)p * stride + off] + a[p] * u;
        u = u / K[p] + mn;
    }
    return u;
}

/* Transpose of the CPML chain: ubar' -> ubar, updating the memory adjoints. */
static double cpml_transpose(double ub, strips s, double* madj, size_t stride, size_t off,
                             const double* a, const double* b, const double* K) {
    for (int i = s.n - 1; i >= 0; i--) {
        const int p = s.p[i];
        double* mb = &madj[(size_t)p * stride + off];
        const double tot = *mb + ub;
        *mb = b[p] * tot;
        ub = ub / K[p] + a[p] * tot;
    }
    return ub;
}

/* Scatter the transposes of D- / D+ applied at cell c (stride s) with adjoint gb into fb. */
static void scatter_dminus(double* fb, size_t c, ptrdiff_t s, int fpad, const double* hd, double gb) {
    for (int k = 1; k <= fpad; k++) {
        fb[c + (k - 1) * s] += hd[k] * gb;
        fb[c - k * s] -= hd[k] * gb;
    }
}
static void scatter_dplus(double* fb, size_t c, ptrdiff_t s, int fpad, const double* hd, double gb) {
    for (int k = 1; k <= fpad; k++) {
        fb[c + k * s] += hd[k] * gb;
        fb[c - (k - 1) * s] -= hd[k] * gb;
    }
}

/* One reverse step: aw holds the adjoint of state n+1 on entry (receiver
 * adjoint sources already added) and of state n on exit.  xn / xn1 are the
 * forward states n and n+1.  Material sensitivities accumulate into g_lam,
 * g_mu ([nzt][nxt]) and g_muzx, g_rzp, g_rxp ([nzt-1][nxt-1]). */
static void adjoint_step(const orc_grid* g, const orc_medium* m, const orc_wave* xn, const orc_wave* xn1,
                         orc_wave* aw, double* g_lam, double* g_mu, double* g_muzx, double* g_rzp,
                         double* g_rxp) {
    const int nxt = g->nxt, nzt = g->nzt, fpad = g->fpad, tp = 2 * (g->npml + 1);
    const double dt = g->dt;
    double hx[7], hz[7];
    for (int k = 1; k <= fpad; k++) { hx[k] = g->hc[k] / g->dx; hz[k] = g->hc[k] / g->dz; }
    /* velocity pass (forward_kernel_PSV_GPU.cu:946-1023), transposed */
    for (int iz = fpad; iz < nzt - fpad; iz++)
        for (int ix = fpad; ix < nxt - fpad; ix++) {
            const size_t c = (size_t)iz * nxt + ix, ca = (size_t)iz * (nxt - 1) + ix;
            const strips sx = x_strips(g, ix, 1), sz = z_strips(g, iz, 1);
            double sxx_x = dplus(xn1->sxx, c, 1, fpad, hx);
            double szx_x = dminus(xn1->szx, c, 1, fpad, hx);
            double szx_z = dminus(xn1->szx, c, nxt, fpad, hz);
            double szz_z = dplus(xn1->szz, c, nxt, fpad, hz);
            sxx_x = cpml_apply(sxx_x, sx, xn->mem_sxx_x, 1, (size_t)iz * tp, g->a, g->b, g->K);
            szx_x = cpml_apply(szx_x, sx, xn->mem_szx_x, 1, (size_t)iz * tp, g->a_half, g->b_half, g->K_half);
            szz_z = cpml_apply(szz_z, sz, xn->mem_szz_z, nxt, ix, g->a, g->b, g->K);
            szx_z = cpml_apply(szx_z, sz, xn->mem_szx_z, nxt, ix, g->a_half, g->b_half, g->K_half);
            const double vxb = aw->vx[c], vzb = aw->vz[c];
            const double rxp = m->rho_xp[ca], rzp = m->rho_zp[ca];
            g_rxp[ca] += vxb * dt * (sxx_x + szx_z);
            g_rzp[ca] += vzb * dt * (szx_x + szz_z);
            const double w1 = dt * rxp * vxb, w2 = dt * rzp * vzb;
            const double gsxx = cpml_transpose(w1, sx, aw->mem_sxx_x, 1, (size_t)iz * tp, g->a, g->b, g->K);
            const double gszx_x =
                cpml_transpose(w2, sx, aw->mem_szx_x, 1, (size_t)iz * tp, g->a_half, g->b_half, g->K_half);
            const double gszz = cpml_transpose(w2, sz, aw->mem_szz_z, nxt, ix, g->a, g->b, g->K);
            const double gszx_z = cpml_transpose(w1, sz, aw->mem_szx_z, nxt, ix, g->a_half, g->b_half, g->K_half);
            scatter_dplus(aw->sxx, c, 1, fpad, hx, gsxx);
            scatter_dminus(aw->szx, c, 1, fpad, hx, gszx_x);
            scatter_dminus(aw->szx, c, nxt, fpad, hz, gszx_z);
            scatter_dplus(aw->szz, c, nxt, fpad, hz, gszz);
        }
    /* stress mirror above the free surface (:934-942), transposed */
    if (g->fsurf)
        for (int ix = fpad; ix < nxt - fpad; ix++)
            for (int s = 1; s <= fpad; s++) {
                IX2(aw->szx, fpad + s, ix, nxt) -= IX2(aw->szx, fpad - s, ix, nxt);
                IX2(aw->szz, fpad + s, ix, nxt) -= IX2(aw->szz, fpad - s, ix, nxt);
                IX2(aw->szx, fpad - s, ix, nxt) = 0.0;
                IX2(aw->szz, fpad - s, ix, nxt) = 0.0;
            }
    /* stress pass (:830-931), transposed */
    for (int iz = fpad; iz < nzt - fpad; iz++)
        for (int ix = fpad; ix < nxt - fpad; ix++) {
            const size_t c = (size_t)iz * nxt + ix, ca = (size_t)iz * (nxt - 1) + ix;
            const strips sx = x_strips(g, ix, 0), sz = z_strips(g, iz, 0);
            double vx_x = dminus(xn->vx, c, 1, fpad, hx);
            double vz_x = dplus(xn->vz, c, 1, fpad, hx);
            double vx_z = dplus(xn->vx, c, nxt, fpad, hz);
            double vz_z = dminus(xn->vz, c, nxt, fpad, hz);
            vx_x = cpml_apply(vx_x, sx, xn->mem_vx_x, 1, (size_t)iz * tp, g->a, g->b, g->K);
            vz_x = cpml_apply(vz_x, sx, xn->mem_vz_x, 1, (size_t)iz * tp, g->a_half, g->b_half, g->K_half);
            vz_z = cpml_apply(vz_z, sz, xn->mem_vz_z, nxt, ix, g->a, g->b, g->K);
            vx_z = cpml_apply(vx_z, sz, xn->mem_vx_z, nxt, ix, g->a_half, g->b_half, g->K_half);
            const double lam = m->lam[c], mu = m->mu[c];
            const double sxxb = aw->sxx[c], szxb = aw->szx[c], szzb = aw->szz[c];
            double ax, bx, az, bz;  /* adjoints of vx_x', vz_x', vx_z', vz_z' */
            if (g->fsurf && iz == fpad) {
                /* sxx = 4 dt vx_x (lam mu + mu^2) / (lam + 2 mu); szz = szx = 0 */
                const double den = lam + 2.0 * mu;
                g_lam[c] += sxxb * vx_x * 4.0 * dt * mu * mu / (den * den);
                g_mu[c] += sxxb * vx_x * 4.0 * dt * (lam * lam + 2.0 * lam * mu + 2.0 * mu * mu) / (den * den);
                ax = sxxb * 4.0 * dt * (lam * mu + mu * mu) / den;
                bx = az = bz = 0.0;
                aw->sxx[c] = aw->szx[c] = aw->szz[c] = 0.0;
            } else {
                const double muzx = m->mu_zx[ca];
                g_muzx[ca] += szxb * dt * (vz_x + vx_z);
                g_lam[c] += (sxxb + szzb) * dt * (vx_x + vz_z);
                g_mu[c] += 2.0 * dt * (sxxb * vx_x + szzb * vz_z);
                ax = dt * (lam + 2.0 * mu) * sxxb + dt * lam * szzb;
                bz = dt * lam * sxxb + dt * (lam + 2.0 * mu) * szzb;
                bx = az = dt * muzx * szxb;
            }
            ax = cpml_transpose(ax, sx, aw->mem_vx_x, 1, (size_t)iz * tp, g->a, g->b, g->K);
            bx = cpml_transpose(bx, sx, aw->mem_vz_x, 1, (size_t)iz * tp, g->a_half, g->b_half, g->K_half);
            bz = cpml_transpose(bz, sz, aw->mem_vz_z, nxt, ix, g->a, g->b, g->K);
            az = cpml_transpose(az, sz, aw->mem_vx_z, nxt, ix, g->a_half, g->b_half, g->K_half);
            scatter_dminus(aw->vx, c, 1, fpad, hx, ax);
            scatter_dplus(aw->vz, c, 1, fpad, hx, bx);
            scatter_dplus(aw->vx, c, nxt, fpad, hz, az);
            scatter_dminus(aw->vz, c, nxt, fpad, hz, bz);
        }
}

int orc_exact_gradient(int ishot, const orc_grid* g, const double* lam, const double* mu, const double* rho,
                       const orc_seis* src, const double* src_signal, const orc_seis* rec, const double* obs,
                       double* misfit, double* grad_lam, double* grad_mu, double* grad_rho) {
    int rc = check_grid(g);
    if (rc) return rc;
    const int nt = g->nt, nzt = g->nzt, nxt = g->nxt;
    const double dt = g->dt;
    const st_sizes ss = state_sizes(g);
    const size_t na = (size_t)(nzt - 1) * (nxt - 1);
    int K = 1;
    while ((long long)K * K < nt) K++;
    const int nck = (nt + K - 1) / K;
    double* mzx = (double*)calloc(3 * na, sizeof(double));
    double* chk = (double*)calloc((size_t)nck * ss.total, sizeof(double));
    double* seg = (double*)calloc((size_t)(K + 1) * ss.total, sizeof(double));
    double* adj = (double*)calloc(ss.total, sizeof(double));
    double* we = (double*)calloc(ss.n, sizeof(double));
    double* gavg = (double*)calloc(3 * na, sizeof(double));
    double* recs = (double*)calloc((size_t)(rec ? rec->n : 0) * nt + 1, sizeof(double));
    if (!mzx || !chk || !seg || !adj || !we || !gavg || !recs) {
        free(mzx); free(chk); free(seg); free(adj); free(we); free(gavg); free(recs);
        return -4;
    }
    orc_average(nzt, nxt, lam, mu, rho, mzx, mzx + na, mzx + 2 * na);
    orc_medium med = {lam, mu, mzx, mzx + na, mzx + 2 * na};
    double *g_muzx = gavg, *g_rzp = gavg + na, *g_rxp = gavg + 2 * na;
    memset(grad_lam, 0, ss.n * sizeof(double));
    memset(grad_mu, 0, ss.n * sizeof(double));
    memset(grad_rho, 0, ss.n * sizeof(double));
    /* forward sweep: checkpoints every K steps, records kept */
    orc_wave w;
    wave_view(g, seg, we, &w);
    double J = 0.0;
    for (int it = 0; it < nt; it++) {
        if (it % K == 0) memcpy(chk + (size_t)(it / K) * ss.total, seg, ss.total * sizeof(double));
        fwd_step(g, &med, &w, it, ishot, src, src_signal);
        for (int ir = 0; rec && ir < rec->n; ir++)
            if (rec->shot[ir] == ishot && rec->comp[ir] == 2) {
                const double v = IX2(w.vz, rec->z[ir], rec->x[ir], nxt);
                recs[(size_t)ir * nt + it] = v;
                const double d = v - obs[(size_t)ir * nt + it];
                J += 0.5 * dt * d * d;
            }
    }
    /* reverse sweep, segment by segment */
    orc_wave aw;
    wave_view(g, adj, we, &aw);
    for (int j = nck - 1; j >= 0; j--) {
        const int k0 = j * K, k1 = k0 + K < nt ? k0 + K : nt;
        memcpy(seg, chk + (size_t)j * ss.total, ss.total * sizeof(double));
        for (int it = k0; it < k1; it++) {
            double* nxtst = seg + (size_t)(it - k0 + 1) * ss.total;
            memcpy(nxtst, nxtst - ss.total, ss.total * sizeof(double));
            orc_wave ws;
            wave_view(g, nxtst, we, &ws);
            fwd_step(g, &med, &ws, it, ishot, src, src_signal);
        }
        for (int it = k1 - 1; it >= k0; it--) {
            for (int ir = 0; rec && ir < rec->n; ir++)
                if (rec->shot[ir] == ishot && rec->comp[ir] == 2)
                    IX2(aw.vz, rec->z[ir], rec->x[ir], nxt) +=
                        dt * (recs[(size_t)ir * nt + it] - obs[(size_t)ir * nt + it]);
            orc_wave xn, xn1;
            wave_view(g, seg + (size_t)(it - k0) * ss.total, we, &xn);
            wave_view(g, seg + (size_t)(it - k0 + 1) * ss.total, we, &xn1);
            adjoint_step(g, &med, &xn, &xn1, &aw, grad_lam, grad_mu, g_muzx, g_rzp, g_rxp);
        }
    }
    /* staggered averages (fd_medium.cu:128-159) -> raw mu and rho */
    for (int iz = 0; iz < nzt - 1; iz++)
        for (int ix = 0; ix < nxt - 1; ix++) {
            const size_t a = (size_t)iz * (nxt - 1) + ix;
            const double m00 = IX2(mu, iz, ix, nxt), m01 = IX2(mu, iz, ix + 1, nxt);
            const double m10 = IX2(mu, iz + 1, ix, nxt), m11 = IX2(mu, iz + 1, ix + 1, nxt);
            if (m00 != 0.0 && m01 != 0.0 && m10 != 0.0 && m11 != 0.0) {
                const double h = mzx[a], q = g_muzx[a] * h * h / 4.0;
                IX2(grad_mu, iz, ix, nxt) += q / (m00 * m00);
                IX2(grad_mu, iz, ix + 1, nxt) += q / (m01 * m01);
                IX2(grad_mu, iz + 1, ix, nxt) += q / (m10 * m10);
                IX2(grad_mu, iz + 1, ix + 1, nxt) += q / (m11 * m11);
            }
            const double r00 = IX2(rho, iz, ix, nxt), r10 = IX2(rho, iz + 1, ix, nxt);
            const double r01 = IX2(rho, iz, ix + 1, nxt);
            const int zguard = (r00 < 1e-4 && r10 < 1e-4) || (r00 < 1e-4 && r01 < 1e-4);
            if (!zguard) {
                const double rz = mzx[na + a], dz = -0.5 * rz * rz * g_rzp[a];
                IX2(grad_rho, iz, ix, nxt) += dz;
                IX2(grad_rho, iz + 1, ix, nxt) += dz;
            }
            const double rx = mzx[2 * na + a], dx = -0.5 * rx * rx * g_rxp[a];
            IX2(grad_rho, iz, ix, nxt) += dx;
            IX2(grad_rho, iz, ix + 1, nxt) += dx;
        }
    if (misfit) *misfit = J;
    free(mzx); free(chk); free(seg); free(adj); free(we); free(gavg); free(recs);
    return 0;
}

/* ---------------------------------------------------------------------------
 * The reference's gradient of one shot (orc_forward with storage, then
 * orc_l2_adjoint_sources on the shot's receivers, then orc_adjoint) with the
 * forward wavefield held as full states every `interval` steps instead of the
 * whole storage: the backward restores the state at the start of each segment,
 * re-runs the segment's forward steps keeping their sampled window fields, and
 * runs the segment's adjoint steps from them.  The statements and their order
 * are those of the stored sequence, so the results are bit-identical; memory is
 * ceil(nt/interval) states plus interval frames of window samples (a config-3
 * shot: ~2.5 GB instead of 73 GB).
 * ------------------------------------------------------------------------- */
int orc_gradient_ckpt(int ishot, const orc_grid* g, const orc_medium* m, const orc_seis* src,
                      const double* src_signal, const orc_seis* rec, const double* obs, const double* res_in,
                      double* rec_signal, const orc_fwi* f, int interval, double* misfit, double* grad_lam,
                      double* grad_mu, double* grad_rho, double* we_fwd, double* we_adj) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!f || !f->fwinv || interval < 1) return -5;
    const int nxt = g->nxt, nt = g->nt;
    const st_sizes s = state_sizes(g);
    const int nseg = (nt + interval - 1) / interval;
    const int nfz = orc_nfz(f), nfx = orc_nfx(f);
    const size_t nf = (size_t)nfz * nfx;
    double* snaps = (double*)malloc((size_t)nseg * s.total * sizeof(double));
    double* work = (double*)calloc(s.total, sizeof(double));
    double* we = (double*)calloc(s.n, sizeof(double));
    double* seg = (double*)malloc((size_t)interval * 5 * nf * sizeof(double));
    double* ux = (double*)calloc(s.n, sizeof(double));
    double* uz = (double*)calloc(s.n, sizeof(double));
    double* adjst = (double*)calloc(s.total, sizeof(double));
    double* adjwe = (double*)calloc(s.n, sizeof(double));
    double* res = (double*)calloc((size_t)(rec ? rec->n : 0) * nt + 1, sizeof(double));
    if (!snaps || !work || !we || !seg || !ux || !uz || !adjst || !adjwe || !res) {
        free(snaps); free(work); free(we); free(seg); free(ux); free(uz); free(adjst); free(adjwe); free(res);
        return -4;
    }
    orc_wave w;
    wave_view(g, work, we, &w);
    /* forward sweep from rest: a state every `interval` steps, seismograms */
    for (int it = 0; it < nt; it++) {
        if (it % interval == 0) memcpy(snaps + (size_t)(it / interval) * s.total, work, s.total * sizeof(double));
        stress_pass(g, m, &w);
        velocity_pass(g, m, &w);
        for (int is = 0; src && is < src->n; is++)
            if (src->shot[is] == ishot && src->comp[is] == 2)
                IX2(w.vz, src->z[is], src->x[is], nxt) += src_signal[(size_t)is * nt + it];
        for (int ir = 0; rec && ir < rec->n; ir++)
            if (rec->shot[ir] == ishot && rec->comp[ir] == 2)
                rec_signal[(size_t)ir * nt + it] = IX2(w.vz, rec->z[ir], rec->x[ir], nxt);
    }
    if (we_fwd) memcpy(we_fwd, we, s.n * sizeof(double));
    /* residual and misfit of the shot's receivers (calculate_l2_adjoint_sources) */
    double J = 0.0;
    int blow = 0;
    for (int ir = 0; rec && ir < rec->n; ir++) {
        if (rec->shot[ir] != ishot || rec->comp[ir] != 2) continue;
        for (int it = 0; it < nt; it++) {
            size_t i = (size_t)ir * nt + it;
            double diff = rec_signal[i] - obs[i];
            J += 0.5 * g->dt * diff * diff;
            res[i] = res_in ? res_in[i] : diff;
            if (fabs(diff) > 1.0e+10) blow = 1;
        }
    }
    *misfit = J;
    /* backward: segments from the last one down, each recomputed from its state */
    orc_wave wa, wf;
    wave_view(g, adjst, adjwe, &wa);
    memset(grad_lam, 0, nf * sizeof(double));
    memset(grad_mu, 0, nf * sizeof(double));
    memset(grad_rho, 0, nf * sizeof(double));
    double* st[5];
    for (int q = 0; q < 5; q++) st[q] = seg + (size_t)q * interval * nf;
    for (int sgi = nseg - 1; sgi >= 0; sgi--) {
        const int t0 = sgi * interval, t1 = (t0 + interval < nt) ? t0 + interval : nt;
        memcpy(work, snaps + (size_t)sgi * s.total, s.total * sizeof(double));
        wave_view(g, work, we, &wf);
        for (int it = t0; it < t1; it++) {
            if (!(it % f->fwi_dt)) {
                const int fr = it - t0;
                for (int iz = f->z1; iz < f->z2; iz += f->fwi_dz) {
                    int zf = (iz - f->z1) / f->fwi_dz;
                    for (int ix = f->x1; ix < f->x2; ix += f->fwi_dx) {
                        int xf = (ix - f->x1) / f->fwi_dx;
                        size_t o = ((size_t)fr * nfz + zf) * nfx + xf, c = (size_t)iz * nxt + ix;
                        st[2][o] = wf.sxx[c];
                        st[3][o] = wf.szx[c];
                        st[4][o] = wf.szz[c];
                        st[0][o] = wf.vx[c] / g->dt;
                        st[1][o] = wf.vz[c] / g->dt;
                    }
                }
            }
            if (it + 1 < t1) fwd_step(g, m, &wf, it, ishot, src, src_signal);
        }
        const double* const cst[5] = {st[0], st[1], st[2], st[3], st[4]};
        for (int it = t1 - 1; it >= t0; it--)
            ref_adjoint_step(ishot, g, m, &wa, ux, uz, rec, res, f, cst, it, it - t0, grad_lam, grad_mu, grad_rho);
    }
    if (we_adj) memcpy(we_adj, adjwe, s.n * sizeof(double));
    free(snaps); free(work); free(we); free(seg); free(ux); free(uz); free(adjst); free(adjwe); free(res);
    return blow ? 1 : 0;
}
