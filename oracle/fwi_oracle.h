/*
 * fwi_oracle.h -- CPU restatement of the 2-D elastic P-SV FWI hot path (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: only tests/, the smoke
 * check and the CPU-baseline leg of bench.py may load it, and only as the
 * checker.  The product (libfwi_psv.so) never links or calls it.
 *
 * What it restates (reference = Mohammad-debug/CUDA_FWI, paths relative to the
 * reference project root):
 *   - Holberg coefficient table     CUDA_week2/holbergcoeff.cu:6-60
 *   - CPML coefficient profile      CUDA_week2/fd_cpml.cu:59-192
 *   - staggered material averages   CUDA_week2/fd_medium.cu:128-159
 *   - Ricker wavelet                CUDA_week2/fd_seismogram.cu:166-185
 *   - forward time loop             CUDA_week2/forward_kernel_PSV_GPU.cu:681-1085
 *   - adjoint loop + gradient       CUDA_week2/adjoint_kernel_PSV_GPU.cu:688-1102
 *   - L2 misfit / adjoint source    CUDA_week2/fd_wave_model.cu:972-1002
 *   - energy-weight preconditioning CUDA_week2/fd_wave_model.cu:1004-1052
 *   - bounded material update       CUDA_week2/fd_medium.cu:161-240
 *   - parabolic step fit            CUDA_week2/fwi_step_length_estimation.cu:226-271
 *
 * The reference implements only fdorder 2.  Orders 4..12 are this oracle's
 * generalisation: each one-sided difference becomes
 *   D+ f(i) = sum_k hc[k] (f[i+k]   - f[i-k+1]) / dx
 *   D- f(i) = sum_k hc[k] (f[i+k-1] - f[i-k]  ) / dx ,   k = 1..fdorder/2
 * which reduces to the reference's expressions (and its evaluation order) at
 * fdorder 2.  Parity at fdorder 2 is pinned against the reference's own CPU
 * functions compiled from its sources (oracle/build_ref.sh); at orders 4 and 8
 * the oracle is the FP64 restatement itself.
 *
 * Array layouts follow the reference: row-major [z][x] with padded extents
 * nzt x nxt for the wavefield, lam and mu; (nzt-1) x (nxt-1) for mu_zx,
 * rho_zp, rho_xp; CPML x-strips [nzt][2(npml+1)], z-strips [2(npml+1)][nxt];
 * FWI storage [nft][nfz][nfx]; gradients [nfz][nfx].
 */
#ifndef FWI_ORACLE_H
#define FWI_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PI 3.14159265 /* the reference's PI (CUDA_week2/globvar.cuh:18) */

typedef struct orc_grid {
    int nt, nzt, nxt, fpad, ppad, npml, fsurf, fdorder;
    double dt, dx, dz;
    double hc[7];
    /* CPML profiles, each 2*(npml+1) long */
    const double *a, *b, *K, *a_half, *b_half, *K_half;
} orc_grid;

typedef struct orc_medium {
    const double *lam, *mu;                /* [nzt][nxt]       */
    const double *mu_zx, *rho_zp, *rho_xp; /* [nzt-1][nxt-1]   */
} orc_medium;

typedef struct orc_wave {
    double *vx, *vz, *sxx, *szx, *szz, *We;           /* [nzt][nxt] */
    double *mem_vx_x, *mem_vz_x, *mem_sxx_x, *mem_szx_x; /* [nzt][2(npml+1)] */
    double *mem_vx_z, *mem_vz_z, *mem_szz_z, *mem_szx_z; /* [2(npml+1)][nxt] */
} orc_wave;

typedef struct orc_seis {
    int n;
    const int *x, *z, *comp, *shot; /* padded grid indices; comp 2 = vz */
} orc_seis;

typedef struct orc_fwi {
    int fwinv, fwi_dt, fwi_dx, fwi_dz, x1, x2, z1, z2;
    double *vx, *vz, *sxx, *szx, *szz; /* [nft][nfz][nfx] */
} orc_fwi;

int orc_nft(int nt, int fwi_dt);
int orc_nfz(const orc_fwi* f);
int orc_nfx(const orc_fwi* f);

/* holbergcoeff.cu:6-60.  Returns 0, or -1 for an order/error row outside the table. */
int orc_holberg(int fdorder, int max_rel_err, double hc[7]);

/* fd_cpml.cu:59-192.  Arrays are 2*(npml+1) long. */
void orc_cpml(int npml, double dh, double fpml, double npower, double k_max_pml, double rcoef,
              double damp_v_pml, double dt, double* a, double* b, double* K, double* a_half,
              double* b_half, double* K_half);

/* fd_medium.cu:128-159 over dimz = nzt-1, dimx = nxt-1 (input pitch nxt, output pitch nxt-1). */
void orc_average(int nzt, int nxt, const double* lam, const double* mu, const double* rho,
                 double* mu_zx, double* rho_zp, double* rho_xp);

/* fd_seismogram.cu:166-185 (shape 1 = Ricker; other shapes leave signal untouched). */
void orc_wavelet(double* signal, int nt, double dt, double amp, double fc, double ts, int shape);

/* fd_grid.cu:52-71 */
void orc_total_grid(int nx, int nz, int fdorder, int npml, int fsurf, int* fpad, int* ppad,
                    int* nxt, int* nzt);

/* forward_kernel_PSV_GPU.cu:681-1085 minus the CSV snapshot writer.  State, CPML
 * memory, We and storage are reset at entry exactly as the reference does. */
int orc_forward(int ishot, const orc_grid* g, const orc_medium* m, orc_wave* w,
                const orc_seis* src, const double* src_signal, /* [nsrc][nt] */
                const orc_seis* rec, double* rec_signal,       /* [nrec][nt] */
                orc_fwi* f);

/* adjoint_kernel_PSV_GPU.cu:688-1102.  adj_signal is the residual, injected at
 * the receiver positions (the reference passes the receivers as its sources). */
int orc_adjoint(int ishot, const orc_grid* g, const orc_medium* m, orc_wave* w,
                const orc_seis* adj, const double* adj_signal, const orc_fwi* f,
                double* grad_lam, double* grad_mu, double* grad_rho);

/* fd_wave_model.cu:972-1002: J = sum 0.5 dt (syn-obs)^2, syn <- syn-obs.
 * Returns 1 in *blowup when |diff| > 1e10 (the reference exits there). */
double orc_l2_adjoint_sources(int nr, int nt, double dt, double* signal, const double* signal_meas,
                              int* blowup);

/* fd_medium.cu:253-277 */
void orc_medium_average(int nzt, int nxt, const double* lam, const double* mu, const double* rho,
                        double* c_lam, double* c_mu, double* c_rho);

/* fd_wave_model.cu:1004-1052, including its mixed grid/sub-grid indexing.
 * Grads have pitch nfx; Ws, Wr have pitch nxt. */
void orc_scale_gradients(int nxt, const double* Ws, const double* Wr, double c_rho, double c_lam,
                         double c_mu, int nz, int nx, int z1, int x1, int fdz, int fdx,
                         int grad_pitch, double* grad_lam, double* grad_mu, double* grad_rho);

/* fd_medium.cu:161-240 with arrays of pitch `pitch` (mat) and `gpitch` (grad). */
void orc_grad_update(double* mat, double* mat_new, const double* grad, int pitch, int gpitch,
                     double step_length, int dimz, int dimx, int z1, int x1, int fwi_dz,
                     int fwi_dx, int override_, int mat_type);

/* fwi_step_length_estimation.cu:226-271 and solvelin.cu:6-42 (float temporaries kept). */
double orc_calc_opt_step(const double* L2, const double* sl);

/* Exact discrete adjoint of orc_forward's time stepping (no reference
 * counterpart): dJ/dlam, dJ/dmu, dJ/drho on the padded grid [nzt][nxt] of
 * J = sum_it sum_r 0.5 dt (rec_r(it) - obs_r(it))^2 over the receivers of
 * `ishot` (obs is [nrec][nt] in receiver order), with lam, mu, rho the raw
 * [nzt][nxt] models (the staggered averages are differentiated too).
 * Returns 0, a check_grid code, or -4 when out of memory. */
int orc_exact_gradient(int ishot, const orc_grid* g, const double* lam, const double* mu, const double* rho,
                       const orc_seis* src, const double* src_signal, const orc_seis* rec, const double* obs,
                       double* misfit, double* grad_lam, double* grad_mu, double* grad_rho);

/* Threads of the cell loops (OpenMP builds); returns the count in use. */
int orc_set_threads(int n);

/* orc_forward (storage) + orc_l2_adjoint_sources (the shot's receivers) +
 * orc_adjoint for one shot, bit-identical, with the forward wavefield kept as
 * a full state every `interval` steps and recomputed per segment.  f gives the
 * window (its storage pointers are not used); obs [nrec][nt]; res_in, when not
 * NULL, replaces the residual the adjoint injects ([nrec][nt], the shot's rows;
 * the misfit still comes from obs); writes
 * rec_signal [nrec][nt] (the shot's rows), *misfit, the gradients [nfz][nfx]
 * and, when not NULL, the forward and adjoint energy [nzt][nxt].  Returns 0,
 * 1 when |syn - obs| > 1e10 somewhere, < 0 on bad arguments or no memory. */
int orc_gradient_ckpt(int ishot, const orc_grid* g, const orc_medium* m, const orc_seis* src,
                      const double* src_signal, const orc_seis* rec, const double* obs, const double* res_in,
                      double* rec_signal, const orc_fwi* f, int interval, double* misfit, double* grad_lam,
                      double* grad_mu, double* grad_rho, double* we_fwd, double* we_adj);

#ifdef __cplusplus
}
#endif
#endif
