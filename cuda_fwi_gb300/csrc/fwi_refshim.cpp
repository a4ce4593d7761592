// fwi_refshim.cpp -- definitions of the reference's GPU propagator symbols
// (CUDA_week2/fd_kernel.cuh:75-173 of Mohammad-debug/CUDA_FWI) on top of the
// engine's flat C calls fwi_psv_forward_kernel / fwi_psv_adjoint_kernel.
// Host arrays arrive as the reference's contiguous row-pointer tables
// (CUDA_week2/util.cu:25-42), so p[0] is the flat buffer.
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include <string>

#include "../../include/fwi_psv.h"
#include "../../include/fwi_psv_ref.hpp"
#include "fwi_host.h"

namespace {

// Status of the calling thread's last drop-in call (the reference signatures
// return void; fwi_psv_ref_status() hands it to callers that want it).
thread_local int g_ref_status = FWI_OK;

double* flat(real_sim** p) { return p ? p[0] : nullptr; }
double* flat3(real_sim*** p) { return (p && p[0]) ? p[0][0] : nullptr; }

void report(int status, const char* where) {
    g_ref_status = status;
    if (status != FWI_OK)
        std::fprintf(stderr, "fwi_psv: %s failed: %s (%s)\n", where, fwi_psv_strerror(status),
                     fwi_psv_last_error());
}

// Copies between the caller's host arrays and its FP64 device buffers.  The
// first failing copy is recorded (fwi_psv_last_error, fwi_psv_ref_status) and
// every later copy of the same call is skipped.
struct Copier {
    const char* where;
    int status = FWI_OK;
    void run(double* dst, const double* src, size_t n, cudaMemcpyKind kind, const char* what) {
        if (status != FWI_OK || !dst || !src || !n) return;
        const cudaError_t e = cudaMemcpy(dst, src, n * sizeof(double), kind);
        if (e != cudaSuccess) {
            status = fwi::fail(FWI_ERR_CUDA, std::string(where) + ": copy of " + what + " " +
                                                 (kind == cudaMemcpyHostToDevice ? "to" : "from") +
                                                 " the device failed: " + cudaGetErrorString(e));
        }
    }
    void to_device(double* dst, const double* src, size_t n, const char* what) {
        run(dst, src, n, cudaMemcpyHostToDevice, what);
    }
    void from_device(double* dst, const double* src, size_t n, const char* what) {
        run(dst, src, n, cudaMemcpyDeviceToHost, what);
    }
};

struct Sizes {
    size_t cells, xs, zs, store;
    Sizes(int nt, int nzt, int nxt, int npml, bool fwinv, int fdt, int fdx, int fdz, int x1, int x2,
          int z1, int z2) {
        const size_t tp = 2 * (size_t)(npml + 1);
        cells = (size_t)nzt * nxt;
        xs = (size_t)nzt * tp;
        zs = tp * (size_t)nxt;
        store = 0;
        if (fwinv && fdt > 0 && fdx > 0 && fdz > 0)
            store = (size_t)(1 + (nt - 1) / fdt) * (1 + (z2 - z1) / fdz) * (1 + (x2 - x1) / fdx);
    }
};

}  // namespace

void forward_kernel_PSV_GPU(int ishot, int nt, int nzt, int nxt, int fpad, int ppad, real_sim dt,
                            real_sim dx, real_sim dz, int snap_interval, bool fsurf, real_sim* hc,
                            int fdorder, real_sim** vx, real_sim** vz, real_sim** sxx,
                            real_sim** szx, real_sim** szz, real_sim** lam, real_sim** mu,
                            real_sim** mu_zx, real_sim** rho_zp, real_sim** rho_xp, int npml,
                            real_sim* a, real_sim* b, real_sim* K, real_sim* a_half,
                            real_sim* b_half, real_sim* K_half, real_sim** mem_vx_x,
                            real_sim** mem_vx_z, real_sim** mem_vz_x, real_sim** mem_vz_z,
                            real_sim** mem_sxx_x, real_sim** mem_szx_x, real_sim** mem_szz_z,
                            real_sim** mem_szx_z, int nsrc, ivec src_x, ivec src_z,
                            ivec src_comp, real_sim** src_signal, ivec source_to_fire_shot,
                            int nrec, ivec rec_x, ivec rec_z, ivec rec_comp,
                            real_sim** rec_signal, ivec receiver_to_record_shot, bool fwinv,
                            int fwi_dt, int fwi_dx, int fwi_dz, int fwi_x1, int fwi_x2,
                            int fwi_z1, int fwi_z2, real_sim*** fwi_vx, real_sim*** fwi_vz,
                            real_sim*** fwi_sxx, real_sim*** fwi_szx, real_sim*** fwi_szz,
                            real_sim* d_a, real_sim* d_b, real_sim* d_K, real_sim* d_a_half,
                            real_sim* d_b_half, real_sim* d_K_half, real_sim* d_vx,
                            real_sim* d_vz, real_sim* d_sxx, real_sim* d_szx, real_sim* d_szz,
                            real_sim* d_We, real_sim* d_fwi_vx, real_sim* d_fwi_vz,
                            real_sim* d_fwi_sxx, real_sim* d_fwi_szx, real_sim* d_fwi_szz,
                            real_sim* d_mem_vx_x, real_sim* d_mem_vx_z, real_sim* d_mem_vz_x,
                            real_sim* d_mem_vz_z, real_sim* d_mem_sxx_x, real_sim* d_mem_szx_x,
                            real_sim* d_mem_szz_z, real_sim* d_mem_szx_z, real_sim* d_lam,
                            real_sim* d_mu, real_sim* d_mu_zx, real_sim* d_rho_zp,
                            real_sim* d_rho_xp) {
    (void)d_a; (void)d_b; (void)d_K; (void)d_a_half; (void)d_b_half; (void)d_K_half;
    (void)d_lam; (void)d_mu; (void)d_mu_zx; (void)d_rho_zp; (void)d_rho_xp;
    const Sizes S(nt, nzt, nxt, npml, fwinv, fwi_dt, fwi_dx, fwi_dz, fwi_x1, fwi_x2, fwi_z1, fwi_z2);
    std::vector<double> we(S.cells);
    // The shipped GPU driver leaves the host FWI storage unallocated
    // (fd_wave_model.cu:292); fall back to temporaries for the device copy.
    std::vector<double> tmp;
    double* st[5] = {flat3(fwi_vx), flat3(fwi_vz), flat3(fwi_sxx), flat3(fwi_szx), flat3(fwi_szz)};
    if (fwinv && !(st[0] && st[1] && st[2] && st[3] && st[4])) {
        tmp.assign(5 * S.store, 0.0);
        for (int q = 0; q < 5; q++) st[q] = tmp.data() + q * S.store;
    }
    const int rc = fwi_psv_forward_kernel(
        ishot, nt, nzt, nxt, fpad, ppad, dt, dx, dz, snap_interval, fsurf ? 1 : 0, hc, fdorder,
        flat(vx), flat(vz), flat(sxx), flat(szx), flat(szz), we.data(), flat(lam), flat(mu),
        flat(mu_zx), flat(rho_zp), flat(rho_xp), npml, a, b, K, a_half, b_half, K_half,
        flat(mem_vx_x), flat(mem_vx_z), flat(mem_vz_x), flat(mem_vz_z), flat(mem_sxx_x),
        flat(mem_szx_x), flat(mem_szz_z), flat(mem_szx_z), nsrc, src_x.data(), src_z.data(),
        src_comp.data(), flat(src_signal), source_to_fire_shot.data(), nrec, rec_x.data(),
        rec_z.data(), rec_comp.data(), flat(rec_signal), receiver_to_record_shot.data(),
        fwinv ? 1 : 0, fwi_dt, fwi_dx, fwi_dz, fwi_x1, fwi_x2, fwi_z1, fwi_z2, st[0], st[1], st[2],
        st[3], st[4]);
    report(rc, "forward_kernel_PSV_GPU");
    if (rc != FWI_OK) return;
    Copier c{"forward_kernel_PSV_GPU"};
    c.to_device(d_vx, flat(vx), S.cells, "vx");
    c.to_device(d_vz, flat(vz), S.cells, "vz");
    c.to_device(d_sxx, flat(sxx), S.cells, "sxx");
    c.to_device(d_szx, flat(szx), S.cells, "szx");
    c.to_device(d_szz, flat(szz), S.cells, "szz");
    c.to_device(d_We, we.data(), S.cells, "We");
    c.to_device(d_mem_vx_x, flat(mem_vx_x), S.xs, "mem_vx_x");
    c.to_device(d_mem_vz_x, flat(mem_vz_x), S.xs, "mem_vz_x");
    c.to_device(d_mem_sxx_x, flat(mem_sxx_x), S.xs, "mem_sxx_x");
    c.to_device(d_mem_szx_x, flat(mem_szx_x), S.xs, "mem_szx_x");
    c.to_device(d_mem_vx_z, flat(mem_vx_z), S.zs, "mem_vx_z");
    c.to_device(d_mem_vz_z, flat(mem_vz_z), S.zs, "mem_vz_z");
    c.to_device(d_mem_szz_z, flat(mem_szz_z), S.zs, "mem_szz_z");
    c.to_device(d_mem_szx_z, flat(mem_szx_z), S.zs, "mem_szx_z");
    if (fwinv) {
        c.to_device(d_fwi_vx, st[0], S.store, "fwi_vx");
        c.to_device(d_fwi_vz, st[1], S.store, "fwi_vz");
        c.to_device(d_fwi_sxx, st[2], S.store, "fwi_sxx");
        c.to_device(d_fwi_szx, st[3], S.store, "fwi_szx");
        c.to_device(d_fwi_szz, st[4], S.store, "fwi_szz");
    }
    report(c.status, "forward_kernel_PSV_GPU");
}

void adjoint_kernel_PSV_GPU(int ishot, int nt, int nzt, int nxt, int fpad, int ppad, real_sim dt,
                            real_sim dx, real_sim dz, int snap_interval, bool fsurf, real_sim* hc,
                            int fdorder, real_sim** vx, real_sim** vz, real_sim** sxx,
                            real_sim** szx, real_sim** szz, real_sim** lam, real_sim** mu,
                            real_sim** mu_zx, real_sim** rho_zp, real_sim** rho_xp, int npml,
                            real_sim* a, real_sim* b, real_sim* K, real_sim* a_half,
                            real_sim* b_half, real_sim* K_half, real_sim** mem_vx_x,
                            real_sim** mem_vx_z, real_sim** mem_vz_x, real_sim** mem_vz_z,
                            real_sim** mem_sxx_x, real_sim** mem_szx_x, real_sim** mem_szz_z,
                            real_sim** mem_szx_z, int nsrc, ivec src_x, ivec src_z,
                            ivec src_comp, real_sim** src_signal, ivec source_to_fire_shot,
                            bool fwinv, int fwi_dt, int fwi_dx, int fwi_dz, int fwi_x1,
                            int fwi_x2, int fwi_z1, int fwi_z2, real_sim*** fwi_vx,
                            real_sim*** fwi_vz, real_sim*** fwi_sxx, real_sim*** fwi_szx,
                            real_sim*** fwi_szz, real_sim** grad_lam, real_sim** grad_mu,
                            real_sim** grad_rho, real_sim* d_a, real_sim* d_b, real_sim* d_K,
                            real_sim* d_a_half, real_sim* d_b_half, real_sim* d_K_half,
                            real_sim* d_vx, real_sim* d_vz, real_sim* d_sxx, real_sim* d_szx,
                            real_sim* d_szz, real_sim* d_We, real_sim* d_fwi_vx,
                            real_sim* d_fwi_vz, real_sim* d_fwi_sxx, real_sim* d_fwi_szx,
                            real_sim* d_fwi_szz, real_sim* d_mem_vx_x, real_sim* d_mem_vx_z,
                            real_sim* d_mem_vz_x, real_sim* d_mem_vz_z, real_sim* d_mem_sxx_x,
                            real_sim* d_mem_szx_x, real_sim* d_mem_szz_z, real_sim* d_mem_szx_z,
                            real_sim* d_grad_lam, real_sim* d_grad_mu, real_sim* d_grad_rho,
                            real_sim* d_lam, real_sim* d_mu, real_sim* d_mu_zx,
                            real_sim* d_rho_zp, real_sim* d_rho_xp) {
    (void)d_a; (void)d_b; (void)d_K; (void)d_a_half; (void)d_b_half; (void)d_K_half;
    (void)d_lam; (void)d_mu; (void)d_mu_zx; (void)d_rho_zp; (void)d_rho_xp;
    const Sizes S(nt, nzt, nxt, npml, fwinv, fwi_dt, fwi_dx, fwi_dz, fwi_x1, fwi_x2, fwi_z1, fwi_z2);
    const size_t ng = fwinv ? (size_t)(1 + (fwi_z2 - fwi_z1) / fwi_dz) * (1 + (fwi_x2 - fwi_x1) / fwi_dx) : 0;
    // Forward storage: the device copy written by forward_kernel_PSV_GPU when
    // given, else the host arrays.
    std::vector<double> tmp;
    double* st[5] = {flat3(fwi_vx), flat3(fwi_vz), flat3(fwi_sxx), flat3(fwi_szx), flat3(fwi_szz)};
    double* dst[5] = {d_fwi_vx, d_fwi_vz, d_fwi_sxx, d_fwi_szx, d_fwi_szz};
    Copier in{"adjoint_kernel_PSV_GPU"};
    if (fwinv && dst[0] && dst[1] && dst[2] && dst[3] && dst[4]) {
        tmp.assign(5 * S.store, 0.0);
        static const char* names[5] = {"d_fwi_vx", "d_fwi_vz", "d_fwi_sxx", "d_fwi_szx", "d_fwi_szz"};
        for (int q = 0; q < 5; q++) {
            st[q] = tmp.data() + q * S.store;
            in.from_device(st[q], dst[q], S.store, names[q]);
        }
    }
    if (in.status != FWI_OK) {
        report(in.status, "adjoint_kernel_PSV_GPU");
        return;
    }
    std::vector<double> we(S.cells), gtmp;
    double* g[3] = {flat(grad_lam), flat(grad_mu), flat(grad_rho)};
    if (!(g[0] && g[1] && g[2])) {
        gtmp.assign(3 * std::max<size_t>(ng, 1), 0.0);
        for (int q = 0; q < 3; q++) g[q] = gtmp.data() + q * std::max<size_t>(ng, 1);
    }
    const int rc = fwi_psv_adjoint_kernel(
        ishot, nt, nzt, nxt, fpad, ppad, dt, dx, dz, snap_interval, fsurf ? 1 : 0, hc, fdorder,
        flat(vx), flat(vz), flat(sxx), flat(szx), flat(szz), we.data(), flat(lam), flat(mu),
        flat(mu_zx), flat(rho_zp), flat(rho_xp), npml, a, b, K, a_half, b_half, K_half,
        flat(mem_vx_x), flat(mem_vx_z), flat(mem_vz_x), flat(mem_vz_z), flat(mem_sxx_x),
        flat(mem_szx_x), flat(mem_szz_z), flat(mem_szx_z), nsrc, src_x.data(), src_z.data(),
        src_comp.data(), flat(src_signal), source_to_fire_shot.data(), fwinv ? 1 : 0, fwi_dt,
        fwi_dx, fwi_dz, fwi_x1, fwi_x2, fwi_z1, fwi_z2, st[0], st[1], st[2], st[3], st[4], g[0],
        g[1], g[2]);
    report(rc, "adjoint_kernel_PSV_GPU");
    if (rc != FWI_OK) return;
    Copier c{"adjoint_kernel_PSV_GPU"};
    c.to_device(d_vx, flat(vx), S.cells, "vx");
    c.to_device(d_vz, flat(vz), S.cells, "vz");
    c.to_device(d_sxx, flat(sxx), S.cells, "sxx");
    c.to_device(d_szx, flat(szx), S.cells, "szx");
    c.to_device(d_szz, flat(szz), S.cells, "szz");
    c.to_device(d_We, we.data(), S.cells, "We");
    c.to_device(d_mem_vx_x, flat(mem_vx_x), S.xs, "mem_vx_x");
    c.to_device(d_mem_vz_x, flat(mem_vz_x), S.xs, "mem_vz_x");
    c.to_device(d_mem_sxx_x, flat(mem_sxx_x), S.xs, "mem_sxx_x");
    c.to_device(d_mem_szx_x, flat(mem_szx_x), S.xs, "mem_szx_x");
    c.to_device(d_mem_vx_z, flat(mem_vx_z), S.zs, "mem_vx_z");
    c.to_device(d_mem_vz_z, flat(mem_vz_z), S.zs, "mem_vz_z");
    c.to_device(d_mem_szz_z, flat(mem_szz_z), S.zs, "mem_szz_z");
    c.to_device(d_mem_szx_z, flat(mem_szx_z), S.zs, "mem_szx_z");
    c.to_device(d_grad_lam, g[0], ng, "grad_lam");
    c.to_device(d_grad_mu, g[1], ng, "grad_mu");
    c.to_device(d_grad_rho, g[2], ng, "grad_rho");
    report(c.status, "adjoint_kernel_PSV_GPU");
}

extern "C" int fwi_psv_ref_status(void) { return g_ref_status; }
