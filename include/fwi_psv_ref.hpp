// fwi_psv_ref.hpp -- C++ drop-in declarations with the exact signatures of the
// reference's GPU propagators (Mohammad-debug/CUDA_FWI,
// CUDA_week2/fd_kernel.cuh:75-120 and :123-173).  A reference-style driver
// (CUDA_week2/fd_wave_model.cu) that includes its own fd_kernel.cuh links
// against libfwi_psv.so unchanged: the definitions live in
// cuda_fwi_gb300/csrc/fwi_refshim.cpp and run on the sm_103a engine.
//
// Semantics (the reference's CPU twin, which the shipped GPU code was meant to
// match): state, CPML memory and storage are reset at entry; host rec_signal
// rows of `ishot` and the host wavefield receive the results; the FP64 device
// buffers passed as d_* receive the final wavefield, d_We, the CPML memory and
// the FWI storage ([nft][nfz][nfx], velocities divided by dt), and the adjoint
// also fills d_grad_* and the host gradients.  Errors (a failed engine call or
// a failed copy into or out of the caller's d_* buffers) are printed to stderr,
// recorded for fwi_psv_last_error() and fwi_psv_ref_status(), and make the call
// return early (no exit()).
#pragma once

#include <vector>

using real_sim = double;
using ivec = std::vector<int>;

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
                            real_sim* d_rho_xp);

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
                            real_sim* d_rho_zp, real_sim* d_rho_xp);

// Status of the calling thread's last forward_kernel_PSV_GPU /
// adjoint_kernel_PSV_GPU call: FWI_OK (0) or an FWI_ERR_* code.  No counterpart
// in the reference (whose propagators exit() on a CUDA error,
// forward_kernel_PSV_GPU.cu:19-27); a reference-style driver that wants to
// react to errors calls it after each propagator call.
extern "C" int fwi_psv_ref_status(void);
