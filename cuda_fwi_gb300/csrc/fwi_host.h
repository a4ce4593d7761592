// fwi_host.h -- host-side building blocks shared by the C ABI and the engine.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace fwi {

// Thread-local detail message for fwi_psv_last_error().
void set_error(const std::string& msg);
const char* last_error();
int fail(int status, const std::string& msg);

// CUDA_week2/holbergcoeff.cu:6-60
int holberg(int fdorder, int max_rel_err, double hc[7]);
// CUDA_week2/fd_cpml.cu:59-192
void cpml_profile(int npml, double dh, double fpml, double npower, double kmax, double rcoef,
                  double damp, double dt, double* a, double* b, double* K, double* ah, double* bh,
                  double* Kh);
// CUDA_week2/fd_grid.cu:52-71
void total_grid(int nx, int nz, int fdorder, int npml, int fsurf, int* fpad, int* ppad, int* nxt,
                int* nzt);
// CUDA_week2/fd_seismogram.cu:166-185
void wavelet(double* s, int nt, double dt, double amp, double fc, double ts, int shape);
// CUDA_week2/fd_medium.cu:128-159 (outputs pitch nxt-1)
void average_parameters(int nzt, int nxt, const double* mu, const double* rho, double* mu_zx,
                        double* rho_zp, double* rho_xp);

// Binomial (Revolve-style) reversal schedule over n super-steps with s
// checkpoint slots.  Actions are executed in order by the engine.
struct Action {
    enum Kind : int { ADVANCE = 0, SAVE = 1, RESTORE = 2, ADJOINT = 3 } kind;
    int a, b;  // ADVANCE: state a -> b; SAVE/RESTORE: slot a holds state b; ADJOINT: super-step a
};
// Plan the reversal of super-steps [0, n) given that the working buffer starts
// at state 0 and state 0 can always be restored for free (it is all zeros).
// Returns the number of ADVANCE super-steps in *fwd_cost.
std::vector<Action> plan_binomial(int n, int slots, long long* fwd_cost);
// Minimal forward cost of reversing l super-steps with s free slots (DP-free closed form).
long long binomial_cost(int l, int s);

}  // namespace fwi
