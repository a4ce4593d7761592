// fwi_host.cpp -- host-side setup of the FWI hot path (FP64) and the binomial
// checkpoint planner.  Formulas follow the reference (Mohammad-debug/CUDA_FWI,
// paths relative to its root) as cited per function.
#include "fwi_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/fwi_psv.h"

namespace fwi {

namespace {
thread_local std::string g_last_error;
constexpr double kPi = 3.14159265;  // the reference's PI (CUDA_week2/globvar.cuh:18)
}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }
int fail(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

// Holberg (1987) staggered-grid coefficients; rows: max relative error index
// 0..4 (0 = Taylor); columns: fdorder 2..12; entry 0 = the table's accuracy
// figure, 1..6 = coefficients.  The values are the published table that
// CUDA_week2/holbergcoeff.cu:10-52 also carries.
static const double kHolberg[5][6][7] = {
    {{23.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0},
     {8.0, 9.0 / 8.0, -1.0 / 24.0, 0.0, 0.0, 0.0, 0.0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0.0, 0.0, 0.0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0.0, 0.0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0,
      35.0 / 294912.0, 0.0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0, -5445.0 / 1835008.0,
      847.0 / 2359296.0, -63.0 / 2883584.0}},
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

int holberg(int fdorder, int max_rel_err, double hc[7]) {
    if (fdorder < 2 || fdorder > 12 || (fdorder & 1))
        return fail(FWI_ERR_INVALID, "fdorder must be even and in 2..12");
    if (max_rel_err < 0 || max_rel_err > 4)
        return fail(FWI_ERR_INVALID, "max_relative_error must be in 0..4");
    std::memcpy(hc, kHolberg[max_rel_err][fdorder / 2 - 1], 7 * sizeof(double));
    return FWI_OK;
}

// Damping d, stretch K and frequency shift alpha at a depth `dist` into a layer
// of thickness `thick` (negative = outside); fd_cpml.cu:95-114 for both sides.
static void cpml_point(double dist, double thick, double d0, double npower, double kmax,
                       double amax, double* d, double* K, double* alpha) {
    *d = 0.0;
    *alpha = 0.0;
    if (dist >= 0) {
        const double xn = dist / thick;
        *d = d0 * std::pow(xn, npower);
        *K = 1.0 + (kmax - 1.0) * std::pow(xn, npower);
        *alpha = amax * (1.0 - xn);
    }
    if (*alpha < 0.0) *alpha = 0.0;
}

void cpml_profile(int npml, double dh, double fpml, double npower, double kmax, double rcoef,
                  double damp, double dt, double* a, double* b, double* K, double* ah, double* bh,
                  double* Kh) {
    const double amax = 2.0 * kPi * (fpml / 2.0);
    const double thick = npml * dh;
    const double d0 = -(npower + 1) * damp * std::log(rcoef) / (2.0 * thick);
    const int n = 2 * (npml + 1);
    for (int i = 0; i < n; i++) {
        a[i] = ah[i] = 0.0;
        b[i] = bh[i] = 1.0;
        K[i] = Kh[i] = 1.0;
        const double x = dh * double(i);
        // left layer counts inwards from the outer edge, right layer outwards
        // from dh*(npml+1) (fd_cpml.cu:92-93 and :138-139)
        const double dist = i <= npml ? thick - x : x - dh * (npml + 1);
        const double dist_h = i <= npml ? thick - (x + dh / 2.0) : (x + dh / 2.0) - dh * (npml + 1);
        double d, al, dhh, alh;
        cpml_point(dist, thick, d0, npower, kmax, amax, &d, &K[i], &al);
        cpml_point(dist_h, thick, d0, npower, kmax, amax, &dhh, &Kh[i], &alh);
        b[i] = std::exp(-(d / K[i] + al) * dt);
        bh[i] = std::exp(-(dhh / Kh[i] + alh) * dt);
        if (std::fabs(d) > 1.0e-6) a[i] = d * (b[i] - 1.0) / (K[i] * (d + K[i] * al));
        if (std::fabs(dhh) > 1.0e-6) ah[i] = dhh * (bh[i] - 1.0) / (Kh[i] * (dhh + Kh[i] * alh));
    }
}

void total_grid(int nx, int nz, int fdorder, int npml, int fsurf, int* fpad, int* ppad, int* nxt,
                int* nzt) {
    *fpad = fdorder / 2;
    *ppad = npml + *fpad;
    *nxt = nx + 2 * *ppad;
    *nzt = fsurf ? nz + *ppad + *fpad : nz + 2 * *ppad;
}

void wavelet(double* s, int nt, double dt, double amp, double fc, double ts, int shape) {
    if (shape != 1) return;  // only the Ricker shape exists in the reference
    const double fci = 1.0 / fc;
    for (int it = 0; it < nt; it++) {
        const double tau = kPi * (it * dt - 1.5 * fci - ts) / (1.5 * fci);
        s[it] = amp * (1.0 - 2.0 * tau * tau) * std::exp(-2.0 * tau * tau);
    }
}

void average_parameters(int nzt, int nxt, const double* mu, const double* rho, double* mu_zx,
                        double* rho_zp, double* rho_xp) {
    const int pz = nzt - 1, px = nxt - 1;
    for (int iz = 0; iz < pz; iz++) {
        const double* m0 = mu + (size_t)iz * nxt;
        const double* m1 = m0 + nxt;
        const double* r0 = rho + (size_t)iz * nxt;
        const double* r1 = r0 + nxt;
        for (int ix = 0; ix < px; ix++) {
            const size_t o = (size_t)iz * px + ix;
            const bool zero = m0[ix] == 0.0 || m0[ix + 1] == 0.0 || m1[ix] == 0.0 || m1[ix + 1] == 0.0;
            mu_zx[o] = zero ? 0.0
                            : 4.0 / ((1.0 / m0[ix]) + (1.0 / m0[ix + 1]) + (1.0 / m1[ix]) +
                                     (1.0 / m1[ix + 1]));
            rho_zp[o] = 1.0 / (0.5 * (r0[ix] + r1[ix]));
            rho_xp[o] = 1.0 / (0.5 * (r0[ix] + r0[ix + 1]));
            // Near-void guards; the second one writes rho_zp too, as the
            // reference does (fd_medium.cu:148-154).
            if (r0[ix] < 1e-4 && r1[ix] < 1e-4) rho_zp[o] = 0.0;
            if (r0[ix] < 1e-4 && r0[ix + 1] < 1e-4) rho_zp[o] = 0.0;
        }
    }
}

// ---------------------------------------------------------------------------
// Binomial checkpointing.  beta(S, r) = C(S + r, S) is the longest chain that
// S stored states (the segment start included) reverse with r sweeps; the
// minimal number of forward steps to reverse l steps is
//   r*l - beta(S+1, r-1),  beta(S, r-1) < l <= beta(S, r)
// (Griewank & Walther, "Algorithm 799: revolve", ACM TOMS 26(1), 2000).
// ---------------------------------------------------------------------------
static long long beta(int S, int r) {
    if (r < 0) return 0;
    long double v = 1.0L;  // C(S + r, r), saturated
    for (int i = 1; i <= r; i++) {
        v = v * (long double)(S + i) / (long double)i;
        if (v > 4.0e18L) return (long long)4e18;
    }
    return (long long)(v + 0.5L);
}

long long binomial_cost(int l, int s) {
    if (l <= 1) return 0;
    const int S = s + 1;
    if (s == 0) return (long long)l * (l - 1) / 2;
    int r = 0;
    while (beta(S, r) < l) r++;
    return (long long)r * l - beta(S + 1, r - 1);
}

namespace {
struct Planner {
    std::vector<Action> out;
    long long cost = 0;
    std::vector<int> free_slots;
    int working = 0;  // state held by the working buffer
    void advance(int a, int b) {
        if (b > a) {
            out.push_back({Action::ADVANCE, a, b});
            cost += b - a;
        }
        working = b;
    }
    void restore(int slot, int state) {
        if (working != state) out.push_back({Action::RESTORE, slot, state});
        working = state;
    }
    // Reverse [a, b): the state a is held in `slot` (-1: zero state) and is in
    // the working buffer; s free slots remain.
    void rev(int a, int b, int slot, int s) {
        const int l = b - a;
        if (l == 1) {
            restore(slot, a);
            out.push_back({Action::ADJOINT, a, 0});
            return;
        }
        if (s == 0) {
            for (int i = b - 1; i >= a; i--) {
                restore(slot, a);
                advance(a, i);
                out.push_back({Action::ADJOINT, i, 0});
            }
            return;
        }
        const long long best = binomial_cost(l, s);
        const int S = s + 1;
        int r = 0;
        while (beta(S, r) < l) r++;
        int j = std::max<long long>(1, (long long)l - beta(S - 1, r));
        for (; j < l; j++)
            if (j + binomial_cost(l - j, s - 1) + binomial_cost(j, s) == best) break;
        if (j >= l) j = 1;
        const int m = a + j;
        restore(slot, a);
        advance(a, m);
        const int ms = free_slots.back();
        free_slots.pop_back();
        out.push_back({Action::SAVE, ms, m});
        rev(m, b, ms, s - 1);
        free_slots.push_back(ms);
        restore(slot, a);
        rev(a, m, slot, s);
    }
};
}  // namespace

std::vector<Action> plan_binomial(int n, int slots, long long* fwd_cost) {
    Planner p;
    for (int i = slots - 1; i >= 0; i--) p.free_slots.push_back(i);
    if (n > 0) p.rev(0, n, -1, slots);
    if (fwd_cost) *fwd_cost = p.cost;
    return p.out;
}

}  // namespace fwi
