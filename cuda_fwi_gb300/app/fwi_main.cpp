// fwi_main.cpp -- the reference's INI-driven program on the GB300 engine.
//
//   fwi_run CONFIG.ini [--out DIR] [--device N] [--batch N] [--dry-run]
//
// Mirrors Mohammad-debug/CUDA_FWI's main (CUDA_week2/main.cu) and
// FDWaveModel (fd_wave_model.cu:33-75): read [FDM], [grid], [medium],
// [PML_boundary], [source], [receiver] and [full_waveform_inversion], pad the
// grid (fd_grid.cu:52-71), place the seismograms on it (fd_seismogram.cu
// :153-163), build the CPML profile (fd_cpml.cu:59-192) and the Holberg
// coefficients, then either
//   forward modelling (full_waveform_inversion = 0, fd_wave_model.cu:133-230):
//     the homogeneous medium with the reference's stiffer circle
//     (fd_medium.cu:80-101), all shots run together, receiver traces to
//     io/receiver/rec_signal.csv and szz snapshots every snap_interval steps to
//     io/snap_data/vz_snap<k>.csv (the reference's file name; the last shot's);
//   full waveform inversion (= 1, fd_wave_model.cu:232-955): from the
//     homogeneous medium, fwi_psv_fwi_run one iteration at a time, models to
//     io/density_snap/{density,lam,mu}_snap<iter>.csv after each iteration.
// Files are written as the reference writes them ("value, " per sample, one
// line per row, default ostream formatting).
//
// Differences, each stated at its place below: observed data are read from
// [receiver] signal_file when measurement_records = 1 (the reference
// allocates them and never fills them); the FWI window is clipped to the
// padded grid (its defaults reach past it); missing per-seismogram entries of
// a vector repeat its last entry (the reference reads past the vector); a
// failed step-length search or an unconverged loop returns status 1 as the
// reference's exit codes do, after writing the outputs.  Keys the reference
// does not have: [FDM] fwi_order = per_shot|summed, trial_misfit =
// last_shot|sum (defaults: the reference's behaviour), checkpoints (binomial
// slots per shot, 0 = as memory allows); [medium] lam_file, mu_file, rho_file
// (CSV models [nzt][nxt] replacing the homogeneous medium).
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "fwi_psv.h"
#include "ini.hpp"

namespace {

struct Seis {
    std::vector<int> x, z, comp, shot;
    std::vector<double> signal;  // sources: [n][nt]
};

struct Config {
    // [FDM]
    int fdorder = 2, max_rel_err = 1, fwinv = 0, nshots = 1, max_iter = 500;
    double max_error = 1.0e-3;
    int order = FWI_ORDER_PER_SHOT, trial = FWI_TRIAL_LAST_SHOT, checkpoints = 0;
    // [grid]
    int nx = 201, nz = 101, nt = 0, snap_interval = 0, fsurf = 0;
    double dx = 1.25, dz = 1.25, dt = 0.00025;
    // [medium]
    double rho = 0.0, vp = 0.0, vs = 0.0;
    std::string lam_file, mu_file, rho_file;
    // [PML_boundary]
    int npml = 10;
    double dh = 0.1, fpml = 20.0, npower = 2.0, kmax = 1.0, rcoef = 0.001, damp = 0.0;
    // derived grid
    int fpad = 0, ppad = 0, nxt = 0, nzt = 0;
    double hc[7] = {0, 0, 0, 0, 0, 0, 0};
    std::vector<double> a, b, K, ah, bh, Kh;
    Seis src, rec;
    int measurement = 0;
    std::string obs_file;
    // [full_waveform_inversion]
    int fdt = 1, fdx = 1, fdz = 1, x1 = 0, x2 = 0, z1 = 0, z2 = 0;
};

int fail(const std::string& msg) {
    std::cerr << "fwi_run: " << msg << std::endl;
    return 2;
}

int check(int st, const char* where) {
    if (st != FWI_OK) std::cerr << "fwi_run: " << where << ": " << fwi_psv_last_error() << std::endl;
    return st;
}

std::vector<int> ints(const std::vector<double>& v, int n) {
    std::vector<int> out(n);
    for (int i = 0; i < n; i++) out[i] = (int)(i < (int)v.size() ? v[i] : v.back());
    return out;
}
std::vector<double> reals(const std::vector<double>& v, int n) {
    std::vector<double> out(n);
    for (int i = 0; i < n; i++) out[i] = i < (int)v.size() ? v[i] : v.back();
    return out;
}

int load(const char* path, Config& c) {
    IniFile ini(path);
    if (ini.ParseError() < 0) return fail(std::string("can't load ") + path);
    c.fdorder = (int)ini.GetInteger("FDM", "fdorder", 2);
    c.max_rel_err = (int)ini.GetInteger("FDM", "max_relative_error", 1);
    c.fwinv = (int)ini.GetInteger("FDM", "full_waveform_inversion", 0);
    c.nshots = (int)ini.GetInteger("FDM", "nshots", 1);
    c.max_iter = (int)ini.GetInteger("FDM", "max_iteration", 500);
    c.max_error = ini.GetReal("FDM", "max_error", 1.0e-3);
    const std::string ord = ini.Get("FDM", "fwi_order", "per_shot");
    c.order = ord.rfind("summed", 0) == 0 ? FWI_ORDER_SUMMED : FWI_ORDER_PER_SHOT;
    const std::string tr = ini.Get("FDM", "trial_misfit", "last_shot");
    c.trial = tr.rfind("sum", 0) == 0 ? FWI_TRIAL_SUM : FWI_TRIAL_LAST_SHOT;
    c.checkpoints = (int)ini.GetInteger("FDM", "checkpoints", 0);
    // [grid] (fd_grid.cu:25-45)
    const double t = ini.GetReal("grid", "time", 0);
    c.nx = (int)ini.GetInteger("grid", "nx", 201);
    c.nz = (int)ini.GetInteger("grid", "nz", 101);
    c.dx = ini.GetReal("grid", "dx", 1.25);
    c.dz = ini.GetReal("grid", "dz", 1.25);
    c.dt = ini.GetReal("grid", "dt", 0.00025);
    c.nt = (int)ini.GetInteger("grid", "nt", (long)std::ceil(t / c.dt));
    c.snap_interval = (int)ini.GetInteger("grid", "snap_interval", c.nt - 1);
    c.fsurf = (int)ini.GetInteger("grid", "free_surface", 0);
    // [medium] (fd_medium.cu:37-52)
    c.rho = ini.GetReal("medium", "scalar_rho", 0.0);
    c.vp = ini.GetReal("medium", "scalar_vp", 0.0);
    c.vs = ini.GetReal("medium", "scalar_vs", 0.0);
    c.lam_file = ini.Get("medium", "lam_file", "");
    c.mu_file = ini.Get("medium", "mu_file", "");
    c.rho_file = ini.Get("medium", "rho_file", "");
    // [PML_boundary] (fd_cpml.cu:33-47)
    c.npml = (int)ini.GetInteger("PML_boundary", "npml", 10);
    c.dh = ini.GetReal("PML_boundary", "dh", 0.1);
    c.fpml = ini.GetReal("PML_boundary", "fpml", 20.0);
    c.npower = ini.GetReal("PML_boundary", "npower", 2.0);
    c.kmax = ini.GetReal("PML_boundary", "k_max_PML", 1.0);
    c.rcoef = ini.GetReal("PML_boundary", "rcoef", 0.001);
    c.damp = ini.GetReal("PML_boundary", "damp_v_PML", 0.0);
    if (c.nt < 1) return fail("nt must be >= 1");
    if (check(fwi_psv_total_grid(c.nx, c.nz, c.fdorder, c.npml, c.fsurf, &c.fpad, &c.ppad, &c.nxt, &c.nzt),
              "total_grid"))
        return 2;
    if (check(fwi_psv_holberg(c.fdorder, c.max_rel_err, c.hc), "holberg")) return 2;
    const int tp = 2 * (c.npml + 1);
    for (auto* v : {&c.a, &c.b, &c.K, &c.ah, &c.bh, &c.Kh}) v->assign(tp, 0.0);
    if (c.npml > 0 && check(fwi_psv_cpml_profile(c.npml, c.dh, c.fpml, c.npower, c.kmax, c.rcoef, c.damp, c.dt,
                                                 c.a.data(), c.b.data(), c.K.data(), c.ah.data(), c.bh.data(),
                                                 c.Kh.data()),
                            "cpml_profile"))
        return 2;
    // seismograms (fd_seismogram.cu:40-150); positions moved onto the padded
    // grid (:153-163); vectors shorter than nseis repeat their last entry
    const int zoff = c.fsurf ? c.fpad : c.ppad;
    for (int sr = 0; sr < 2; sr++) {
        const char* sec = sr ? "receiver" : "source";
        Seis& s = sr ? c.rec : c.src;
        const int n = (int)ini.GetInteger(sec, "nseis", 1);
        s.x = ints(ini.GetVector(sec, "x_seis", "{0};"), n);
        s.z = ints(ini.GetVector(sec, "z_seis", "{0};"), n);
        s.comp = ints(ini.GetVector(sec, "component_type", "{0};"), n);
        s.shot = ints(ini.GetVector(sec, "shot_to_fire", "{0};"), n);
        for (int i = 0; i < n; i++) {
            s.x[i] += c.ppad;
            s.z[i] += zoff;
        }
        if (!sr) {
            const auto shape = ints(ini.GetVector(sec, "shape", "{0};"), n);
            const auto amp = reals(ini.GetVector(sec, "amplitude", "{0.0};"), n);
            const auto fc = reals(ini.GetVector(sec, "peak_frequency", "{0.0};"), n);
            const auto ts = reals(ini.GetVector(sec, "time_shift", "{0.0};"), n);
            // create_wavelet (fd_seismogram.cu:166-185) fills shape 1 (Ricker)
            // only; other shapes leave the signal at zero
            s.signal.assign((size_t)n * c.nt, 0.0);
            for (int i = 0; i < n; i++)
                if (shape[i] == 1 &&
                    check(fwi_psv_wavelet(s.signal.data() + (size_t)i * c.nt, c.nt, c.dt, amp[i], fc[i], ts[i],
                                          shape[i]),
                          "wavelet"))
                    return 2;
        } else {
            c.measurement = (int)ini.GetInteger(sec, "measurement_records", 0);
            c.obs_file = ini.Get(sec, "signal_file", "");
        }
    }
    // [full_waveform_inversion] (fd_fwi.cu:26-51: the intervals' z key is
    // read as "grid_interval_y"; defaults z2 = nzt-1, x2 = nxt-1, then the
    // padding offsets; the window is clipped to the padded grid here)
    c.fdt = (int)ini.GetInteger("full_waveform_inversion", "time_interval", 1);
    c.fdx = (int)ini.GetInteger("full_waveform_inversion", "grid_interval_x", 1);
    c.fdz = (int)ini.GetInteger("full_waveform_inversion", "grid_interval_y", 1);
    c.x1 = (int)ini.GetInteger("full_waveform_inversion", "left_grid", 0);
    c.x2 = (int)ini.GetInteger("full_waveform_inversion", "right_grid", 0);
    c.z1 = (int)ini.GetInteger("full_waveform_inversion", "top_grid", 0);
    c.z2 = (int)ini.GetInteger("full_waveform_inversion", "bottom_grid", 0);
    if (c.z2 == 0) c.z2 = c.nzt - 1;
    if (c.x2 == 0) c.x2 = c.nxt - 1;
    c.x1 += c.ppad;
    c.x2 += c.ppad;
    c.z1 += zoff;
    c.z2 += zoff;
    c.x2 = std::min(c.x2, c.nxt);
    c.z2 = std::min(c.z2, c.nzt);
    return 0;
}

// Homogeneous medium (fd_medium.cu:54-78), with the reference's stiffer circle
// (lam x 1.3 where (iz-nzt/2)^2 + (ix-nxt/2)^2 < nzt^2/49, fd_medium.cu:80-101)
// for forward modelling; CSV models replace it when given.
int read_csv(const std::string& path, int rows, int cols, std::vector<double>& out);

int medium(const Config& c, bool circle, std::vector<double>& lam, std::vector<double>& mu,
           std::vector<double>& rho) {
    const size_t n = (size_t)c.nzt * c.nxt;
    const double smu = c.vs * c.vs * c.rho, slam = c.vp * c.vp * c.rho - 2.0 * smu;
    lam.assign(n, slam);
    mu.assign(n, smu);
    rho.assign(n, c.rho);
    if (circle)
        for (int iz = 0; iz < c.nzt; iz++)
            for (int ix = 0; ix < c.nxt; ix++)
                if ((iz - c.nzt / 2) * (iz - c.nzt / 2) + (ix - c.nxt / 2) * (ix - c.nxt / 2) < c.nzt * c.nzt / 49)
                    lam[(size_t)iz * c.nxt + ix] = 1.3 * slam;
    if (!c.lam_file.empty() && read_csv(c.lam_file, c.nzt, c.nxt, lam)) return 2;
    if (!c.mu_file.empty() && read_csv(c.mu_file, c.nzt, c.nxt, mu)) return 2;
    if (!c.rho_file.empty() && read_csv(c.rho_file, c.nzt, c.nxt, rho)) return 2;
    return 0;
}

// "v, v, v, \n" rows as the reference writes them
int read_csv(const std::string& path, int rows, int cols, std::vector<double>& out) {
    std::ifstream in(path);
    if (!in) return fail("can't read " + path);
    out.assign((size_t)rows * cols, 0.0);
    std::string line;
    int r = 0;
    while (r < rows && std::getline(in, line)) {
        std::stringstream ss(line);
        std::string tok;
        int k = 0;
        while (std::getline(ss, tok, ',')) {
            if (tok.find_first_not_of(" \t\r") == std::string::npos) continue;
            if (k < cols) out[(size_t)r * cols + k] = std::atof(tok.c_str());
            k++;
        }
        if (k < cols) return fail(path + ": row " + std::to_string(r) + " has " + std::to_string(k) + " values, " +
                                  std::to_string(cols) + " expected");
        r++;
    }
    if (r < rows) return fail(path + ": " + std::to_string(r) + " rows, " + std::to_string(rows) + " expected");
    return 0;
}

void mkdirs(const std::string& d) {
    std::string cur;
    std::stringstream ss(d);
    std::string part;
    if (!d.empty() && d[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0755);
    }
}

bool write_csv(const std::string& path, const double* a, int rows, int cols) {
    std::ofstream f(path);
    if (!f) return false;
    for (int r = 0; r < rows; r++) {
        for (int k = 0; k < cols; k++) f << a[(size_t)r * cols + k] << ", ";
        f << std::endl;
    }
    return (bool)f;
}

void print_config(const Config& c) {
    std::cout << "{\"fdorder\": " << c.fdorder << ", \"fwinv\": " << c.fwinv << ", \"nshots\": " << c.nshots
              << ", \"nt\": " << c.nt << ", \"nx\": " << c.nx << ", \"nz\": " << c.nz << ", \"nxt\": " << c.nxt
              << ", \"nzt\": " << c.nzt << ", \"fpad\": " << c.fpad << ", \"ppad\": " << c.ppad
              << ", \"fsurf\": " << c.fsurf << ", \"snap_interval\": " << c.snap_interval << ", \"dt\": " << c.dt
              << ", \"window\": [" << c.fdt << ", " << c.fdx << ", " << c.fdz << ", " << c.x1 << ", " << c.x2 << ", "
              << c.z1 << ", " << c.z2 << "], \"src\": [";
    for (size_t i = 0; i < c.src.x.size(); i++)
        std::cout << (i ? ", " : "") << "[" << c.src.x[i] << ", " << c.src.z[i] << ", " << c.src.comp[i] << ", "
                  << c.src.shot[i] << "]";
    std::cout << "], \"rec\": [";
    for (size_t i = 0; i < c.rec.x.size(); i++)
        std::cout << (i ? ", " : "") << "[" << c.rec.x[i] << ", " << c.rec.z[i] << ", " << c.rec.comp[i] << ", "
                  << c.rec.shot[i] << "]";
    std::cout.precision(17);
    std::cout << "], \"hc1\": " << c.hc[1] << ", \"cpml_b0\": " << (c.b.empty() ? 0.0 : c.b[0]) << "}" << std::endl;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: fwi_run CONFIG.ini [--out DIR] [--device N] [--batch N] [--dry-run]" << std::endl;
        return 2;
    }
    std::string out = ".";
    int device = 0, batch = 0;
    bool dry = false;
    for (int i = 2; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "--out" && i + 1 < argc) out = argv[++i];
        else if (a == "--device" && i + 1 < argc) device = std::atoi(argv[++i]);
        else if (a == "--batch" && i + 1 < argc) batch = std::atoi(argv[++i]);
        else if (a == "--dry-run") dry = true;
        else return fail("unknown argument " + a);
    }
    Config c;
    if (load(argv[1], c)) return 2;
    if (dry) {
        print_config(c);
        return 0;
    }
    std::vector<double> lam, mu, rho;
    if (medium(c, c.fwinv == 0, lam, mu, rho)) return 2;
    fwi_psv_desc d = {c.nt, c.nzt, c.nxt, c.fpad, c.ppad, c.npml, c.fsurf, c.fdorder, c.dt, c.dx, c.dz,
                      {c.hc[0], c.hc[1], c.hc[2], c.hc[3], c.hc[4], c.hc[5], c.hc[6]},
                      c.a.data(), c.b.data(), c.K.data(), c.ah.data(), c.bh.data(), c.Kh.data()};
    fwi_psv_engine* e = nullptr;
    if (check(fwi_psv_create(&d, device, &e), "create")) return 2;
    int rc = 0;
    const int nsrc = (int)c.src.x.size(), nrec = (int)c.rec.x.size();
    std::vector<int> shots(c.nshots);
    for (int s = 0; s < c.nshots; s++) shots[s] = s;
    do {
        if ((rc = check(fwi_psv_set_model_lmr(e, lam.data(), mu.data(), rho.data()), "set_model"))) break;
        if ((rc = check(fwi_psv_set_sources(e, nsrc, c.src.x.data(), c.src.z.data(), c.src.comp.data(),
                                            c.src.shot.data(), c.src.signal.data()),
                        "set_sources")))
            break;
        if ((rc = check(fwi_psv_set_receivers(e, nrec, c.rec.x.data(), c.rec.z.data(), c.rec.comp.data(),
                                              c.rec.shot.data()),
                        "set_receivers")))
            break;
        if ((rc = check(fwi_psv_set_exec(e, 1, 0, 0, batch), "set_exec"))) break;
        if (!c.fwinv) {
            // forward modelling: all shots together
            mkdirs(out + "/io/receiver");
            if (c.snap_interval > 0) {
                mkdirs(out + "/io/snap_data");
                if ((rc = check(fwi_psv_set_snapshots(e, c.snap_interval, 4), "set_snapshots"))) break;
            }
            std::vector<double> recs((size_t)std::max(nrec, 1) * c.nt, 0.0);
            if ((rc = check(fwi_psv_forward(e, c.nshots, shots.data(), nullptr, recs.data(), nullptr, 0), "forward")))
                break;
            if (!write_csv(out + "/io/receiver/rec_signal.csv", recs.data(), nrec, c.nt)) {
                rc = fail("can't write rec_signal.csv");
                break;
            }
            if (c.snap_interval > 0) {
                std::vector<double> snap((size_t)c.nzt * c.nxt);
                const int nsnap = 1 + (c.nt - 1) / c.snap_interval;
                for (int k = 0; k < nsnap && !rc; k++) {
                    if ((rc = check(fwi_psv_snapshot(e, c.nshots - 1, k, snap.data()), "snapshot"))) break;
                    write_csv(out + "/io/snap_data/vz_snap" + std::to_string(k) + ".csv", snap.data(), c.nzt, c.nxt);
                }
            }
            std::cout << "forward modelling: " << c.nshots << " shot(s), " << c.nt << " steps; traces in "
                      << out << "/io/receiver/rec_signal.csv" << std::endl;
            break;
        }
        // full waveform inversion
        if (!c.measurement || c.obs_file.empty()) {
            rc = fail("full waveform inversion needs [receiver] measurement_records = 1 and signal_file");
            break;
        }
        std::vector<double> obs;
        if ((rc = read_csv(c.obs_file, nrec, c.nt, obs))) break;
        if ((rc = check(fwi_psv_set_fwi(e, c.fdt, c.fdx, c.fdz, c.x1, c.x2, c.z1, c.z2), "set_fwi"))) break;
        if ((rc = check(fwi_psv_set_strategy(e, FWI_STORE_BINOMIAL, c.checkpoints, 0), "set_strategy"))) break;
        mkdirs(out + "/io/density_snap");
        fwi_psv_fwi_opts o = {1, c.max_error, 0.01, c.order, c.trial, 1, nullptr, nullptr, nullptr, 0.0, nullptr};
        std::vector<fwi_psv_fwi_iter> log((size_t)c.nshots);
        bool converged = false;
        for (int iter = 1; iter <= c.max_iter && !rc; iter++) {
            int done = 0;
            if ((rc = check(fwi_psv_fwi_run(e, &o, c.nshots, shots.data(), obs.data(), lam.data(), mu.data(),
                                            rho.data(), log.data(), &done),
                            "fwi_run")))
                break;
            for (int k = 0; k < done; k++) {
                std::cout << "iteration " << iter << ": L2 = " << log[k].misfit << ", step length = "
                          << log[k].step_length << ", trials = " << log[k].trials << ", " << log[k].seconds << " s"
                          << std::endl;
                if (log[k].step_length > 0) o.step_length = log[k].step_length;
                if (log[k].misfit < c.max_error) converged = true;
                if (log[k].status == 1) {
                    std::cout << "Step length estimation failed !" << std::endl;
                    rc = 1;
                }
            }
            write_csv(out + "/io/density_snap/density_snap" + std::to_string(iter) + ".csv", rho.data(), c.nzt, c.nxt);
            write_csv(out + "/io/density_snap/lam_snap" + std::to_string(iter) + ".csv", lam.data(), c.nzt, c.nxt);
            write_csv(out + "/io/density_snap/mu_snap" + std::to_string(iter) + ".csv", mu.data(), c.nzt, c.nxt);
            if (converged) break;
        }
        if (!rc && !converged) {
            std::cout << "Error: convergence not reached within maximum iteration" << std::endl;
            rc = 1;
        }
    } while (false);
    fwi_psv_destroy(e);
    return rc;
}
