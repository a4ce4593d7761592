// fwi_optim.cu -- the FWI optimiser on top of the engine's C ABI.
//
// Reference sequence (Mohammad-debug/CUDA_FWI, CUDA_week2/):
//   per iteration  fd_wave_model.cu:750-955: average_parameters, medium_average,
//                  forward + residual + adjoint per shot, energy-weight scaling,
//                  step-length estimation, material update
//   step length    fwi_step_length_estimation.cu:16-223 (trial updates and
//                  forward runs over all shots, state machine of conditions
//                  1.1/1.2/2.1/2.2), parabola fit :226-271 with solvelin.cu:6-42
//   update         FDMedium::fwi_grad_update, fd_medium.cu:161-240
// The models, the gradients and every update live in device memory (FP64);
// the misfit sweeps and gradients are the engine's batched launches; the
// host runs the search's control flow on scalars.  The driver's own kernels
// and copies run on the legacy default stream; the engine runs on its own
// stream and returns only when its work is done, so the driver synchronises
// its stream before handing a model to the engine.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fwi_psv.h"
#include "fwi_alloc.hpp"
#include "fwi_host.h"

namespace {

#define OPT_CUDA(expr)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess)                                                                  \
            return fwi::fail(FWI_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)
#define OPT_TRY(expr)                 \
    do {                              \
        int _s = (expr);              \
        if (_s != FWI_OK) return _s;  \
    } while (0)

struct Window {
    int nxt, x1, x2, z1, z2, fdx, fdz, nfz, nfx;
};

// mat_new = mat + sn * grad on the window samples, clamped to [lo, hi], and
// the old value kept where the result is negative (fd_medium.cu:201-214).
__global__ void update_kernel(const double* __restrict__ old, double* __restrict__ cur,
                              const double* __restrict__ grad, double sn, double lo, double hi, Window w) {
    const size_t n = (size_t)w.nfz * w.nfx;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int zf = (int)(i / w.nfx), xf = (int)(i % w.nfx);
        const int iz = w.z1 + zf * w.fdz, ix = w.x1 + xf * w.fdx;
        if (iz >= w.z2 || ix >= w.x2) continue;
        const size_t c = (size_t)iz * w.nxt + ix;
        double v = old[c] + sn * grad[i];
        if (v < lo) v = lo;
        if (v > hi) v = hi;
        if (v < 0.0) v = old[c];
        cur[c] = v;
    }
}

// max(0, max over window samples of m): non-negative doubles order like their bits.
__global__ void window_max_kernel(const double* __restrict__ m, Window w, unsigned long long* __restrict__ out) {
    const size_t n = (size_t)w.nfz * w.nfx;
    double best = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int zf = (int)(i / w.nfx), xf = (int)(i % w.nfx);
        const int iz = w.z1 + zf * w.fdz, ix = w.x1 + xf * w.fdx;
        if (iz >= w.z2 || ix >= w.x2) continue;
        best = fmax(best, m[(size_t)iz * w.nxt + ix]);
    }
    atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

// Fixed-shape partial sums (block b sums its own contiguous chunk in a fixed
// tree order), so the total is the same on every run.
constexpr int kSumBlocks = 512, kSumThreads = 256;
__global__ void partial_sums_kernel(const double* __restrict__ a, size_t n, double* __restrict__ partial) {
    __shared__ double sh[kSumThreads];
    const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const size_t b0 = blockIdx.x * chunk, b1 = b0 + chunk < n ? b0 + chunk : n;
    double s = 0.0;
    for (size_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += a[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

struct DevBuf {
    void* p = nullptr;
    fwi::DeviceAllocator al;  // the allocator that made p
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { fwi::device_free(p, al); }
    int alloc(size_t bytes) {
        if (fwi::device_alloc(&p, bytes, &al) != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return fwi::fail(FWI_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed");
        }
        return FWI_OK;
    }
    double* d() const { return static_cast<double*>(p); }
};

// matType 1 (rho), 2 (lam), 3 (mu) limits of fwi_grad_update (fd_medium.cu:172-183)
constexpr double kLo[3] = {0.0, 0.0, 1.5}, kHi[3] = {48.0e9, 27.0e9, 3000.0};  // lam, mu, rho

struct Driver {
    fwi_psv_engine* e = nullptr;
    fwi_psv_layout L{};
    Window w{};
    size_t n = 0, nf = 0;
    DevBuf cur[3], old[3], grad[3], scratch;
    std::vector<int> shots;
    const double* obs = nullptr;
    bool obs_uploaded = false;
    int trial_mode = FWI_TRIAL_SUM;
    double norm[3] = {0, 0, 0};  // mat_max / grad_max per parameter
    std::vector<double> hg[3];

    int init(fwi_psv_engine* eng) {
        e = eng;
        OPT_TRY(fwi_psv_get_layout(e, &L));
        OPT_CUDA(cudaSetDevice(L.device));
        w = {L.nxt, L.x1, L.x2, L.z1, L.z2, L.fwi_dx, L.fwi_dz, L.nfz, L.nfx};
        n = (size_t)L.nzt * L.nxt;
        nf = (size_t)L.nfz * L.nfx;
        for (int q = 0; q < 3; q++) {
            OPT_TRY(cur[q].alloc(n * 8));
            OPT_TRY(old[q].alloc(n * 8));
            OPT_TRY(grad[q].alloc(nf * 8));
            hg[q].assign(nf, 0.0);
        }
        OPT_TRY(scratch.alloc(kSumBlocks * 8 + 16));
        return FWI_OK;
    }
    int blocks(size_t m) const { return (int)std::min<size_t>((m + 255) / 256, 4096); }

    int materials(DevBuf* m) {
        OPT_CUDA(cudaStreamSynchronize(0));
        return fwi_psv_set_model_device(e, m[0].d(), m[1].d(), m[2].d());
    }
    ~Driver() {
        if (e) fwi_psv_set_precondition(e, 0, 1.0, 1.0, 1.0);
    }

    // C_lam, C_mu, C_rho of the current model (fd_medium.cu:253-277)
    int medium_average(double c[3]) {
        std::vector<double> part(kSumBlocks);
        for (int q = 0; q < 3; q++) {
            partial_sums_kernel<<<kSumBlocks, kSumThreads>>>(cur[q].d(), n, scratch.d());
            OPT_CUDA(cudaGetLastError());
            OPT_CUDA(cudaMemcpy(part.data(), scratch.p, kSumBlocks * 8, cudaMemcpyDeviceToHost));
            double s = 0.0;
            for (double v : part) s += v;
            c[q] = s / (double)n;
        }
        return FWI_OK;
    }

    // gradient of the given shots at the current model (scaled, summed) -> device grad[]
    int gradient(const int* ids, int m, double* misfit_out, double c[3], int precond) {
        OPT_TRY(fwi_psv_set_precondition(e, precond, c[0], c[1], c[2]));
        std::vector<double> mis(m);
        const int flags = obs_uploaded ? FWI_FWD_RESIDENT_OBS : 0;
        OPT_TRY(fwi_psv_gradient(e, m, ids, obs_uploaded ? nullptr : obs, mis.data(), hg[0].data(), hg[1].data(),
                                 hg[2].data(), flags));
        if (!obs_uploaded && m == (int)shots.size()) obs_uploaded = true;
        double s = 0.0;
        for (double v : mis) s += v;
        if (misfit_out) *misfit_out = s;
        for (int q = 0; q < 3; q++) OPT_CUDA(cudaMemcpy(grad[q].d(), hg[q].data(), nf * 8, cudaMemcpyHostToDevice));
        return FWI_OK;
    }

    // step normalisation step * mat_max / grad_max of fwi_grad_update; grad_max
    // is the signed value of the largest |grad| met in row-major order, as the
    // reference's loop leaves it (fd_medium.cu:187-196)
    int normalise() {
        for (int q = 0; q < 3; q++) {
            unsigned long long* mx = reinterpret_cast<unsigned long long*>(scratch.d());
            OPT_CUDA(cudaMemset(mx, 0, 8));
            window_max_kernel<<<blocks(nf), 256>>>(old[q].d(), w, mx);
            OPT_CUDA(cudaGetLastError());
            unsigned long long bits = 0;
            OPT_CUDA(cudaMemcpy(&bits, mx, 8, cudaMemcpyDeviceToHost));
            double mat_max;
            std::memcpy(&mat_max, &bits, 8);
            double gmax = 0.0;
            for (int zf = 0; zf < L.nfz; zf++) {
                if (L.z1 + zf * L.fwi_dz >= L.z2) break;
                for (int xf = 0; xf < L.nfx; xf++) {
                    if (L.x1 + xf * L.fwi_dx >= L.x2) break;
                    const double g = hg[q][(size_t)zf * L.nfx + xf];
                    if (std::fabs(g) > gmax) gmax = g;
                }
            }
            norm[q] = gmax != 0.0 ? mat_max / gmax : 0.0;
        }
        return FWI_OK;
    }

    // cur = old + update(step): lam, mu with step, rho with half of it
    int apply(double step) {
        const double f[3] = {step, step, 0.5 * step};
        for (int q = 0; q < 3; q++) {
            OPT_CUDA(cudaMemcpy(cur[q].p, old[q].p, n * 8, cudaMemcpyDeviceToDevice));
            update_kernel<<<blocks(nf), 256>>>(old[q].d(), cur[q].d(), grad[q].d(), f[q] * norm[q], kLo[q], kHi[q], w);
            OPT_CUDA(cudaGetLastError());
        }
        return FWI_OK;
    }

    // misfit of the trial model cur (all shots; the last shot's in the reference mode)
    int trial_misfit(double* out) {
        OPT_TRY(materials(cur));
        std::vector<double> mis(shots.size());
        const int flags = obs_uploaded ? FWI_FWD_RESIDENT_OBS : 0;
        OPT_TRY(fwi_psv_misfit(e, (int)shots.size(), shots.data(), obs_uploaded ? nullptr : obs, mis.data(), flags));
        obs_uploaded = true;
        double s = 0.0;
        for (double v : mis) s += v;
        *out = trial_mode == FWI_TRIAL_LAST_SHOT ? mis.back() : s;
        return FWI_OK;
    }

    int commit() {
        for (int q = 0; q < 3; q++) OPT_CUDA(cudaMemcpy(old[q].p, cur[q].p, n * 8, cudaMemcpyDeviceToDevice));
        return FWI_OK;
    }
    int restore() {
        for (int q = 0; q < 3; q++) OPT_CUDA(cudaMemcpy(cur[q].p, old[q].p, n * 8, cudaMemcpyDeviceToDevice));
        return FWI_OK;
    }

    double model_error(const fwi_psv_fwi_opts* o) {
        const double* t[3] = {o->true_lam, o->true_mu, o->true_rho};
        if (!t[0] || !t[1] || !t[2]) return -1.0;
        std::vector<double> h(n);
        double acc = 0.0;
        for (int q = 0; q < 3; q++) {
            if (cudaMemcpy(h.data(), cur[q].p, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) return -1.0;
            double num = 0.0, den = 0.0;
            for (size_t i = 0; i < n; i++) {
                const double d = h[i] - t[q][i];
                num += d * d;
                den += t[q][i] * t[q][i];
            }
            acc += den > 0 ? num / den : 0.0;
        }
        return std::sqrt(acc / 3.0);
    }
};

int driver_trial(void* ctx, double step, double* misfit) {
    Driver* d = static_cast<Driver*>(ctx);
    OPT_TRY(d->apply(step));
    return d->trial_misfit(misfit);
}

}  // namespace

extern "C" double fwi_psv_calc_opt_step(const double L2[3], const double sl[3]) {
    // Gauss elimination without pivoting on A = [1, sl, sl^2] (solvelin.cu:10-24,
    // its multiplier in float) and back substitution from the last row with a
    // float accumulator (solvelin.cu:27-40; the reference starts one row past
    // the end, an out-of-bounds read this version does not reproduce)
    double A[3][3], b[3], x[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; i++) {
        A[i][0] = 1.0;
        A[i][1] = sl[i];
        A[i][2] = sl[i] * sl[i];
        b[i] = L2[i];
    }
    for (int k = 0; k < 2; k++)
        for (int r = k; r < 2; r++) {
            const float f = (float)(A[r + 1][k] / A[k][k]);
            for (int c = 0; c < 3; c++) A[r + 1][c] = A[r + 1][c] - f * A[k][c];
            b[r + 1] = b[r + 1] - f * b[k];
        }
    for (int k = 2; k >= 0; k--) {
        float acc = (float)b[k];
        for (int c = 2; c > k; c--) acc = (float)(acc - A[k][c] * x[c]);
        x[k] = acc / A[k][k];
    }
    return -x[1] / (2.0 * x[2]);
}

extern "C" int fwi_psv_step_search(double est, double L2_0, fwi_psv_trial_fn trial, void* ctx, double* opt,
                                   int* trials, int* status) {
    if (!trial || !opt) return fwi::fail(FWI_ERR_INVALID, "null trial callback or output");
    const double scale = 2.0;  // est_scale_factor
    const int stepmax = 6;
    double L2[4] = {L2_0, 0.0, 0.0, L2_0}, sl[4] = {0.0, 0.0, 0.0, 0.0};
    int step1 = 0, step2 = 0, itest = 1, count = 0, calls = 0, st = 0;
    while (step2 != 1 || step1 != 1) {
        OPT_TRY(trial(ctx, est, &L2[itest]));
        calls++;
        sl[itest] = est;
        sl[0] = 0.0;
        if (step1 == 1 && L2[1] < L2[2]) {  // condition 2.2: the minimum is bracketed
            sl[2] = est;
            step2 = 1;
        } else if (step1 == 1) {  // 2.1: grow the third step
            sl[2] = est;
            est = est + est / scale;
            count++;
        } else if (L2[0] > L2[1]) {  // 1.2: a step reduced the misfit; look for a larger one
            sl[1] = est;
            step1 = 1;
            itest = 2;
            count = 0;
            est = est + est / scale;
        } else {  // 1.1: shrink
            est = est / scale;
            count++;
        }
        if (step1 == 0 && count > stepmax) {
            st = 1;  // the reference exits the program here
            break;
        }
        if (step1 == 1 && count > stepmax) {
            st = 2;  // calculate with the less optimal bracket
            step1 = step2 = 1;
        }
    }
    *opt = st == 1 ? 0.0 : fwi_psv_calc_opt_step(L2, sl);
    if (trials) *trials = calls;
    if (status) *status = st;
    return FWI_OK;
}

// ---------------------------------------------------------------------------
// FWI-iteration resume file (no reference counterpart)
// ---------------------------------------------------------------------------
// Layout: a header, `entries` log records, then lam, mu, rho ([nzt][nxt] FP64).
// The header carries what the continuation must match (cells, shots, order,
// trial mode, preconditioning, the first step estimate) and the loop state.
struct ResumeHeader {
    char magic[8];
    long long cells;
    int nshots, order, trial, precondition;
    int iters_done, entries, stopped, pad;
    double step_length0, step;
};
static const char kResumeMagic[8] = {'F', 'W', 'I', 'P', 'S', 'V', 'R', '1'};

static bool resume_matches(const ResumeHeader& h, const fwi_psv_fwi_opts* o, size_t cells, int nshots) {
    return std::memcmp(h.magic, kResumeMagic, 8) == 0 && h.cells == (long long)cells && h.nshots == nshots &&
           h.order == o->order && h.trial == o->trial_misfit && h.precondition == o->precondition &&
           h.step_length0 == o->step_length && h.iters_done >= 0 && h.entries >= 0;
}

// Write the state (the model from the device) beside the file, then rename it
// over the file, so an interrupted write leaves the previous state.
static int resume_save(const char* path, const ResumeHeader& h, const fwi_psv_fwi_iter* log,
                       const std::vector<double>* model) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return fwi::fail(FWI_ERR_IO, "cannot write the resume file " + tmp);
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
    if (h.entries > 0) ok = ok && std::fwrite(log, sizeof(fwi_psv_fwi_iter), h.entries, f) == (size_t)h.entries;
    for (int q = 0; q < 3; q++) ok = ok && std::fwrite(model[q].data(), 8, model[q].size(), f) == model[q].size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fwi::fail(FWI_ERR_IO, std::string("cannot write the resume file ") + path);
    }
    return FWI_OK;
}

// Read a resume file if there is one: *found = false when the file does not
// exist; FWI_ERR_INVALID when it belongs to another run or is cut short.
static int resume_load(const char* path, const fwi_psv_fwi_opts* o, size_t cells, int nshots, int capacity,
                       ResumeHeader* h, fwi_psv_fwi_iter* log, std::vector<double>* model, bool* found) {
    *found = false;
    FILE* f = std::fopen(path, "rb");
    if (!f) return FWI_OK;
    bool ok = std::fread(h, sizeof(*h), 1, f) == 1 && resume_matches(*h, o, cells, nshots);
    if (ok && h->entries > capacity) {
        std::fclose(f);
        return fwi::fail(FWI_ERR_INVALID, std::string("the resume file ") + path + " holds " +
                                              std::to_string(h->entries) + " log entries, more than max_iter allows (" +
                                              std::to_string(capacity) + ")");
    }
    if (ok && h->entries > 0) ok = std::fread(log, sizeof(fwi_psv_fwi_iter), h->entries, f) == (size_t)h->entries;
    for (int q = 0; q < 3 && ok; q++) {
        model[q].resize(cells);
        ok = std::fread(model[q].data(), 8, cells, f) == cells;
    }
    std::fclose(f);
    if (!ok) return fwi::fail(FWI_ERR_INVALID, std::string("the resume file ") + path +
                                                   " does not belong to this run (grid, shots or options) or is cut short");
    *found = true;
    return FWI_OK;
}

extern "C" int fwi_psv_fwi_run(fwi_psv_engine* e, const fwi_psv_fwi_opts* o, int nshots, const int* ids,
                               const double* obs, double* lam, double* mu, double* rho, fwi_psv_fwi_iter* log,
                               int* done) {
    if (!e || !o || nshots < 1 || !ids || !obs || !lam || !mu || !rho || !log)
        return fwi::fail(FWI_ERR_INVALID, "bad arguments to fwi_psv_fwi_run");
    if (o->max_iter < 0 || !(o->step_length > 0) || !(o->restart_step >= 0.0) ||
        (o->order != FWI_ORDER_SUMMED && o->order != FWI_ORDER_PER_SHOT) ||
        (o->trial_misfit != FWI_TRIAL_SUM && o->trial_misfit != FWI_TRIAL_LAST_SHOT))
        return fwi::fail(FWI_ERR_INVALID, "bad FWI options");
    Driver d;
    OPT_TRY(d.init(e));
    d.shots.assign(ids, ids + nshots);
    d.obs = obs;
    d.trial_mode = o->trial_misfit;
    double* host[3] = {lam, mu, rho};
    double step = o->step_length;
    int entries = 0, iter0 = 0;
    bool stop = false;
    ResumeHeader rh{};
    std::vector<double> rm[3];
    const int capacity = o->max_iter * (o->order == FWI_ORDER_SUMMED ? 1 : nshots);
    if (o->resume_file) {
        bool found = false;
        OPT_TRY(resume_load(o->resume_file, o, d.n, nshots, capacity, &rh, log, rm, &found));
        if (found) {
            for (int q = 0; q < 3; q++) std::memcpy(host[q], rm[q].data(), d.n * 8);
            step = rh.step;
            entries = rh.entries;
            iter0 = rh.iters_done;
            stop = rh.stopped != 0;
        } else {
            std::memcpy(rh.magic, kResumeMagic, 8);
            rh.cells = (long long)d.n;
            rh.nshots = nshots;
            rh.order = o->order;
            rh.trial = o->trial_misfit;
            rh.precondition = o->precondition;
            rh.step_length0 = o->step_length;
        }
    }
    for (int q = 0; q < 3; q++) {
        OPT_CUDA(cudaMemcpy(d.cur[q].p, host[q], d.n * 8, cudaMemcpyHostToDevice));
        OPT_CUDA(cudaMemcpy(d.old[q].p, host[q], d.n * 8, cudaMemcpyHostToDevice));
    }
    for (int iter = iter0; iter < o->max_iter && !stop; iter++) {
        double c[3];
        OPT_TRY(d.medium_average(c));
        OPT_TRY(d.materials(d.cur));
        const int groups = o->order == FWI_ORDER_SUMMED ? 1 : nshots;
        for (int gidx = 0; gidx < groups && !stop; gidx++) {
            const auto t0 = std::chrono::steady_clock::now();
            fwi_psv_fwi_iter& rec = log[entries];
            rec = fwi_psv_fwi_iter{0.0, 0.0, 0, 0, -1.0, 0.0};
            const int* gs = o->order == FWI_ORDER_SUMMED ? ids : ids + gidx;
            const int gm = o->order == FWI_ORDER_SUMMED ? nshots : 1;
            double L0 = 0.0;
            OPT_TRY(d.materials(d.cur));
            OPT_TRY(d.gradient(gs, gm, &L0, c, o->precondition));
            if (o->order == FWI_ORDER_PER_SHOT && o->trial_misfit == FWI_TRIAL_SUM) {
                // the search compares all-shot misfits: its step-0 value too
                std::vector<double> mis(nshots);
                OPT_TRY(fwi_psv_misfit(e, nshots, ids, d.obs_uploaded ? nullptr : obs, mis.data(),
                                       d.obs_uploaded ? FWI_FWD_RESIDENT_OBS : 0));
                d.obs_uploaded = true;
                L0 = 0.0;
                for (double v : mis) L0 += v;
            }
            rec.misfit = L0;
            if (L0 < o->max_error) {
                rec.model_error = d.model_error(o);
                rec.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                entries++;
                stop = true;
                break;
            }
            OPT_TRY(d.normalise());
            double opt = 0.0;
            int trials = 0, status = 0;
            OPT_TRY(fwi_psv_step_search(step, L0, driver_trial, &d, &opt, &trials, &status));
            if (status == 1 && o->restart_step > 0.0) {
                // opt-in continuation: one more search on the same gradient from restart_step
                int more = 0;
                OPT_TRY(fwi_psv_step_search(o->restart_step, L0, driver_trial, &d, &opt, &more, &status));
                trials += more;
            }
            rec.trials = trials;
            rec.status = status;
            if (status == 1) {
                OPT_TRY(d.restore());  // no step reduced the misfit: keep the model, stop
                stop = true;
            } else {
                OPT_TRY(d.apply(opt));
                OPT_TRY(d.commit());
                rec.step_length = opt;
                step = opt;
            }
            rec.model_error = d.model_error(o);
            rec.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            entries++;
        }
        if (o->resume_file) {
            rh.iters_done = iter + 1;
            rh.entries = entries;
            rh.stopped = stop ? 1 : 0;
            rh.step = step;
            for (int q = 0; q < 3; q++) {
                rm[q].resize(d.n);
                OPT_CUDA(cudaMemcpy(rm[q].data(), d.cur[q].p, d.n * 8, cudaMemcpyDeviceToHost));
            }
            OPT_TRY(resume_save(o->resume_file, rh, log, rm));
        }
    }
    for (int q = 0; q < 3; q++) OPT_CUDA(cudaMemcpy(host[q], d.cur[q].p, d.n * 8, cudaMemcpyDeviceToHost));
    if (done) *done = entries;
    return FWI_OK;
}
