// ref_driver.cpp -- a reference-style caller of the drop-in propagators.
//
// Calls forward_kernel_PSV_GPU and adjoint_kernel_PSV_GPU exactly the way the
// reference's FWI driver does (Mohammad-debug/CUDA_FWI,
// CUDA_week2/fd_wave_model.cu:498-591): host wavefields, materials, CPML memory
// and signals as contiguous row-pointer tables (the layout of
// CUDA_week2/util.cu:25-42, p[0] is the flat buffer), FWI storage as 3-D
// tables, source/receiver descriptions as std::vector<int> passed by value,
// and every d_* argument a cudaMalloc'd FP64 device buffer
// (fd_wave_model.cu:313-433).  Between the two calls it forms the residual in
// place and the misfit (calculate_l2_adjoint_sources, fd_wave_model.cu:972-1002)
// and reads d_We back, as the reference's driver does.
//
// Input and output are "named array" files (see read_blobs): the inputs of
// one shot (grid, hc, CPML profiles, lam/mu/rho and their staggered averages,
// acquisition, signals, observed data, FWI window); the outputs are the host
// results and copies of the device buffers the propagators filled.
//
// Usage: ref_driver IN OUT    (exit status 0 on success)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "fwi_psv.h"
#include "fwi_psv_ref.hpp"

namespace {

// ---- named-array files: repeated {u32 name length, name, u32 kind (0 f64,
// 1 i32), u64 count, data} -------------------------------------------------
struct Blobs {
    std::map<std::string, std::vector<double>> f;
    std::map<std::string, std::vector<int>> i;
};

bool read_blobs(const char* path, Blobs& b) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return false;
    while (true) {
        uint32_t nl = 0;
        if (std::fread(&nl, 4, 1, fp) != 1) break;
        std::string name(nl, '\0');
        uint32_t kind = 0;
        uint64_t n = 0;
        if (std::fread(&name[0], 1, nl, fp) != nl || std::fread(&kind, 4, 1, fp) != 1 ||
            std::fread(&n, 8, 1, fp) != 1) {
            std::fclose(fp);
            return false;
        }
        bool ok;
        if (kind == 0) {
            auto& v = b.f[name];
            v.resize(n);
            ok = std::fread(v.data(), 8, n, fp) == n;
        } else {
            auto& v = b.i[name];
            v.resize(n);
            ok = std::fread(v.data(), 4, n, fp) == n;
        }
        if (!ok) {
            std::fclose(fp);
            return false;
        }
    }
    std::fclose(fp);
    return true;
}

void put(FILE* fp, const std::string& name, const double* p, size_t n) {
    const uint32_t nl = (uint32_t)name.size(), kind = 0;
    const uint64_t cnt = n;
    std::fwrite(&nl, 4, 1, fp);
    std::fwrite(name.data(), 1, nl, fp);
    std::fwrite(&kind, 4, 1, fp);
    std::fwrite(&cnt, 8, 1, fp);
    std::fwrite(p, 8, n, fp);
}

// ---- the reference's host table layouts ---------------------------------
// Contiguous 2-D table: one block of dim1*dim2 values and dim1 row pointers.
struct Table2 {
    std::vector<double> data;
    std::vector<double*> rows;
    Table2(int dim1, int dim2, const double* init = nullptr) : data((size_t)dim1 * dim2, 0.0), rows(dim1) {
        if (init) std::memcpy(data.data(), init, data.size() * sizeof(double));
        for (int k = 0; k < dim1; k++) rows[k] = data.data() + (size_t)k * dim2;
    }
    double** p() { return rows.data(); }
};
// Contiguous 3-D table [dim1][dim2][dim3].
struct Table3 {
    std::vector<double> data;
    std::vector<double*> rows;
    std::vector<double**> planes;
    Table3(int dim1, int dim2, int dim3) : data((size_t)dim1 * dim2 * dim3, 0.0), rows((size_t)dim1 * dim2),
                                          planes(dim1) {
        for (size_t r = 0; r < rows.size(); r++) rows[r] = data.data() + r * dim3;
        for (int k = 0; k < dim1; k++) planes[k] = rows.data() + (size_t)k * dim2;
    }
    double*** p() { return planes.data(); }
};

// FP64 device buffer, cudaMalloc'd and zeroed.
struct Dev {
    double* p = nullptr;
    size_t n = 0;
    explicit Dev(size_t count) : n(count) {
        if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(double)) != cudaSuccess) p = nullptr;
        if (p) cudaMemset(p, 0, std::max<size_t>(count, 1) * sizeof(double));
    }
    ~Dev() { cudaFree(p); }
    std::vector<double> host() const {
        std::vector<double> h(n);
        if (n) cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost);
        return h;
    }
    Dev(const Dev&) = delete;
    Dev& operator=(const Dev&) = delete;
};

int fail(const char* what) {
    std::fprintf(stderr, "ref_driver: %s\n", what);
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) return fail("usage: ref_driver IN OUT");
    Blobs in;
    if (!read_blobs(argv[1], in)) return fail("cannot read the input file");
    auto I = [&](const char* k) { return in.i.at(k)[0]; };
    auto F = [&](const char* k) -> std::vector<double>& { return in.f.at(k); };
    const int ishot = I("shot"), nt = I("nt"), nzt = I("nzt"), nxt = I("nxt"), fpad = I("fpad");
    const int ppad = I("ppad"), npml = I("npml"), fdorder = I("fdorder");
    const bool fsurf = I("fsurf") != 0;
    const double dt = F("dt")[0], dx = F("dx")[0], dz = F("dz")[0];
    const int fdt = I("fwi_dt"), fdx = I("fwi_dx"), fdz = I("fwi_dz");
    const int x1 = I("x1"), x2 = I("x2"), z1 = I("z1"), z2 = I("z2");
    const int nft = 1 + (nt - 1) / fdt, nfz = 1 + (z2 - z1) / fdz, nfx = 1 + (x2 - x1) / fdx;
    const int tp = 2 * (npml + 1);
    const size_t cells = (size_t)nzt * nxt, xs = (size_t)nzt * tp, zs = (size_t)tp * nxt;
    const size_t store = (size_t)nft * nfz * nfx, ng = (size_t)nfz * nfx;

    // host state, materials, CPML memory (the reference's FDWave / FDMedium / FDCpml members)
    Table2 vx(nzt, nxt), vz(nzt, nxt), sxx(nzt, nxt), szx(nzt, nxt), szz(nzt, nxt);
    Table2 lam(nzt, nxt, F("lam").data()), mu(nzt, nxt, F("mu").data());
    Table2 mu_zx(nzt - 1, nxt - 1, F("mu_zx").data()), rho_zp(nzt - 1, nxt - 1, F("rho_zp").data());
    Table2 rho_xp(nzt - 1, nxt - 1, F("rho_xp").data());
    Table2 m_vx_x(nzt, tp), m_vz_x(nzt, tp), m_sxx_x(nzt, tp), m_szx_x(nzt, tp);
    Table2 m_vx_z(tp, nxt), m_vz_z(tp, nxt), m_szz_z(tp, nxt), m_szx_z(tp, nxt);
    std::vector<double> hc = F("hc"), a = F("cpml_a"), b = F("cpml_b"), K = F("cpml_K");
    std::vector<double> ah = F("cpml_a_half"), bh = F("cpml_b_half"), Kh = F("cpml_K_half");
    // acquisition (FDSeismogram: ivec members, signals as 2-D tables)
    const std::vector<int> src_x = in.i.at("src_x"), src_z = in.i.at("src_z"), src_comp = in.i.at("src_comp");
    const std::vector<int> src_shot = in.i.at("src_shot");
    const std::vector<int> rec_x = in.i.at("rec_x"), rec_z = in.i.at("rec_z"), rec_comp = in.i.at("rec_comp");
    const std::vector<int> rec_shot = in.i.at("rec_shot");
    const int nsrc = (int)src_x.size(), nrec = (int)rec_x.size();
    Table2 src_signal(nsrc, nt, F("src_signal").data());
    Table2 rec_signal(nrec, nt), rec_meas(nrec, nt, F("obs").data());
    // FWI storage and gradients (FDFWI members)
    Table3 fwi_vx(nft, nfz, nfx), fwi_vz(nft, nfz, nfx), fwi_sxx(nft, nfz, nfx), fwi_szx(nft, nfz, nfx);
    Table3 fwi_szz(nft, nfz, nfx);
    Table2 grad_lam(nfz, nfx), grad_mu(nfz, nfx), grad_rho(nfz, nfx);

    // device buffers, as fd_wave_model.cu:313-433 allocates them
    Dev d_a(tp), d_b(tp), d_K(tp), d_ah(tp), d_bh(tp), d_Kh(tp);
    Dev d_vx(cells), d_vz(cells), d_sxx(cells), d_szx(cells), d_szz(cells), d_We(cells);
    Dev d_fvx(store), d_fvz(store), d_fsxx(store), d_fszx(store), d_fszz(store);
    Dev d_mvx_x(xs), d_mvx_z(zs), d_mvz_x(xs), d_mvz_z(zs), d_msxx_x(xs), d_mszx_x(xs), d_mszz_z(zs),
        d_mszx_z(zs);
    Dev d_glam(ng), d_gmu(ng), d_grho(ng);
    Dev d_lam(cells), d_mu(cells), d_mu_zx(cells), d_rho_zp(cells), d_rho_xp(cells);
    for (Dev* d : {&d_a, &d_vx, &d_fvx, &d_mvx_x, &d_glam, &d_lam})
        if (!d->p) return fail("cudaMalloc failed");
    cudaMemcpy(d_a.p, a.data(), tp * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(d_b.p, b.data(), tp * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(d_K.p, K.data(), tp * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(d_ah.p, ah.data(), tp * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(d_bh.p, bh.data(), tp * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(d_Kh.p, Kh.data(), tp * 8, cudaMemcpyHostToDevice);

    const bool fwinv = true;
    forward_kernel_PSV_GPU(ishot, nt, nzt, nxt, fpad, ppad, dt, dx, dz, 0, fsurf, hc.data(), fdorder, vx.p(),
                           vz.p(), sxx.p(), szx.p(), szz.p(), lam.p(), mu.p(), mu_zx.p(), rho_zp.p(), rho_xp.p(),
                           npml, a.data(), b.data(), K.data(), ah.data(), bh.data(), Kh.data(), m_vx_x.p(),
                           m_vx_z.p(), m_vz_x.p(), m_vz_z.p(), m_sxx_x.p(), m_szx_x.p(), m_szz_z.p(), m_szx_z.p(),
                           nsrc, src_x, src_z, src_comp, src_signal.p(), src_shot, nrec, rec_x, rec_z, rec_comp,
                           rec_signal.p(), rec_shot, fwinv, fdt, fdx, fdz, x1, x2, z1, z2, fwi_vx.p(), fwi_vz.p(),
                           fwi_sxx.p(), fwi_szx.p(), fwi_szz.p(), d_a.p, d_b.p, d_K.p, d_ah.p, d_bh.p, d_Kh.p,
                           d_vx.p, d_vz.p, d_sxx.p, d_szx.p, d_szz.p, d_We.p, d_fvx.p, d_fvz.p, d_fsxx.p, d_fszx.p,
                           d_fszz.p, d_mvx_x.p, d_mvx_z.p, d_mvz_x.p, d_mvz_z.p, d_msxx_x.p, d_mszx_x.p,
                           d_mszz_z.p, d_mszx_z.p, d_lam.p, d_mu.p, d_mu_zx.p, d_rho_zp.p, d_rho_xp.p);
    if (fwi_psv_ref_status() != FWI_OK) return fail("forward_kernel_PSV_GPU reported an error");
    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return fail("cannot write the output file");
    put(out, "fwd_rec", rec_signal.data.data(), rec_signal.data.size());
    put(out, "fwd_vx", vx.data.data(), cells);
    put(out, "fwd_vz", vz.data.data(), cells);
    put(out, "fwd_szz", szz.data.data(), cells);
    {
        const std::vector<double> we = d_We.host(), dvz = d_vz.host(), dsxx = d_sxx.host(), st = d_fszz.host();
        const std::vector<double> svx = d_fvx.host();
        put(out, "fwd_d_We", we.data(), we.size());
        put(out, "fwd_d_vz", dvz.data(), dvz.size());
        put(out, "fwd_d_sxx", dsxx.data(), dsxx.size());
        put(out, "fwd_d_store_szz", st.data(), st.size());
        put(out, "fwd_d_store_vx", svx.data(), svx.size());
    }
    put(out, "fwd_store_sxx", fwi_sxx.data.data(), store);

    // residual in place and misfit over the receivers of this shot
    double misfit = 0.0;
    for (int r = 0; r < nrec; r++) {
        if (rec_shot[r] != ishot || rec_comp[r] != 2) continue;
        for (int t = 0; t < nt; t++) {
            const double d = rec_signal.rows[r][t] - rec_meas.rows[r][t];
            misfit += 0.5 * dt * d * d;
            rec_signal.rows[r][t] = d;
        }
    }
    put(out, "misfit", &misfit, 1);

    // the adjoint sources are the receivers carrying the residual
    adjoint_kernel_PSV_GPU(ishot, nt, nzt, nxt, fpad, ppad, dt, dx, dz, 0, fsurf, hc.data(), fdorder, vx.p(),
                           vz.p(), sxx.p(), szx.p(), szz.p(), lam.p(), mu.p(), mu_zx.p(), rho_zp.p(), rho_xp.p(),
                           npml, a.data(), b.data(), K.data(), ah.data(), bh.data(), Kh.data(), m_vx_x.p(),
                           m_vx_z.p(), m_vz_x.p(), m_vz_z.p(), m_sxx_x.p(), m_szx_x.p(), m_szz_z.p(), m_szx_z.p(),
                           nrec, rec_x, rec_z, rec_comp, rec_signal.p(), rec_shot, fwinv, fdt, fdx, fdz, x1, x2, z1,
                           z2, fwi_vx.p(), fwi_vz.p(), fwi_sxx.p(), fwi_szx.p(), fwi_szz.p(), grad_lam.p(),
                           grad_mu.p(), grad_rho.p(), d_a.p, d_b.p, d_K.p, d_ah.p, d_bh.p, d_Kh.p, d_vx.p, d_vz.p,
                           d_sxx.p, d_szx.p, d_szz.p, d_We.p, d_fvx.p, d_fvz.p, d_fsxx.p, d_fszx.p, d_fszz.p,
                           d_mvx_x.p, d_mvx_z.p, d_mvz_x.p, d_mvz_z.p, d_msxx_x.p, d_mszx_x.p, d_mszz_z.p,
                           d_mszx_z.p, d_glam.p, d_gmu.p, d_grho.p, d_lam.p, d_mu.p, d_mu_zx.p, d_rho_zp.p,
                           d_rho_xp.p);
    if (fwi_psv_ref_status() != FWI_OK) {
        std::fclose(out);
        return fail("adjoint_kernel_PSV_GPU reported an error");
    }
    put(out, "adj_grad_lam", grad_lam.data.data(), ng);
    put(out, "adj_grad_mu", grad_mu.data.data(), ng);
    put(out, "adj_grad_rho", grad_rho.data.data(), ng);
    put(out, "adj_vz", vz.data.data(), cells);
    {
        const std::vector<double> gl = d_glam.host(), gm = d_gmu.host(), gr = d_grho.host(), we = d_We.host();
        put(out, "adj_d_grad_lam", gl.data(), gl.size());
        put(out, "adj_d_grad_mu", gm.data(), gm.size());
        put(out, "adj_d_grad_rho", gr.data(), gr.size());
        put(out, "adj_d_We", we.data(), we.size());
    }
    std::fclose(out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(cudaGetErrorString(e));
    return 0;
}
