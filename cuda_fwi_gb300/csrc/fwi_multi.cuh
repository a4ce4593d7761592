// fwi_multi.cuh -- independent models of uneven grid size, order and nt in
// one launch per pass (part of fwi_engine.cu's translation unit: it uses the
// kernel dispatch, buffers and small kernels defined there).
//
// Each model ("item") keeps its own padded grid, materials, CPML profile,
// sources, receivers and time length; the reference's per-shot call
// (forward_kernel_PSV_GPU / adjoint_kernel_PSV_GPU for one shot of one
// model) becomes one slot of a work-list that spans every model.  The
// cell-mapped kernels read all geometry from the item descriptor of each tile,
// so one launch covers tiles of models of different sizes; models of one
// fdorder share a launch (the kernels are templated on the half order).
//
// Uneven nt: the items of a group are sorted by nt (descending) and their
// tiles laid out item-major, so the items still running at time step it are a
// prefix of the list: each launch covers that prefix only.  One binomial
// reversal plan over the longest nt serves every item (an item simply has no
// tiles in the steps at or beyond its own nt), so the whole gradient -- forward
// sweep with checkpoints, recomputation, adjoint -- is one CUDA graph.
//
// Autotuning: per order group, the thread mapping and tile height of the
// forward pair (vectorised cells, scalar cells, z-march with 8..64-row tiles)
// and of the adjoint stress pass are timed on the group's own tiles and the
// fastest kept; choices are cached in a JSON file keyed by the GPU and the
// group's shape ($FWI_PSV_TUNE_CACHE, default ~/.cache/cuda_fwi_gb300/autotune.json).
#pragma once

#include <sys/stat.h>

#include <cstdlib>
#include <fstream>
#include <sstream>

namespace fwi {

struct MultiItem {
    int nt, nzt, nxt, fpad, ppad, npml, fsurf, fdorder, tp, pitch, pnx, pnz;
    double dt, dx, dz, hc[7];
    size_t field, xstrip, zstrip, state;
    size_t off_state, off_field, off_mat, off_cpml, off_grad, off_rec, off_src;  // floats
    int nfz, nfx, wz1;
    int nsrc, nrec;
    size_t evc_f, evc_a;  // offsets of the [nxt+1] column tables
    int group;
};

struct TuneChoice {
    int fmap = 2, ftz = 0, amap = 1, atz = 0;
    double fms = 0, ams = 0;
    bool cached = false;
};

struct MultiEngine {
    int device = 0, num_sms = 1;
    cudaStream_t stream = nullptr;
    std::vector<MultiItem> items;
    int n = 0, nt_max = 0;
    size_t total_state = 0, total_field = 0, total_mat = 0, total_cpml = 0, total_grad = 0;
    size_t total_rec = 0, total_src = 0;
    DBuf d_fwd, d_adj, d_ws, d_wr, d_ux, d_uz, d_grad, d_mat, d_cpml, d_srcsig, d_rec, d_resid, d_obs;
    DBuf d_rowmis, d_blow, d_snap, d_items_f, d_items_a, d_evcol, d_ev, d_evx, d_err, d_rows;
    DBuf d_mmaps, d_gids;   // TMA maps per model; member lists of the groups (events)
    bool mmaps_built = false;
    // Copy-free checkpointing (every group on the TMA tiles): buffer k < slots
    // is checkpoint memory, buffer `slots` is d_fwd; per buffer and model the
    // maps of that buffer's forward state and descriptors writing to it.
    DBuf d_mmaps_b, d_items_b;
    int mmaps_b_slots = -1;
    struct Group {
        int fp = 0;
        std::vector<int> members;  // item indices, nt descending
        TuneChoice tune;
        KernelSet kf{}, ka{};
        TmaMultiSet tm{};
        int gid_off = 0;  // this group's member list in d_gids
        DBuf tiles_f, tiles_a;
        std::vector<int> cum_f, cum_a;  // tiles of the first k members
        int occ_f = 1, occ_v = 1, occ_a = 1;
    };
    std::vector<std::unique_ptr<Group>> groups;
    int slots_req = 32, slots = 0, use_graphs = 1, tune_on = 1;
    std::vector<Action> plan;
    long long plan_cost = 0;
    std::map<std::string, cudaGraphExec_t> graphs;
    std::map<std::string, int64_t> graph_launches;
    int64_t launches_now = 0;
    fwi_psv_stats stats{};
    bool tuned = false;
    std::vector<int> row_item;  // receiver rows (all items) -> item

    ~MultiEngine() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        if (stream) cudaStreamDestroy(stream);
    }
    int bind() {
        CUDA_TRY(cudaSetDevice(device));
        return FWI_OK;
    }
    void drop_graphs() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }

    // ---- set-up ------------------------------------------------------------
    int init(int nm, const fwi_psv_model* m, int dev) {
        if (nm < 1 || !m) return fail(FWI_ERR_INVALID, "empty model list");
        device = dev;
        FWI_TRY(bind());
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
        n = nm;
        items.resize(n);
        std::vector<float> mat_h, cpml_h, src_h;
        for (int b = 0; b < n; b++) {
            const fwi_psv_desc& d = m[b].grid;
            MultiItem& I = items[b];
            I.nt = d.nt; I.nzt = d.nzt; I.nxt = d.nxt; I.fpad = d.fpad; I.ppad = d.ppad; I.npml = d.npml;
            I.fsurf = d.fsurf ? 1 : 0; I.fdorder = d.fdorder; I.dt = d.dt; I.dx = d.dx; I.dz = d.dz;
            std::memcpy(I.hc, d.hc, sizeof I.hc);
            const std::string tag = "model " + std::to_string(b) + ": ";
            if (d.fdorder < 2 || d.fdorder > 12 || (d.fdorder & 1) || d.fpad != d.fdorder / 2)
                return fail(FWI_ERR_INVALID, tag + "fdorder must be even in 2..12 with fpad = fdorder/2");
            if (d.npml < 0 || d.ppad != d.npml + d.fpad) return fail(FWI_ERR_INVALID, tag + "ppad != npml + fpad");
            if (d.nt < 1 || !(d.dt > 0) || !(d.dx > 0) || !(d.dz > 0)) return fail(FWI_ERR_INVALID, tag + "nt, dt, dx, dz");
            if (d.nxt < 2 * d.ppad + 2 || d.nzt < (I.fsurf ? d.ppad + d.fpad + 2 : 2 * d.ppad + 2))
                return fail(FWI_ERR_INVALID, tag + "grid too small");
            if (!m[b].lam || !m[b].mu || !m[b].rho) return fail(FWI_ERR_INVALID, tag + "null material array");
            I.tp = 2 * (I.npml + 1);
            I.pitch = (int)round_up(I.nxt, 32);
            I.pnx = I.nxt - 2 * I.ppad + I.fpad - 1;
            I.pnz = I.fsurf ? I.nzt - 2 * I.ppad + I.fpad - 2 : I.nzt - 2 * I.ppad + I.fpad - 1;
            I.field = (size_t)I.nzt * I.pitch;
            I.xstrip = round_up((size_t)I.nzt * I.tp, 32);
            I.zstrip = (size_t)I.tp * I.pitch;
            I.state = round_up(5 * I.field + 4 * I.xstrip + 4 * I.zstrip, 64);
            I.wz1 = I.fsurf ? I.fpad : 0;
            I.nfz = I.nzt - I.wz1;
            I.nfx = I.nxt;
            I.off_state = total_state;
            total_state += I.state;
            I.off_field = total_field;
            total_field += I.field;
            I.off_mat = total_mat;
            total_mat += 5 * I.field;
            I.off_cpml = total_cpml;
            total_cpml += round_up(12 * (size_t)I.tp, 32);
            I.off_grad = total_grad;
            total_grad += round_up(3 * (size_t)I.nfz * I.nfx, 32);
            I.nsrc = m[b].nsrc;
            I.nrec = m[b].nrec;
            I.off_src = total_src;
            total_src += (size_t)std::max(I.nsrc, 1) * I.nt;
            I.off_rec = total_rec;
            total_rec += (size_t)std::max(I.nrec, 1) * I.nt;
            nt_max = std::max(nt_max, I.nt);
            for (int i = 0; i < I.nsrc; i++)
                if (m[b].src_x[i] < I.fpad || m[b].src_x[i] >= I.nxt - I.fpad || m[b].src_z[i] < I.fpad ||
                    m[b].src_z[i] >= I.nzt - I.fpad)
                    return fail(FWI_ERR_INVALID, tag + "source outside the interior");
            for (int i = 0; i < I.nrec; i++)
                if (m[b].rec_x[i] < I.fpad || m[b].rec_x[i] >= I.nxt - I.fpad || m[b].rec_z[i] < I.fpad ||
                    m[b].rec_z[i] >= I.nzt - I.fpad)
                    return fail(FWI_ERR_INVALID, tag + "receiver outside the interior");
            // CPML profile (index npml must be the identity, as for the single-model engine)
            std::vector<float> cp(round_up(12 * (size_t)I.tp, 32), 0.f);
            if (I.npml > 0) {
                if (!d.a || !d.b || !d.K || !d.a_half || !d.b_half || !d.K_half)
                    return fail(FWI_ERR_INVALID, tag + "CPML profiles are required when npml > 0");
                if (d.a[I.npml] != 0.0 || d.a_half[I.npml] != 0.0 || d.K[I.npml] != 1.0 || d.K_half[I.npml] != 1.0)
                    return fail(FWI_ERR_UNSUPPORTED, tag + "CPML profile index npml must be damping-free");
                for (int i = 0; i < I.tp; i++) {
                    cp[0 * I.tp + i] = (float)d.a[i];
                    cp[1 * I.tp + i] = (float)d.b[i];
                    cp[2 * I.tp + i] = (float)(1.0 / d.K[i]);
                    cp[3 * I.tp + i] = (float)d.a_half[i];
                    cp[4 * I.tp + i] = (float)d.b_half[i];
                    cp[5 * I.tp + i] = (float)(1.0 / d.K_half[i]);
                }
                interleave_cpml(cp.data(), I.tp);
            }
            cpml_h.insert(cpml_h.end(), cp.begin(), cp.end());
            // materials, dt-scaled (the same FP64 averages as fwi_psv_set_model_lmr)
            const size_t na = (size_t)(I.nzt - 1) * (I.nxt - 1);
            std::vector<double> mz(na), rz(na), rx(na);
            average_parameters(I.nzt, I.nxt, m[b].mu, m[b].rho, mz.data(), rz.data(), rx.data());
            std::vector<float> h(5 * I.field, 0.f);
            for (int iz = 0; iz < I.nzt; iz++)
                for (int ix = 0; ix < I.nxt; ix++) {
                    const size_t o = (size_t)iz * I.pitch + ix, c = (size_t)iz * I.nxt + ix;
                    h[o] = (float)(I.dt * m[b].lam[c]);
                    h[I.field + o] = (float)(2.0 * I.dt * m[b].mu[c]);
                    if (iz < I.nzt - 1 && ix < I.nxt - 1) {
                        const size_t a = (size_t)iz * (I.nxt - 1) + ix;
                        h[2 * I.field + o] = (float)(I.dt * mz[a]);
                        h[3 * I.field + o] = (float)(I.dt * rx[a]);
                        h[4 * I.field + o] = (float)(I.dt * rz[a]);
                    }
                }
            mat_h.insert(mat_h.end(), h.begin(), h.end());
            std::vector<float> s((size_t)std::max(I.nsrc, 1) * I.nt, 0.f);
            for (size_t i = 0; i < (size_t)I.nsrc * I.nt; i++) s[i] = (float)m[b].src_signal[i];
            src_h.insert(src_h.end(), s.begin(), s.end());
        }
        FWI_TRY(d_mat.ensure(mat_h.size() * 4));
        FWI_TRY(d_cpml.ensure(cpml_h.size() * 4 + 16));
        FWI_TRY(d_srcsig.ensure(src_h.size() * 4));
        CUDA_TRY(cudaMemcpy(d_mat.p, mat_h.data(), mat_h.size() * 4, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_cpml.p, cpml_h.data(), cpml_h.size() * 4, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_srcsig.p, src_h.data(), src_h.size() * 4, cudaMemcpyHostToDevice));
        // buffers
        FWI_TRY(d_fwd.ensure(total_state * 4));
        FWI_TRY(d_adj.ensure(total_state * 4));
        for (DBuf* b : {&d_ws, &d_wr, &d_ux, &d_uz}) FWI_TRY(b->ensure(total_field * 4));
        FWI_TRY(d_grad.ensure(total_grad * 4));
        FWI_TRY(d_rec.ensure(total_rec * 4));
        FWI_TRY(d_resid.ensure(total_rec * 4));
        FWI_TRY(d_obs.ensure(total_rec * 4));
        FWI_TRY(d_err.ensure(16));
        CUDA_TRY(cudaMemset(d_err.p, 0, 16));
        FWI_TRY(d_blow.ensure(16));
        // events (sources then receivers of each column, sorted as the single-model engine does)
        struct Ev { int x, z, kind, idx, code; };
        std::vector<int> cols_f, cols_a, evx;
        std::vector<int2> evf, eva;
        size_t nrows = 0;
        for (int b = 0; b < n; b++) nrows += items[b].nrec;
        row_item.assign(nrows, 0);
        std::vector<int2> ev_all;  // flat forward then adjoint entries share one array
        std::vector<Ev> all_f, all_a;
        size_t row0 = 0;
        for (int b = 0; b < n; b++) {
            MultiItem& I = items[b];
            std::vector<Ev> ef, ea;
            for (int i = 0; i < I.nsrc; i++) ef.push_back({m[b].src_x[i], m[b].src_z[i], 0, i, i});
            for (int r = 0; r < I.nrec; r++) {
                ef.push_back({m[b].rec_x[r], m[b].rec_z[r], 1, r, ~r});
                ea.push_back({m[b].rec_x[r], m[b].rec_z[r], 0, r, r});
                row_item[row0 + r] = b;
            }
            row0 += I.nrec;
            auto cmp = [](const Ev& u, const Ev& v) {
                if (u.x != v.x) return u.x < v.x;
                if (u.z != v.z) return u.z < v.z;
                if (u.kind != v.kind) return u.kind < v.kind;
                return u.idx < v.idx;
            };
            std::sort(ef.begin(), ef.end(), cmp);
            std::sort(ea.begin(), ea.end(), cmp);
            auto fill = [&](std::vector<Ev>& ev, std::vector<int>& cols, size_t* off) {
                *off = cols.size();
                const int base = (int)ev_all.size();
                size_t k = 0;
                for (int x = 0; x <= I.nxt; x++) {
                    while (k < ev.size() && ev[k].x < x) k++;
                    cols.push_back(base + (int)k);
                }
                for (auto& e : ev) {
                    ev_all.push_back(make_int2(e.z, e.code));
                    evx.push_back(e.x);
                }
            };
            fill(ef, cols_f, &I.evc_f);
            fill(ea, cols_a, &I.evc_a);
        }
        const size_t ncols_f = cols_f.size();
        cols_f.insert(cols_f.end(), cols_a.begin(), cols_a.end());
        for (int b = 0; b < n; b++) items[b].evc_a += ncols_f;
        FWI_TRY(d_evcol.ensure(cols_f.size() * 4));
        FWI_TRY(d_ev.ensure(std::max<size_t>(1, ev_all.size()) * 8));
        FWI_TRY(d_evx.ensure(std::max<size_t>(1, evx.size()) * 4));
        CUDA_TRY(cudaMemcpy(d_evcol.p, cols_f.data(), cols_f.size() * 4, cudaMemcpyHostToDevice));
        if (!ev_all.empty()) {
            CUDA_TRY(cudaMemcpy(d_ev.p, ev_all.data(), ev_all.size() * 8, cudaMemcpyHostToDevice));
            CUDA_TRY(cudaMemcpy(d_evx.p, evx.data(), evx.size() * 4, cudaMemcpyHostToDevice));
        }
        FWI_TRY(d_rowmis.ensure(std::max<size_t>(1, nrows) * 8));
        // descriptors
        std::vector<ItemDesc> itf(n), ita(n);
        for (int b = 0; b < n; b++) {
            fill_item(itf[b], b, false);
            fill_item(ita[b], b, true);
        }
        FWI_TRY(d_items_f.ensure(n * sizeof(ItemDesc)));
        FWI_TRY(d_items_a.ensure(n * sizeof(ItemDesc)));
        CUDA_TRY(cudaMemcpy(d_items_f.p, itf.data(), n * sizeof(ItemDesc), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_items_a.p, ita.data(), n * sizeof(ItemDesc), cudaMemcpyHostToDevice));
        // groups by half order, members by nt descending
        std::map<int, int> gidx;
        for (int b = 0; b < n; b++) {
            auto it = gidx.find(items[b].fpad);
            if (it == gidx.end()) {
                it = gidx.emplace(items[b].fpad, (int)groups.size()).first;
                groups.emplace_back(new Group());
                groups.back()->fp = items[b].fpad;
            }
            items[b].group = it->second;
            groups[it->second]->members.push_back(b);
        }
        for (auto& g : groups)
            std::stable_sort(g->members.begin(), g->members.end(),
                             [&](int u, int v) { return items[u].nt > items[v].nt; });
        std::vector<int> gids;
        for (auto& g : groups) {
            g->gid_off = (int)gids.size();
            gids.insert(gids.end(), g->members.begin(), g->members.end());
        }
        FWI_TRY(d_gids.ensure(gids.size() * 4));
        CUDA_TRY(cudaMemcpy(d_gids.p, gids.data(), gids.size() * 4, cudaMemcpyHostToDevice));
        for (auto& g : groups) FWI_TRY(apply_choice(*g, g->tune));
        return FWI_OK;
    }

    // The maps of a model's forward state held at fwd_base (+ its offset):
    // the stress pass, the velocity pass and the adjoint pass's forward fields.
    int forward_maps(MultiMaps& M, int b, float* fwd_base) {
        const MultiItem& I = items[b];
        const int FPv = I.fpad, hx = (FPv + 3) / 4 * 4;
        const int wx = kTmaTX + 2 * hx, wz = kTmaTZ + 2 * FPv;
        const size_t rb = (size_t)I.pitch * 4, sb = I.state * 4, f = I.field;
        float* sf = fwd_base + I.off_state;
        const int X = I.nxt, Z = I.nzt;
        FWI_TRY(make_map(&M.sf.vx, sf + F_VX * f, X, Z, 1, rb, sb, wx, wz));
        FWI_TRY(make_map(&M.sf.vz, sf + F_VZ * f, X, Z, 1, rb, sb, wx, wz));
        FWI_TRY(make_map(&M.sf.sxx, sf + F_SXX * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
        FWI_TRY(make_map(&M.sf.szx, sf + F_SZX * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
        FWI_TRY(make_map(&M.sf.szz, sf + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
        FWI_TRY(make_map(&M.vf.sxx, sf + F_SXX * f, X, Z, 1, rb, sb, wx, kTmaTZ));
        FWI_TRY(make_map(&M.vf.szx, sf + F_SZX * f, X, Z, 1, rb, sb, wx, wz));
        FWI_TRY(make_map(&M.vf.szz, sf + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, wz));
        FWI_TRY(make_map(&M.vf.vx, sf + F_VX * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
        FWI_TRY(make_map(&M.vf.vz, sf + F_VZ * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
        FWI_TRY(make_map(&M.a.fvx, sf + F_VX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
        FWI_TRY(make_map(&M.a.fvz, sf + F_VZ * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
        FWI_TRY(make_map(&M.a.fsxx, sf + F_SXX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
        FWI_TRY(make_map(&M.a.fszx, sf + F_SZX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
        FWI_TRY(make_map(&M.a.fszz, sf + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
        return FWI_OK;
    }

    // Tensor maps of every model's states for the TMA-staged passes (one slot
    // per map; addresses are fixed for the engine's lifetime).
    int build_mmaps() {
        if (mmaps_built) return FWI_OK;
        std::vector<MultiMaps> mm(n);
        for (int b = 0; b < n; b++) {
            const MultiItem& I = items[b];
            const int FPv = I.fpad, hx = (FPv + 3) / 4 * 4;
            const int wx = kTmaTX + 2 * hx, wz = kTmaTZ + 2 * FPv, wza = kAdjTZ + 2 * FPv;
            const size_t rb = (size_t)I.pitch * 4, sb = I.state * 4, fb = I.field * 4, f = I.field;
            const float* mat = d_mat.as<float>() + I.off_mat;
            float* sf = d_fwd.as<float>() + I.off_state;
            float* sa = d_adj.as<float>() + I.off_state;
            const int X = I.nxt, Z = I.nzt;
            MultiMaps& M = mm[b];
            FWI_TRY(make_map(&M.sf.vx, sf + F_VX * f, X, Z, 1, rb, sb, wx, wz));
            FWI_TRY(make_map(&M.sf.vz, sf + F_VZ * f, X, Z, 1, rb, sb, wx, wz));
            FWI_TRY(make_map(&M.sf.L, mat, X, Z, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&M.sf.M2, mat + f, X, Z, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&M.sf.MZ, mat + 2 * f, X, Z, 0, rb, 0, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&M.sf.sxx, sf + F_SXX * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&M.sf.szx, sf + F_SZX * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
            FWI_TRY(make_map(&M.sf.szz, sf + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
            for (int a = 0; a < 2; a++) {
                VelMaps& V = a ? M.va : M.vf;
                float* st = a ? sa : sf;
                float* we = (a ? d_wr.as<float>() : d_ws.as<float>()) + I.off_field;
                FWI_TRY(make_map(&V.sxx, st + F_SXX * f, X, Z, 1, rb, sb, wx, kTmaTZ));
                FWI_TRY(make_map(&V.szx, st + F_SZX * f, X, Z, 1, rb, sb, wx, wz));
                FWI_TRY(make_map(&V.szz, st + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, wz));
                FWI_TRY(make_map(&V.BX, mat + 3 * f, X, Z, 0, rb, 0, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&V.BZ, mat + 4 * f, X, Z, 0, rb, 0, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&V.vx, st + F_VX * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&V.vz, st + F_VZ * f, X, Z, 1, rb, sb, kTmaTX, kTmaTZ));
                FWI_TRY(make_map(&V.We, we, X, Z, 1, rb, fb, kTmaTX, kTmaTZ));
            }
            AdjMaps& A = M.a;
            FWI_TRY(make_map(&A.vx, sa + F_VX * f, X, Z, 1, rb, sb, wx, wza));
            FWI_TRY(make_map(&A.vz, sa + F_VZ * f, X, Z, 1, rb, sb, wx, wza));
            FWI_TRY(make_map(&A.L, mat, X, Z, 0, rb, 0, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.M2, mat + f, X, Z, 0, rb, 0, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.MZ, mat + 2 * f, X, Z, 0, rb, 0, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.sxx, sa + F_SXX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.szx, sa + F_SZX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.szz, sa + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.ux, d_ux.as<float>() + I.off_field, X, Z, 1, rb, fb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.uz, d_uz.as<float>() + I.off_field, X, Z, 1, rb, fb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fvx, sf + F_VX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fvz, sf + F_VZ * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fsxx, sf + F_SXX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fszx, sf + F_SZX * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
            FWI_TRY(make_map(&A.fszz, sf + F_SZZ * f, X, Z, 1, rb, sb, kTmaTX, kAdjTZ));
        }
        FWI_TRY(d_mmaps.ensure(mm.size() * sizeof(MultiMaps)));
        CUDA_TRY(cudaMemcpy(d_mmaps.p, mm.data(), mm.size() * sizeof(MultiMaps), cudaMemcpyHostToDevice));
        mmaps_built = true;
        return FWI_OK;
    }

    void fill_item(ItemDesc& d, int b, bool adj, float* fwd_base = nullptr) {
        const MultiItem& I = items[b];
        std::memset(&d, 0, sizeof d);
        d.nzt = I.nzt; d.nxt = I.nxt; d.pitch = I.pitch; d.fpad = I.fpad;
        d.ppad = I.ppad; d.npml = I.npml; d.tp = I.tp; d.pnx = I.pnx;
        d.pnz = I.pnz; d.fsurf = I.fsurf; d.nt = I.nt; d.fwi_dt = 1;
        d.fwi_dx = 1; d.fwi_dz = 1; d.wx1 = 0; d.wx2 = I.nxt;
        d.wz1 = I.wz1; d.wz2 = I.nzt; d.nfz = I.nfz; d.nfx = I.nfx;
        d.dt = (float)I.dt;
        d.inv_dt = (float)(1.0 / I.dt);
        d.gscale = (float)I.dt;
        for (int k = 0; k < kMaxHalf; k++) {
            d.hx[k] = k < I.fpad ? (float)((1.0 / I.dx) * I.hc[k + 1]) : 0.f;
            d.hz[k] = k < I.fpad ? (float)((1.0 / I.dz) * I.hc[k + 1]) : 0.f;
        }
        d.cpml = d_cpml.as<float>() + I.off_cpml;
        const float* mt = d_mat.as<float>() + I.off_mat;
        d.L = mt; d.M2 = mt + I.field; d.MZX = mt + 2 * I.field; d.BX = mt + 3 * I.field; d.BZ = mt + 4 * I.field;
        float* st = (adj ? d_adj.as<float>() : fwd_base ? fwd_base : d_fwd.as<float>()) + I.off_state;
        d.vx = st + F_VX * I.field; d.vz = st + F_VZ * I.field; d.sxx = st + F_SXX * I.field;
        d.szx = st + F_SZX * I.field; d.szz = st + F_SZZ * I.field;
        float* cp = st + 5 * I.field;
        d.mvx_x = cp; d.mvz_x = cp + I.xstrip; d.msxx_x = cp + 2 * I.xstrip; d.mszx_x = cp + 3 * I.xstrip;
        float* zp = cp + 4 * I.xstrip;
        d.mvx_z = zp; d.mvz_z = zp + I.zstrip; d.mszz_z = zp + 2 * I.zstrip; d.mszx_z = zp + 3 * I.zstrip;
        d.We = (adj ? d_wr.as<float>() : d_ws.as<float>()) + I.off_field;
        d.ev_col = d_evcol.as<int>() + (adj ? I.evc_a : I.evc_f);
        d.ev = d_ev.as<int2>();
        d.ev_x = d_evx.as<int>();
        d.inj = adj ? d_resid.as<float>() + I.off_rec : d_srcsig.as<float>() + I.off_src;
        d.rec = d_rec.as<float>() + I.off_rec;
        d.store = nullptr;
        if (adj) {
            d.ux = d_ux.as<float>() + I.off_field;
            d.uz = d_uz.as<float>() + I.off_field;
            const size_t nf = (size_t)I.nfz * I.nfx;
            d.glam = d_grad.as<float>() + I.off_grad;
            d.gmu = d.glam + nf;
            d.grho = d.gmu + nf;
            d.fwd_kind = 1;
            d.fwd = d_fwd.as<float>() + I.off_state;
            d.fwd_fs = (long long)I.field;
        }
    }

    // tiles of a group for a mapping (map 0: tz rows per tile; cell maps: their
    // own height; 3: the TMA tiles, 128 x 16 forward and 128 x 8 adjoint)
    int plan_group(Group& g, int map, int tz, DBuf& buf, std::vector<int>& cum, bool adj) {
        const int rows = map == 0 ? tz : map == 3 ? (adj ? kAdjTZ : kTmaTZ) : MapDims<2>::rows;
        std::vector<Tile> t;
        cum.assign(1, 0);
        for (int b : g.members) {
            const MultiItem& I = items[b];
            for (int x0 = 0; x0 < I.nxt; x0 += kTileX)
                for (int z0 = I.fpad; z0 < I.nzt - I.fpad; z0 += rows)
                    t.push_back({b, x0, z0, std::min(z0 + rows, I.nzt - I.fpad)});
            cum.push_back((int)t.size());
        }
        if (buf.p && buf.bytes < t.size() * sizeof(Tile)) drop_graphs();
        FWI_TRY(buf.ensure(std::max<size_t>(1, t.size()) * sizeof(Tile)));
        CUDA_TRY(cudaMemcpy(buf.p, t.data(), t.size() * sizeof(Tile), cudaMemcpyHostToDevice));
        return FWI_OK;
    }

    int apply_choice(Group& g, const TuneChoice& c) {
        g.tune = c;
        g.kf = kernels_for(g.fp, c.fmap == 3 ? 1 : c.fmap);
        g.ka = kernels_for(g.fp, c.amap == 3 ? 1 : c.amap);
        g.occ_f = std::max(1, g.kf.occ_f());
        g.occ_v = std::max(1, g.kf.occ_v());
        g.occ_a = std::max(1, g.ka.occ_a());
        if (c.fmap == 3 || c.amap == 3) {
            FWI_TRY(build_mmaps());
            g.tm = tma_multi_for(g.fp);
            CUDA_TRY(g.tm.prepare());
        }
        FWI_TRY(plan_group(g, c.fmap == 3 ? 3 : g.kf.map, c.ftz, g.tiles_f, g.cum_f, false));
        FWI_TRY(plan_group(g, c.amap == 3 ? 3 : g.ka.map, c.atz, g.tiles_a, g.cum_a, true));
        drop_graphs();
        return FWI_OK;
    }

    bool copy_free() const {
        if (slots <= 0) return false;
        for (auto& g : groups)
            if (g->tune.fmap != 3 || g->tune.amap != 3) return false;
        return true;
    }
    float* buf(int k) { return k < slots ? snap(k) : d_fwd.as<float>(); }
    // per-buffer maps and descriptors of the copy-free plan (rebuilt when the
    // slot count or the checkpoint memory changes)
    int build_buffers() {
        if (mmaps_b_slots == slots) return FWI_OK;
        FWI_TRY(build_mmaps());
        std::vector<MultiMaps> base(n);
        CUDA_TRY(cudaMemcpy(base.data(), d_mmaps.p, n * sizeof(MultiMaps), cudaMemcpyDeviceToHost));
        const int nbuf = slots + 1;
        std::vector<MultiMaps> mm((size_t)nbuf * n);
        std::vector<ItemDesc> it((size_t)nbuf * n);
        for (int k = 0; k < nbuf; k++)
            for (int b = 0; b < n; b++) {
                MultiMaps& M = mm[(size_t)k * n + b];
                M = base[b];
                FWI_TRY(forward_maps(M, b, buf(k)));
                fill_item(it[(size_t)k * n + b], b, false, buf(k));
            }
        drop_graphs();
        FWI_TRY(d_mmaps_b.ensure(mm.size() * sizeof(MultiMaps)));
        FWI_TRY(d_items_b.ensure(it.size() * sizeof(ItemDesc)));
        CUDA_TRY(cudaMemcpy(d_mmaps_b.p, mm.data(), mm.size() * sizeof(MultiMaps), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(d_items_b.p, it.data(), it.size() * sizeof(ItemDesc), cudaMemcpyHostToDevice));
        mmaps_b_slots = slots;
        return FWI_OK;
    }
    // One recompute step of every active model from buffer x into buffer y
    // (x == y: in place); see the single-model engine's step_bufs.
    void step_bufs(int x, int y, int it) {
        const MultiMaps* mx = d_mmaps_b.as<MultiMaps>() + (size_t)x * n;
        const MultiMaps* my = d_mmaps_b.as<MultiMaps>() + (size_t)y * n;
        const ItemDesc* itm = d_items_b.as<ItemDesc>() + (size_t)y * n;
        const long long msrc = (long long)(buf(x) - buf(y));
        int* err = d_err.as<int>();
        for (auto& gp : groups) {
            Group& g = *gp;
            const int k = active(g, it);
            if (k == 0) continue;
            const int ns = g.cum_f[k];
            const dim3 gs((unsigned)std::max(1, std::min(ns, num_sms)));
            g.tm.stress(gs, stream, mx, my, itm, g.tiles_f.as<Tile>(), ns, it, 0u, 0, msrc, err);
            g.tm.velocity(gs, stream, mx, my, itm, g.tiles_f.as<Tile>(), ns, it, 0u, 0, msrc, err);
            events_list_kernel<<<k, 256, 0, stream>>>(itm, d_gids.as<int>() + g.gid_off, it, FL_INJECT);
            launches_now += 3;
        }
    }
    // The plan from action k on without state copies (the single-model
    // engine's run_plan_copy_free): RESTORE points at the slot's buffer, the
    // next ADVANCE steps out of it, SAVE swaps the working buffer with the
    // slot's free one, ADJOINT reads the forward fields from the buffer that
    // holds them.
    int run_plan_copy_free(size_t k, int last_slot, int last_state, long long* recompute) {
        std::vector<int> phys(slots);
        for (int i = 0; i < slots; i++) phys[i] = i;
        int wb = slots;
        int src = last_slot >= 0 ? phys[last_slot] : wb;
        if (last_slot < 0) CUDA_TRY(cudaMemsetAsync(buf(wb), 0, total_state * 4, stream));
        auto advance = [&](int t0, int t1) {
            for (int it = t0; it < t1; it++) {
                step_bufs(src, wb, it);
                src = wb;
            }
            *recompute += std::max(0, t1 - t0);
        };
        advance(last_state, nt_max - 1);
        for (; k < plan.size(); k++) {
            const Action& a = plan[k];
            switch (a.kind) {
                case Action::ADVANCE:
                    advance(a.a, a.b);
                    break;
                case Action::SAVE:
                    if (src == wb) {
                        std::swap(phys[a.a], wb);
                    } else {
                        FWI_TRY(state_copy(buf(phys[a.a]), buf(src)));
                    }
                    src = phys[a.a];
                    break;
                case Action::RESTORE:
                    if (a.a < 0) {
                        CUDA_TRY(cudaMemsetAsync(buf(wb), 0, total_state * 4, stream));
                        src = wb;
                    } else {
                        src = phys[a.a];
                    }
                    break;
                case Action::ADJOINT:
                    adj_src = d_mmaps_b.as<MultiMaps>() + (size_t)src * n;
                    step(true, a.a, FL_GRAD, FL_INJECT | FL_WE);
                    adj_src = nullptr;
                    break;
            }
        }
        return FWI_OK;
    }
    const MultiMaps* adj_src = nullptr;  // maps naming the forward state of the adjoint pass (null: d_fwd's)

    // number of members of g still running at time step it
    int active(const Group& g, int it) const {
        int k = 0;
        while (k < (int)g.members.size() && items[g.members[k]].nt > it) k++;
        return k;
    }

    // ---- passes ---------------------------------------------------------------
    void step(bool adj, int it, unsigned sflags, unsigned vflags) {
        const ItemDesc* itm = adj ? d_items_a.as<ItemDesc>() : d_items_f.as<ItemDesc>();
        const MultiMaps* mm = d_mmaps.as<MultiMaps>();
        int* err = d_err.as<int>();
        for (auto& gp : groups) {
            Group& g = *gp;
            const int k = active(g, it);
            if (k == 0) continue;
            const int ns = adj ? g.cum_a[k] : g.cum_f[k];
            const bool tma_s = (adj ? g.tune.amap : g.tune.fmap) == 3;
            if (tma_s) {
                const dim3 gs((unsigned)std::max(1, std::min(ns, num_sms)));
                const MultiMaps* ms = adj && adj_src ? adj_src : mm;
                (adj ? g.tm.adjoint : g.tm.stress)(gs, stream, ms, ms, itm, (adj ? g.tiles_a : g.tiles_f).as<Tile>(),
                                                   ns, it, sflags, 0, 0, err);
            } else {
                const int gs = std::max(1, std::min(ns, num_sms * (adj ? g.occ_a : g.occ_f)));
                (adj ? g.ka.stress_a : g.kf.stress_f)(dim3(gs), stream, itm,
                                                      (adj ? g.tiles_a : g.tiles_f).as<Tile>(), ns, it, sflags, err);
            }
            const int nv = g.cum_f[k];
            if (g.tune.fmap == 3) {
                // source injection / recording of the active members in a small kernel after the pass
                const unsigned ev = vflags & (FL_INJECT | FL_RECORD);
                g.tm.velocity(dim3((unsigned)std::max(1, std::min(nv, num_sms))), stream, mm, mm, itm,
                              g.tiles_f.as<Tile>(), nv, it, vflags & ~ev, adj ? 1 : 0, 0, err);
                if (ev) {
                    events_list_kernel<<<k, 256, 0, stream>>>(itm, d_gids.as<int>() + g.gid_off, it, ev);
                    launches_now++;
                }
            } else {
                const int gv = std::max(1, std::min(nv, num_sms * g.occ_v));
                g.kf.velocity(dim3(gv), stream, itm, g.tiles_f.as<Tile>(), nv, it, vflags, err);
            }
            launches_now += 2;
        }
    }
    void forward_steps(int t0, int t1, bool record) {
        for (int it = t0; it < t1; it++)
            step(false, it, 0u, FL_INJECT | (record ? (FL_RECORD | FL_WE) : 0u));
    }
    int state_copy(float* dst, const float* src) {
        CUDA_TRY(device_copy(dst, src, total_state, num_sms, stream));
        return FWI_OK;
    }
    float* snap(int s) { return d_snap.as<float>() + (size_t)s * total_state; }

    template <class F>
    int run_phase(const std::string& key, F&& body) {
        if (!use_graphs) {
            FWI_TRY(body());
            CUDA_TRY(cudaGetLastError());
            return FWI_OK;
        }
        auto itg = graphs.find(key);
        if (itg == graphs.end()) {
            const int64_t before = launches_now;
            CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            const int st = body();
            cudaGraph_t gph = nullptr;
            cudaError_t ec = cudaStreamEndCapture(stream, &gph);
            if (st != FWI_OK) {
                if (gph) cudaGraphDestroy(gph);
                return st;
            }
            if (ec != cudaSuccess) return fail(FWI_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
            cudaGraphExec_t ex = nullptr;
            ec = cudaGraphInstantiate(&ex, gph, 0);
            cudaGraphDestroy(gph);
            if (ec != cudaSuccess) return fail(FWI_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ec));
            itg = graphs.emplace(key, ex).first;
            graph_launches[key] = launches_now - before;
            launches_now = before;
        }
        launches_now += graph_launches[key];
        CUDA_TRY(cudaGraphLaunch(itg->second, stream));
        return FWI_OK;
    }

    // ---- autotuning -------------------------------------------------------------
    static std::string cache_path() {
        const char* e = std::getenv("FWI_PSV_TUNE_CACHE");
        if (e && *e) return e;
        const char* h = std::getenv("HOME");
        return std::string(h && *h ? h : ".") + "/.cache/cuda_fwi_gb300/autotune.json";
    }
    std::string tune_key(const Group& g) const {
        cudaDeviceProp pr{};
        cudaGetDeviceProperties(&pr, device);
        size_t cells = 0;
        int nx_max = 0;
        for (int b : g.members) {
            cells += (size_t)items[b].nzt * items[b].nxt;
            nx_max = std::max(nx_max, items[b].nxt);
        }
        int cb = 0, xb = 0;
        while ((size_t(1) << (cb + 1)) <= cells) cb++;
        while ((1 << (xb + 1)) <= nx_max) xb++;
        std::string name = pr.name;
        for (char& c : name)
            if (c == '"' || c == '\\') c = '_';
        return name + "|sm" + std::to_string(num_sms) + "|fp" + std::to_string(g.fp) + "|cells2^" +
               std::to_string(cb) + "|nx2^" + std::to_string(xb);
    }
    // The cache file: one JSON object, one entry per line, as written below.
    static std::map<std::string, TuneChoice> read_cache(const std::string& path) {
        std::map<std::string, TuneChoice> out;
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line)) {
            const size_t q0 = line.find('"'), q1 = q0 == std::string::npos ? q0 : line.find('"', q0 + 1);
            if (q1 == std::string::npos) continue;
            TuneChoice c;
            auto num = [&](const char* k, double def) {
                const size_t p = line.find(std::string("\"") + k + "\":", q1);
                return p == std::string::npos ? def : std::atof(line.c_str() + p + std::strlen(k) + 3);
            };
            c.fmap = (int)num("fwd_map", -1);
            c.ftz = (int)num("fwd_tz", 0);
            c.amap = (int)num("adj_map", -1);
            c.atz = (int)num("adj_tz", 0);
            c.fms = num("fwd_ms", 0);
            c.ams = num("adj_ms", 0);
            if (c.fmap < 0 || c.amap < 0) continue;
            c.cached = true;
            out[line.substr(q0 + 1, q1 - q0 - 1)] = c;
        }
        return out;
    }
    static void write_cache(const std::string& path, const std::map<std::string, TuneChoice>& all) {
        std::string dir = path.substr(0, path.find_last_of('/'));
        std::string cur;
        std::stringstream ss(dir);
        std::string part;
        if (!dir.empty() && dir[0] == '/') cur = "/";
        while (std::getline(ss, part, '/'))
            if (!part.empty()) {
                cur += part + "/";
                mkdir(cur.c_str(), 0755);
            }
        const std::string tmp = path + ".tmp";
        {
            std::ofstream f(tmp);
            f << "{\n";
            size_t i = 0;
            for (auto& kv : all) {
                const TuneChoice& c = kv.second;
                f << " \"" << kv.first << "\": {\"fwd_map\": " << c.fmap << ", \"fwd_tz\": " << c.ftz
                  << ", \"adj_map\": " << c.amap << ", \"adj_tz\": " << c.atz << ", \"fwd_ms\": " << c.fms
                  << ", \"adj_ms\": " << c.ams << "}" << (++i < all.size() ? "," : "") << "\n";
            }
            f << "}\n";
        }
        std::rename(tmp.c_str(), path.c_str());
    }

    // average device ms of one launch of `what` (0 forward pair, 1 adjoint stress) on all of g
    int time_group(Group& g, int what, double* ms) {
        cudaEvent_t a, b;
        CUDA_TRY(cudaEventCreate(&a));
        CUDA_TRY(cudaEventCreate(&b));
        const int k = (int)g.members.size();
        const MultiMaps* mm = d_mmaps.as<MultiMaps>();
        auto launch = [&]() {
            if (what == 0 && g.tune.fmap == 3) {
                const int ns = g.cum_f[k];
                const dim3 gs((unsigned)std::max(1, std::min(ns, num_sms)));
                g.tm.stress(gs, stream, mm, mm, d_items_f.as<ItemDesc>(), g.tiles_f.as<Tile>(), ns, 0, 0u, 0, 0,
                            d_err.as<int>());
                g.tm.velocity(gs, stream, mm, mm, d_items_f.as<ItemDesc>(), g.tiles_f.as<Tile>(), ns, 0, 0u, 0, 0,
                              d_err.as<int>());
                events_list_kernel<<<k, 256, 0, stream>>>(d_items_f.as<ItemDesc>(), d_gids.as<int>() + g.gid_off, 0,
                                                          FL_INJECT);
            } else if (what == 1 && g.tune.amap == 3) {
                const int ns = g.cum_a[k];
                g.tm.adjoint(dim3((unsigned)std::max(1, std::min(ns, num_sms))), stream, mm, mm,
                             d_items_a.as<ItemDesc>(), g.tiles_a.as<Tile>(), ns, 0, FL_GRAD, 0, 0, d_err.as<int>());
            } else if (what == 0) {
                const int ns = g.cum_f[k];
                g.kf.stress_f(dim3(std::max(1, std::min(ns, num_sms * g.occ_f))), stream, d_items_f.as<ItemDesc>(),
                              g.tiles_f.as<Tile>(), ns, 0, 0u, d_err.as<int>());
                g.kf.velocity(dim3(std::max(1, std::min(ns, num_sms * g.occ_v))), stream, d_items_f.as<ItemDesc>(),
                              g.tiles_f.as<Tile>(), ns, 0, FL_INJECT, d_err.as<int>());
            } else {
                const int ns = g.cum_a[k];
                g.ka.stress_a(dim3(std::max(1, std::min(ns, num_sms * g.occ_a))), stream, d_items_a.as<ItemDesc>(),
                              g.tiles_a.as<Tile>(), ns, 0, FL_GRAD, d_err.as<int>());
            }
        };
        for (int r = 0; r < 2; r++) launch();
        CUDA_TRY(cudaEventRecord(a, stream));
        const int reps = 6;
        for (int r = 0; r < reps; r++) launch();
        CUDA_TRY(cudaEventRecord(b, stream));
        CUDA_TRY(cudaEventSynchronize(b));
        float t = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&t, a, b));
        CUDA_TRY(cudaGetLastError());
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        *ms = t / reps;
        return FWI_OK;
    }

    int autotune() {
        FWI_TRY(bind());
        const std::string path = cache_path();
        auto cache = read_cache(path);
        bool dirty = false;
        for (auto& gp : groups) {
            Group& g = *gp;
            const std::string key = tune_key(g);
            auto hit = cache.find(key);
            if (hit != cache.end()) {
                FWI_TRY(apply_choice(g, hit->second));
                continue;
            }
            TuneChoice best;
            best.fms = best.ams = 1e30;
            std::vector<std::pair<int, int>> fc, ac;
            fc.push_back({3, 0});
            if (g.fp <= 4) fc.push_back({2, 0});
            fc.push_back({1, 0});
            for (int tz : {8, 16, 32, 64}) fc.push_back({0, tz});
            ac.push_back({3, 0});
            ac.push_back({1, 0});
            for (int tz : {16, 32}) ac.push_back({0, tz});
            for (auto& f : fc) {
                TuneChoice c = g.tune;
                c.fmap = f.first;
                c.ftz = f.second;
                FWI_TRY(apply_choice(g, c));
                double ms = 0;
                FWI_TRY(time_group(g, 0, &ms));
                if (ms < best.fms) {
                    best.fms = ms;
                    best.fmap = c.fmap;
                    best.ftz = c.ftz;
                }
            }
            for (auto& f : ac) {
                TuneChoice c = g.tune;
                c.amap = f.first;
                c.atz = f.second;
                FWI_TRY(apply_choice(g, c));
                double ms = 0;
                FWI_TRY(time_group(g, 1, &ms));
                if (ms < best.ams) {
                    best.ams = ms;
                    best.amap = c.amap;
                    best.atz = c.atz;
                }
            }
            FWI_TRY(apply_choice(g, best));
            cache[key] = best;
            dirty = true;
        }
        // the timing runs wrote into the states and gradients: start clean
        CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, total_state * 4, stream));
        CUDA_TRY(cudaMemsetAsync(d_adj.p, 0, total_state * 4, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        if (dirty) write_cache(path, cache);
        tuned = true;
        return FWI_OK;
    }

    // ---- forward modelling only -------------------------------------------------
    int forward(double* const* rec_out) {
        FWI_TRY(bind());
        // the mappings of gradient(), so a forward and a gradient of one engine
        // compute the same traces bit for bit
        if (tune_on && !tuned) FWI_TRY(autotune());
        launches_now = 0;
        FWI_TRY(run_phase("fwdonly", [&]() -> int {
            CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, total_state * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_ws.p, 0, total_field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_rec.p, 0, total_rec * 4, stream));
            forward_steps(0, nt_max, true);
            return FWI_OK;
        }));
        std::vector<float> h(total_rec);
        CUDA_TRY(cudaMemcpyAsync(h.data(), d_rec.p, total_rec * 4, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        int flag = 0;
        FWI_TRY(check_bounds_record());
        CUDA_TRY(cudaMemcpy(&flag, d_err.p, 4, cudaMemcpyDeviceToHost));
        if (flag) return fail(FWI_ERR_CUDA, "a kernel raised its error flag; results discarded");
        for (int b = 0; b < n; b++)
            if (rec_out && rec_out[b])
                for (size_t i = 0; i < (size_t)items[b].nrec * items[b].nt; i++)
                    rec_out[b][i] = h[items[b].off_rec + i];
        stats = fwi_psv_stats{};
        stats.launches = launches_now;
        stats.forward_steps = nt_max;
        stats.batch = n;
        return FWI_OK;
    }

    // ---- gradient ---------------------------------------------------------------
    int gradient(const double* const* obs, double* misfit, double* const* gl, double* const* gm,
                 double* const* gr) {
        FWI_TRY(bind());
        if (!obs) return fail(FWI_ERR_INVALID, "observed data required");
        if (tune_on && !tuned) FWI_TRY(autotune());
        // slots of the common reversal plan over the longest nt
        int want = slots_req > 0 ? std::min(slots_req, nt_max - 1) : 0;
        if (slots_req == 0) {
            size_t fr = 0, tot = 0;
            CUDA_TRY(cudaMemGetInfo(&fr, &tot));
            want = (int)std::min<long long>(nt_max - 1, (long long)(0.8 * fr / (total_state * 4.0)));
        }
        want = std::max(0, want);
        if (want != slots || plan.empty()) {
            slots = want;
            if (slots > 0) {
                if (d_snap.bytes < (size_t)slots * total_state * 4) {
                    drop_graphs();
                    FWI_TRY(d_snap.ensure((size_t)slots * total_state * 4));
                    // the copy-free plan steps into any checkpoint buffer: cells that
                    // no pass writes (grid borders) must read as zero there too
                    CUDA_TRY(cudaMemset(d_snap.p, 0, (size_t)slots * total_state * 4));
                    mmaps_b_slots = -1;
                }
            }
            plan = plan_binomial(nt_max, slots, &plan_cost);
            drop_graphs();
        }
        // observed data (FP32, per model [nrec][nt])
        {
            std::vector<float> h(total_rec, 0.f);
            for (int b = 0; b < n; b++) {
                const MultiItem& I = items[b];
                if (!obs[b] && I.nrec) return fail(FWI_ERR_INVALID, "observed data of model " + std::to_string(b));
                for (size_t i = 0; i < (size_t)I.nrec * I.nt; i++) h[I.off_rec + i] = (float)obs[b][i];
            }
            CUDA_TRY(cudaMemcpyAsync(d_obs.p, h.data(), total_rec * 4, cudaMemcpyHostToDevice, stream));
            CUDA_TRY(cudaStreamSynchronize(stream));
        }
        const bool cfree = copy_free();
        if (cfree) FWI_TRY(build_buffers());
        cudaEvent_t e0, e1;
        CUDA_TRY(cudaEventCreate(&e0));
        CUDA_TRY(cudaEventCreate(&e1));
        launches_now = 0;
        CUDA_TRY(cudaEventRecord(e0, stream));
        std::vector<std::pair<int, int>> saves;
        for (auto& a : plan) {
            if (a.kind == Action::ADJOINT) break;
            if (a.kind == Action::SAVE) saves.push_back({a.b, a.a});
        }
        const std::string sk = "|s" + std::to_string(slots) + (cfree ? "|cf" : "");
        FWI_TRY(run_phase("fwd" + sk, [&]() -> int {
            CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, total_state * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_ws.p, 0, total_field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_rec.p, 0, total_rec * 4, stream));
            int t = 0;
            for (auto& sv : saves) {
                forward_steps(t, sv.first, true);
                t = sv.first;
                FWI_TRY(state_copy(snap(sv.second), d_fwd.as<float>()));
            }
            forward_steps(t, nt_max, true);
            return FWI_OK;
        }));
        // residuals and per-row misfits, one small launch per model
        CUDA_TRY(cudaMemsetAsync(d_blow.p, 0, 4, stream));
        FWI_TRY(d_rows.ensure(std::max<size_t>(1, row_item.size()) * 4));
        {
            std::vector<int> rr(row_item.size());
            size_t r0 = 0;
            for (int b = 0; b < n; b++) {
                for (int r = 0; r < items[b].nrec; r++) rr[r0 + r] = r;
                r0 += items[b].nrec;
            }
            if (!rr.empty())
                CUDA_TRY(cudaMemcpyAsync(d_rows.p, rr.data(), rr.size() * 4, cudaMemcpyHostToDevice, stream));
            r0 = 0;
            for (int b = 0; b < n; b++) {
                const MultiItem& I = items[b];
                if (I.nrec)
                    residual_kernel<<<I.nrec, 256, 0, stream>>>(
                        d_rec.as<float>() + I.off_rec, d_obs.as<float>() + I.off_rec, d_rows.as<int>() + r0,
                        d_resid.as<float>() + I.off_rec, d_rowmis.as<double>() + r0, d_blow.as<int>(), I.nt,
                        0.5 * I.dt);
                r0 += I.nrec;
                launches_now++;
            }
        }
        long long recompute = 0;
        FWI_TRY(run_phase("bwd" + sk, [&]() -> int {
            CUDA_TRY(cudaMemsetAsync(d_adj.p, 0, total_state * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_wr.p, 0, total_field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_ux.p, 0, total_field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_uz.p, 0, total_field * 4, stream));
            CUDA_TRY(cudaMemsetAsync(d_grad.p, 0, total_grad * 4, stream));
            size_t k = 0;
            int last_slot = -1, last_state = 0;
            while (k < plan.size() && plan[k].kind != Action::ADJOINT) {
                if (plan[k].kind == Action::SAVE) {
                    last_slot = plan[k].a;
                    last_state = plan[k].b;
                }
                k++;
            }
            if (cfree) return run_plan_copy_free(k, last_slot, last_state, &recompute);
            if (last_slot >= 0) FWI_TRY(state_copy(d_fwd.as<float>(), snap(last_slot)));
            else CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, total_state * 4, stream));
            forward_steps(last_state, nt_max - 1, false);
            recompute += (nt_max - 1) - last_state;
            for (; k < plan.size(); k++) {
                const Action& a = plan[k];
                switch (a.kind) {
                    case Action::ADVANCE:
                        forward_steps(a.a, a.b, false);
                        recompute += a.b - a.a;
                        break;
                    case Action::SAVE:
                        FWI_TRY(state_copy(snap(a.a), d_fwd.as<float>()));
                        break;
                    case Action::RESTORE:
                        if (a.a < 0) CUDA_TRY(cudaMemsetAsync(d_fwd.p, 0, total_state * 4, stream));
                        else FWI_TRY(state_copy(d_fwd.as<float>(), snap(a.a)));
                        break;
                    case Action::ADJOINT:
                        step(true, a.a, FL_GRAD, FL_INJECT | FL_WE);
                        break;
                }
            }
            return FWI_OK;
        }));
        CUDA_TRY(cudaEventRecord(e1, stream));
        // results
        std::vector<double> rm(row_item.size());
        std::vector<float> g(total_grad);
        int blow = 0;
        if (!rm.empty())
            CUDA_TRY(cudaMemcpyAsync(rm.data(), d_rowmis.p, rm.size() * 8, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaMemcpyAsync(&blow, d_blow.p, 4, cudaMemcpyDeviceToHost, stream));
        const bool want_g = gl || gm || gr;
        if (want_g) CUDA_TRY(cudaMemcpyAsync(g.data(), d_grad.p, total_grad * 4, cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        int flag = 0;
        FWI_TRY(check_bounds_record());
        CUDA_TRY(cudaMemcpy(&flag, d_err.p, 4, cudaMemcpyDeviceToHost));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (flag) return fail(FWI_ERR_CUDA, "a kernel raised its error flag; results discarded");
        size_t r0 = 0;
        for (int b = 0; b < n; b++) {
            double s = 0.0;
            for (int r = 0; r < items[b].nrec; r++) s += rm[r0 + r];
            r0 += items[b].nrec;
            if (misfit) misfit[b] = s;
        }
        for (int b = 0; b < n && want_g; b++) {
            const MultiItem& I = items[b];
            const size_t nf = (size_t)I.nfz * I.nfx;
            double* outs[3] = {gl ? gl[b] : nullptr, gm ? gm[b] : nullptr, gr ? gr[b] : nullptr};
            for (int q = 0; q < 3; q++) {
                if (!outs[q]) continue;
                const float* src = g.data() + I.off_grad + q * nf;
                for (int iz = 0; iz < I.nzt; iz++)
                    for (int ix = 0; ix < I.nxt; ix++)
                        outs[q][(size_t)iz * I.nxt + ix] = iz < I.wz1 ? 0.0 : (double)src[(size_t)(iz - I.wz1) * I.nfx + ix];
            }
        }
        stats = fwi_psv_stats{};
        stats.launches = launches_now;
        stats.forward_steps = nt_max;
        (void)recompute;  // counted while the body runs; a graph replay runs the same plan
        stats.recompute_steps = plan_recompute_steps(plan, nt_max, false);
        stats.adjoint_steps = nt_max;
        stats.device_bytes = (int64_t)(d_fwd.bytes + d_adj.bytes + d_snap.bytes + 4 * d_ws.bytes + d_grad.bytes +
                                       d_mat.bytes + 3 * d_rec.bytes);
        stats.snapshots = slots;
        stats.last_backward_ms = ms;
        stats.batch = n;
        if (blow) return fail(FWI_ERR_DIVERGED, "|syn - obs| exceeded 1e10");
        return FWI_OK;
    }
};

}  // namespace fwi
