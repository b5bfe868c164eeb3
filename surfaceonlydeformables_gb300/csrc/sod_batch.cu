// sod_batch.cu -- batched assembly of many objects of uneven size in persistent launches under a
// CUDA graph.
//
// A batch collects objects (mesh, material, Laplace frequencies, device outputs).  finalize():
//   * picks every object's scatter CTA size with the mesh autotuner and builds its colourings;
//   * lays out one FP64 singular side buffer for all (object, frequency) pairs and the per-star-
//     entry result buffers of the double-float singular passes;
//   * builds the work lists, largest objects first: (object, frequency, star-entry block) items for
//     the singular passes, (object, field vertex, frequency) items for one persistent launch per
//     (pass, CTA size, occupancy, point table) class of the regular passes, whose kernel arguments
//     travel in kernel-parameter space (up to BATCH_OBJS objects per launch);
//   * captures the whole step into a CUDA graph with two concurrent chains:
//       0: polar (G, B) -> combine -> G scatter (B_trans / B_angular fused in),
//       1: Guiggiani (H) -> combine -> H scatter.
// run() replays the graph on the context's stream: one host call per step, no per-object launches.
#include <algorithm>
#include <array>
#include <map>
#include <memory>
#include <numeric>
#include <tuple>
#include <vector>

#include "sod_internal.h"

namespace sod {
constexpr int KMASK_ALL = 15;
struct RegularDeleter {
    void operator()(BatchRegular *r) const { batch_regular_free(r); }
};
}  // namespace sod
using namespace sod;

struct sod_batch {
    sod_context *ctx = nullptr;
    int mask = 0;
    int out_dtype = SOD_C64;
    struct Obj {
        const sod_mesh *mesh;
        double c1, c2, rho;
        std::vector<double> s;
        int order, subdiv, sorder, ssub;
        void *out[4];
        int T[2];
    };
    std::vector<Obj> objs;
    bool ready = false;
    DevBuf dSing, dKcf, dKcd, dItems, dCounters, dS, dRes;
    struct Launch {
        int which, items_off, nitems, threads, counter, chain;
        double evals;  // kernel evaluations (regular), singular quadrature points, or vertex-frequencies
        std::shared_ptr<BatchRegular> reg;  // regular passes: kernel arguments
    };
    std::vector<Launch> launches;
    cudaStream_t cap = nullptr, cap2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~sod_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (cap) cudaStreamDestroy(cap);
        if (cap2) cudaStreamDestroy(cap2);
    }
};

// `which`: 0 polar (double-float), 1 Guiggiani (double-float), 2 G scatter (+B), 3 H scatter,
// 4 B reduction, 5 combine of G/B_trans/B_angular, 6 combine of H
static int issue_launch(sod_batch *b, const sod_batch::Launch &L, cudaStream_t st) {
    const int4 *items = b->dItems.as<int4>() + L.items_off;
    if (L.which >= 2 && L.which <= 4)
        return batch_regular_issue(b->ctx, L.reg.get(), items, L.nitems, b->dCounters.as<int>() + L.counter,
                                   b->dKcf.as<KConst<float>>(), st);
    const int which = L.which >= 5 ? 2 : L.which;
    const int mask = L.which == 6 ? (1 << SOD_H) : L.which == 5 ? (b->mask & ~(1 << SOD_H)) : b->mask;
    return sing_batch_launch(b->ctx, which, mask, b->dSing.as<SingBatchObj>(), items, L.nitems,
                             b->dKcd.as<KConst<double>>(), st);
}

static int finalize_batch(sod_batch *b) {
    sod_context *ctx = b->ctx;
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const int nobj = (int)b->objs.size();
    const bool hasG = (b->mask & (1 << SOD_G)) != 0;
    const int bmask = b->mask & ((1 << SOD_B_TRANS) | (1 << SOD_B_ANGULAR));
    // quadrature tables (deduplicated) and per-frequency constants
    std::vector<PointTable> pts;
    std::map<std::pair<int, int>, int> pt_index;
    std::vector<KConst<float>> kcf;
    std::vector<KConst<double>> kcd;
    std::vector<int> kc_off(nobj), pt_idx(nobj);
    for (int o = 0; o < nobj; o++) {
        auto &ob = b->objs[o];
        auto key = std::make_pair(ob.order, ob.subdiv);
        auto it = pt_index.find(key);
        if (it == pt_index.end()) {
            PointTable pt;
            SOD_TRY(make_point_table(ob.order, ob.subdiv, pt));
            pt_index[key] = (int)pts.size();
            pts.push_back(pt);
            it = pt_index.find(key);
        }
        pt_idx[o] = it->second;
        kc_off[o] = (int)kcd.size();
        for (size_t l = 0; l < ob.s.size() / 2; l++) {
            const KConst<double> k = make_kconst(ob.c1, ob.c2, ob.rho, ob.s[2 * l], ob.s[2 * l + 1]);
            kcd.push_back(k);
            kcf.push_back(to_float(k));
        }
        for (int kd = 0; kd < 2; kd++) {
            ob.T[kd] = 0;
            if (!(b->mask & (1 << kd))) continue;
            const int bm = kd == SOD_G ? bmask : 0;
            int T = ctx->coll_threads;
            int rc = SOD_OK;
            if (T <= 0) rc = autotune_scatter_threads(ctx, const_cast<sod_mesh *>(ob.mesh), kd, bm, &T);
            if (rc == SOD_ERR_UNSUPPORTED) T = SCATTER_GLOBAL_THREADS;  // row block too large: global accumulator
            else if (rc != SOD_OK) return rc;
            ob.T[kd] = T;
        }
    }
    // singular side buffer layout
    std::vector<std::array<long long, 4>> soff(nobj);
    long long stot = 0;
    for (int o = 0; o < nobj; o++) {
        const sod_mesh *m = b->objs[o].mesh;
        const long long nf = (long long)b->objs[o].s.size() / 2, nslots = m->nbr_off.back();
        const long long sfs[4] = {nslots * 9, nslots * 9, (long long)m->nV * 9, (long long)m->nV * 27};
        for (int kd = 0; kd < 4; kd++) {
            soff[o][kd] = stot;
            if (b->mask & (1 << kd)) stot += sfs[kd] * nf;
        }
    }
    SOD_TRY(b->dS.ensure(sizeof(cd) * (size_t)std::max<long long>(stot, 1)));
    // singular passes: geometry tables (built once per mesh and rule), per-star-entry result buffers
    std::vector<SingBatchObj> sing(nobj);
    std::vector<size_t> roff(nobj), goff(nobj);
    size_t rtot = 0;
    for (int o = 0; o < nobj; o++) {
        const sod_mesh *m = b->objs[o].mesh;
        const int nstar = m->star_off.back(), nf = (int)b->objs[o].s.size() / 2;
        roff[o] = rtot;
        rtot += sing_result_elems(b->mask, nstar, nf, false);
        goff[o] = rtot;
        rtot += sing_result_elems(b->mask, nstar, nf, true);
    }
    SOD_TRY(b->dRes.ensure(sizeof(double2) * std::max<size_t>(rtot, 1)));
    for (int o = 0; o < nobj; o++) {
        auto &ob = b->objs[o];
        const sod_mesh *m = ob.mesh;
        const sod_mesh::SingGeom *g = nullptr;
        SOD_TRY(const_cast<sod_mesh *>(m)->sing_geom_for(ob.sorder, ob.ssub, ctx->stream, &g));
        SingBatchObj &d = sing[o];
        d = SingBatchObj{};
        d.nV = m->nV;
        d.nstar = m->star_off.back();
        d.nq2 = g->nq2;
        d.polar = g->polar.as<float2>();
        d.guig = g->guig.as<float2>();
        d.guig_sub = g->guig_sub.as<double>();
        d.star_off = m->dStarOff.as<int>();
        d.star_face = m->dStarFace.as<int>();
        d.star_slot = m->dStarSlot.as<int>();
        d.nbr_off = m->dNbrOff.as<int>();
        d.N = m->dN.as<double>();
        d.Rp = b->dRes.as<double2>() + roff[o];
        d.Rg = b->dRes.as<double2>() + goff[o];
        const long long nslots = m->nbr_off.back();
        const long long sfs[4] = {nslots * 9, nslots * 9, (long long)m->nV * 9, (long long)m->nV * 27};
        for (int kd = 0; kd < 4; kd++) {
            d.S[kd] = (b->mask & (1 << kd)) ? b->dS.as<cd>() + soff[o][kd] : nullptr;
            d.S_fstride[kd] = sfs[kd];
        }
        d.kc_off = kc_off[o];
        d.nf = (int)ob.s.size() / 2;
    }
    SOD_TRY(b->dSing.ensure(sizeof(SingBatchObj) * nobj));
    SOD_CHECK_CUDA(cudaMemcpy(b->dSing.p, sing.data(), sizeof(SingBatchObj) * nobj, cudaMemcpyHostToDevice));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));  // geometry tables are complete before capture
    SOD_TRY(b->dKcf.ensure(sizeof(KConst<float>) * kcf.size()));
    SOD_TRY(b->dKcd.ensure(sizeof(KConst<double>) * kcd.size()));
    SOD_CHECK_CUDA(cudaMemcpy(b->dKcf.p, kcf.data(), sizeof(KConst<float>) * kcf.size(), cudaMemcpyHostToDevice));
    SOD_CHECK_CUDA(cudaMemcpy(b->dKcd.p, kcd.data(), sizeof(KConst<double>) * kcd.size(), cudaMemcpyHostToDevice));
    // work lists, objects ordered by decreasing face count (largest items first)
    std::vector<int> order(nobj);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return b->objs[x].mesh->nF > b->objs[y].mesh->nF; });
    std::vector<int4> items;
    b->launches.clear();
    // singular items: (object, frequency, first star entry) blocks of 128 entries, or (object,
    // frequency, first vertex) blocks of 4 vertices for the combine
    auto add_sing = [&](int which, int chain) {
        const int off = (int)items.size();
        const bool comb = which >= 5;
        double evals = 0;
        for (int o : order) {
            const auto &ob = b->objs[o];
            const int nstar = ob.mesh->star_off.back(), nV = ob.mesh->nV, nf = (int)ob.s.size() / 2;
            const int nq = ob.sorder * ob.ssub;
            const int n = comb ? nV : nstar, step = comb ? 4 : 128;
            for (int fq = 0; fq < nf; fq++)
                for (int x = 0; x < n; x += step) items.push_back(make_int4(o, fq, x, 0));
            evals += comb ? (double)nf * nV : (double)nf * nstar * nq * nq;
        }
        const int n = (int)items.size() - off;
        if (n > 0) b->launches.push_back({which, off, n, 128, (int)b->launches.size(), chain, evals, nullptr});
    };
    if (b->mask & (KMASK_ALL & ~(1 << SOD_H))) {
        add_sing(0, 0);
        add_sing(5, 0);
    }
    if (b->mask & (1 << SOD_H)) {
        add_sing(1, 1);
        add_sing(6, 1);
    }
    // regular passes: one persistent launch per (pass, CTA size, occupancy, point table) class and
    // per BATCH_OBJS objects; a launch shares one dynamic smem size, so small objects are not
    // grouped with large ones that would lower their resident CTAs per SM
    auto add_regular = [&](int which, int chain) -> int {
        const int kind = which == 3 ? SOD_H : SOD_G;
        const int bm = which == 3 ? 0 : bmask;
        // class key (-CTAs per SM, T, point table); per_sm = 1 << 20 marks objects whose row block
        // does not fit in shared memory (accumulators in global memory, a class of their own)
        constexpr int GLOBAL_CLASS = 1 << 20;
        std::map<std::tuple<int, int, int>, std::vector<int>> classes;
        for (int o : order) {
            const auto &ob = b->objs[o];
            int T = 256, per_sm = 0;
            if (which != 4) {
                T = ob.T[kind];
                SOD_TRY(scatter_occupancy(ctx, kind, bm, true, T, scatter_smem_bytes(kind, bm, ob.mesh->nV, T), &per_sm));
                if (per_sm <= 0) {
                    T = SCATTER_GLOBAL_THREADS;
                    per_sm = GLOBAL_CLASS;
                }
            }
            classes[std::make_tuple(-per_sm, T, pt_idx[o])].push_back(o);
        }
        for (auto &c : classes) {
            const int T = std::get<1>(c.first), pi = std::get<2>(c.first);
            const bool global = -std::get<0>(c.first) == GLOBAL_CLASS;
            const auto &members = c.second;
            for (size_t g0 = 0; g0 < members.size(); g0 += BATCH_OBJS) {
                const size_t g1 = std::min(members.size(), g0 + (size_t)BATCH_OBJS);
                size_t sm = 0;
                long long nit = 0;
                for (size_t g = g0; g < g1; g++) {
                    const auto &ob = b->objs[members[g]];
                    if (which != 4) sm = std::max(sm, scatter_smem_bytes(kind, bm, ob.mesh->nV, T));
                    nit += (long long)ob.mesh->nV * (long long)(ob.s.size() / 2);
                }
                std::shared_ptr<BatchRegular> reg;
                if (global) {
                    int grc = SOD_OK;
                    reg.reset(batch_regular_new_global(ctx, which, b->mask, sm, (int)std::min<long long>(nit, 1 << 30),
                                                       pts[pi], &grc),
                              RegularDeleter());
                    SOD_TRY(grc);
                } else {
                    reg.reset(batch_regular_new(which, b->mask, T, sm, pts[pi]), RegularDeleter());
                }
                const int off = (int)items.size();
                double evals = 0;
                for (size_t g = g0; g < g1; g++) {
                    const int o = members[g];
                    const auto &ob = b->objs[o];
                    const sod_mesh *m = ob.mesh;
                    cd *S[4];
                    for (int kd = 0; kd < 4; kd++) S[kd] = b->dS.as<cd>() + soff[o][kd];
                    const sod_mesh::Coloured *col = nullptr;
                    if (which != 4) SOD_TRY(const_cast<sod_mesh *>(m)->coloured_for(T, &col));
                    int slot = 0;
                    SOD_TRY(batch_regular_add(reg.get(), m, b->out_dtype, ob.out, S, col, kc_off[o], &slot));
                    const int nf = (int)ob.s.size() / 2;
                    for (int fq = 0; fq < nf; fq++)
                        for (int i = 0; i < m->nV; i++) items.push_back(make_int4(slot, i, fq, 0));
                    evals += (double)nf * ((double)m->nV * m->nF - 3.0 * m->nF) * pts[pi].n;
                }
                const int n = (int)items.size() - off;
                if (n > 0) b->launches.push_back({which, off, n, T, (int)b->launches.size(), chain, evals, reg});
            }
        }
        return SOD_OK;
    };
    if (hasG) SOD_TRY(add_regular(2, 0));
    if (b->mask & (1 << SOD_H)) SOD_TRY(add_regular(3, 1));
    if (!hasG && bmask) SOD_TRY(add_regular(4, 0));
    SOD_TRY(b->dItems.ensure(sizeof(int4) * std::max<size_t>(items.size(), 1)));
    SOD_CHECK_CUDA(cudaMemcpy(b->dItems.p, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
    SOD_TRY(b->dCounters.ensure(sizeof(int) * std::max<size_t>(b->launches.size(), 1)));
    // capture the step into a CUDA graph: fork chain 1 onto a second stream, join at the end
    if (!b->cap) SOD_CHECK_CUDA(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
    if (!b->cap2) SOD_CHECK_CUDA(cudaStreamCreateWithFlags(&b->cap2, cudaStreamNonBlocking));
    if (!b->fork) SOD_CHECK_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    if (!b->join) SOD_CHECK_CUDA(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming));
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    SOD_CHECK_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    int rc = SOD_OK;
    cudaError_t ce = cudaEventRecord(b->fork, b->cap);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->cap2, b->fork, 0);
    if (ce != cudaSuccess) rc = SOD_ERR_CUDA;
    for (const auto &L : b->launches) {
        if (rc != SOD_OK) break;
        rc = issue_launch(b, L, L.chain ? b->cap2 : b->cap);
    }
    if (rc == SOD_OK) {
        ce = cudaEventRecord(b->join, b->cap2);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->cap, b->join, 0);
        if (ce != cudaSuccess) rc = SOD_ERR_CUDA;
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce_end = cudaStreamEndCapture(b->cap, &g);
    if (rc != SOD_OK) {
        if (g) cudaGraphDestroy(g);
        if (rc == SOD_ERR_CUDA && ce != cudaSuccess) set_error(cudaGetErrorString(ce));
        return rc;
    }
    SOD_CHECK_CUDA(ce_end);
    b->graph = g;
    SOD_CHECK_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->ready = true;
    return SOD_OK;
}

extern "C" {

int sod_batch_create(sod_context *ctx, int kind_mask, int out_dtype, sod_batch **out) {
    SOD_REQUIRE(ctx && out, "null argument");
    SOD_REQUIRE(kind_mask > 0 && kind_mask <= KMASK_ALL, "kind mask must select at least one of G, H, B_trans, B_angular");
    SOD_REQUIRE(out_dtype == SOD_C128 || out_dtype == SOD_C64, "output dtype must be complex128 or complex64");
    auto *b = new sod_batch();
    b->ctx = ctx;
    b->mask = kind_mask;
    b->out_dtype = out_dtype;
    *out = b;
    return SOD_OK;
}

int sod_batch_add(sod_batch *b, const sod_mesh *mesh, double c1, double c2, double rho, const double *s, int nfreq,
                  int order, int subdiv, int sorder, int ssub, void *out_G, void *out_H, void *out_B_trans,
                  void *out_B_angular) {
    SOD_REQUIRE(b && mesh && mesh->ctx == b->ctx, "bad batch or mesh");
    SOD_REQUIRE(s && nfreq >= 1, "need at least one Laplace frequency");
    SOD_REQUIRE(c1 > 0 && c2 > 0 && rho > 0 && std::isfinite(c1) && std::isfinite(c2) && std::isfinite(rho),
                "wave speeds and density must be positive and finite");
    SOD_REQUIRE(sorder >= 1 && sorder <= 5 && ssub >= 1 && ssub <= 8, "singular quadrature order must be 1..5, subdivision 1..8");
    PointTable pt;
    SOD_TRY(make_point_table(order, subdiv, pt));
    void *outs[4] = {out_G, out_H, out_B_trans, out_B_angular};
    for (int kd = 0; kd < 4; kd++) {
        if (!(b->mask & (1 << kd))) continue;
        SOD_REQUIRE(outs[kd] != nullptr && is_device_pointer(outs[kd]), "batch outputs must be device memory");
    }
    for (int l = 0; l < nfreq; l++)
        SOD_REQUIRE(std::isfinite(s[2 * l]) && std::isfinite(s[2 * l + 1]) && (s[2 * l] != 0.0 || s[2 * l + 1] != 0.0),
                    "Laplace frequencies must be finite and non-zero");
    sod_batch::Obj o{mesh, c1, c2, rho, std::vector<double>(s, s + 2 * (size_t)nfreq), order, subdiv, sorder, ssub,
                     {out_G, out_H, out_B_trans, out_B_angular}, {0, 0}};
    b->objs.push_back(std::move(o));
    b->ready = false;
    return SOD_OK;
}

int sod_batch_finalize(sod_batch *b) {
    SOD_REQUIRE(b && !b->objs.empty(), "empty batch");
    return finalize_batch(b);
}

int sod_batch_run(sod_batch *b) {
    SOD_REQUIRE(b, "null batch");
    if (!b->ready) SOD_TRY(finalize_batch(b));
    SOD_CHECK_CUDA(cudaSetDevice(b->ctx->device));
    SOD_CHECK_CUDA(cudaGraphLaunch(b->exec, b->ctx->stream));
    b->ctx->count((int)b->launches.size());
    return SOD_OK;
}

int sod_batch_launch_count(const sod_batch *b) { return b ? (int)b->launches.size() : -1; }

int sod_batch_profile(sod_batch *b, int cap, int *which, double *evals, float *ms) {
    SOD_REQUIRE(b && cap >= 0, "null batch or negative capacity");
    if (!b->ready) SOD_TRY(finalize_batch(b));
    const int n = (int)b->launches.size();
    SOD_REQUIRE(cap >= n && which && evals && ms, "output arrays must hold sod_batch_launch_count() entries");
    SOD_CHECK_CUDA(cudaSetDevice(b->ctx->device));
    std::vector<cudaEvent_t> ev(n + 1, nullptr);
    int rc = SOD_OK;
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) rc = SOD_ERR_CUDA;
    if (rc == SOD_OK && cudaEventRecord(ev[0], b->ctx->stream) != cudaSuccess) rc = SOD_ERR_CUDA;
    for (int k = 0; k < n && rc == SOD_OK; k++) {
        rc = issue_launch(b, b->launches[k], b->ctx->stream);
        if (rc == SOD_OK && cudaEventRecord(ev[k + 1], b->ctx->stream) != cudaSuccess) rc = SOD_ERR_CUDA;
    }
    if (rc == SOD_OK && cudaEventSynchronize(ev[n]) != cudaSuccess) rc = SOD_ERR_CUDA;
    for (int k = 0; k < n && rc == SOD_OK; k++) {
        which[k] = b->launches[k].which;
        evals[k] = b->launches[k].evals;
        if (cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]) != cudaSuccess) rc = SOD_ERR_CUDA;
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (rc != SOD_OK) set_error("batch profiling: a CUDA event call failed");
    return rc;
}

int sod_batch_destroy(sod_batch *b) {
    if (b) {
        cudaSetDevice(b->ctx->device);
        delete b;
    }
    return SOD_OK;
}

}  // extern "C"
