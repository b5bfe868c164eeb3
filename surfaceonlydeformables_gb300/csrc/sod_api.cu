// sod_api.cu -- C ABI, context and mesh management of the GB300 CQBEM library.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <random>
#include <set>

#include "sod_internal.h"

namespace sod {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }

// ---- quadrature tables ----------------------------------------------------------------------
// Triangle rules of Cowper (1973), degrees 1..5, as in include/integrator.hpp:61-88 of the
// reference ({l0, l1, l2, weight}, weights summing to 1), plus the 13-point degree-7 rule
// (Cowper 1973 / Dunavant 1985) whose digits were fixed by solving its moment equations.
static const double TRI1[][4] = {{1. / 3., 1. / 3., 1. / 3., 1.}};
static const double TRI2[][4] = {{0., .5, .5, 1. / 3.}, {.5, 0., .5, 1. / 3.}, {.5, .5, 0., 1. / 3.}};
static const double TRI3[][4] = {{1. / 3., 1. / 3., 1. / 3., -27. / 48.},
                                 {11. / 15., 2. / 15., 2. / 15., 25. / 48.},
                                 {2. / 15., 11. / 15., 2. / 15., 25. / 48.},
                                 {2. / 15., 2. / 15., 11. / 15., 25. / 48.}};
static constexpr double QA4 = 0.445948490915965, QB4 = 0.111690794839005 * 2., QC4 = 0.091576213509771,
                        QD4 = 0.054975871827661 * 2.;
static const double TRI4[][4] = {{1. - 2. * QA4, QA4, QA4, QB4}, {QA4, 1. - 2. * QA4, QA4, QB4},
                                 {QA4, QA4, 1. - 2. * QA4, QB4}, {1. - 2. * QC4, QC4, QC4, QD4},
                                 {QC4, 1. - 2. * QC4, QC4, QD4}, {QC4, QC4, 1. - 2. * QC4, QD4}};
static constexpr double QA5 = 0.470142064105115, QB5 = 0.0661970763942530 * 2., QC5 = 0.101286507323456,
                        QD5 = 0.0629695902724135 * 2.;
static const double TRI5[][4] = {{1. / 3., 1. / 3., 1. / 3., 9. / 40.}, {1. - 2. * QA5, QA5, QA5, QB5},
                                 {QA5, 1. - 2. * QA5, QA5, QB5},         {QA5, QA5, 1. - 2. * QA5, QB5},
                                 {1. - 2. * QC5, QC5, QC5, QD5},         {QC5, 1. - 2. * QC5, QC5, QD5},
                                 {QC5, QC5, 1. - 2. * QC5, QD5}};
static const double TRI7[][4] = {
    {3.3333333333333333333e-1, 3.3333333333333333333e-1, 3.3333333333333333333e-1, -1.4957004446768175063e-1},
    {4.7930806784192034615e-1, 2.6034596607903982693e-1, 2.6034596607903982693e-1, 1.7561525743320781175e-1},
    {2.6034596607903982693e-1, 4.7930806784192034615e-1, 2.6034596607903982693e-1, 1.7561525743320781175e-1},
    {2.6034596607903982693e-1, 2.6034596607903982693e-1, 4.7930806784192034615e-1, 1.7561525743320781175e-1},
    {8.6973979419556837692e-1, 6.5130102902215811538e-2, 6.5130102902215811538e-2, 5.334723560883849127e-2},
    {6.5130102902215811538e-2, 8.6973979419556837692e-1, 6.5130102902215811538e-2, 5.334723560883849127e-2},
    {6.5130102902215811538e-2, 6.5130102902215811538e-2, 8.6973979419556837692e-1, 5.334723560883849127e-2},
    {4.8690315425316411793e-2, 3.1286549600487386141e-1, 6.384441885698097268e-1, 7.711376089025714026e-2},
    {4.8690315425316411793e-2, 6.384441885698097268e-1, 3.1286549600487386141e-1, 7.711376089025714026e-2},
    {3.1286549600487386141e-1, 4.8690315425316411793e-2, 6.384441885698097268e-1, 7.711376089025714026e-2},
    {3.1286549600487386141e-1, 6.384441885698097268e-1, 4.8690315425316411793e-2, 7.711376089025714026e-2},
    {6.384441885698097268e-1, 4.8690315425316411793e-2, 3.1286549600487386141e-1, 7.711376089025714026e-2},
    {6.384441885698097268e-1, 3.1286549600487386141e-1, 4.8690315425316411793e-2, 7.711376089025714026e-2}};

const double (*tri_rule_table(int order, int &n))[4] {
    switch (order) {
    case 1: n = 1; return TRI1;
    case 2: n = 3; return TRI2;
    case 3: n = 4; return TRI3;
    case 4: n = 6; return TRI4;
    case 5: n = 7; return TRI5;
    case 7: n = 13; return TRI7;
    default: n = 0; return nullptr;
    }
}

// 1-D Gauss-Legendre on [-1,1] (include/integrator.hpp:117-133 of the reference)
static const double GL1[][2] = {{0., 2.}};
static const double GL2[][2] = {{-0.5773502691896257645092, 1.}, {0.5773502691896257645092, 1.}};
static const double GL3[][2] = {{-0.7745966692414833770359, 0.5555555555555555555556},
                                {0., 0.8888888888888888888889},
                                {0.7745966692414833770359, 0.555555555555555555556}};
static const double GL4[][2] = {{-0.861136311594052575224, 0.3478548451374538573731},
                                {-0.3399810435848562648027, 0.6521451548625461426269},
                                {0.3399810435848562648027, 0.6521451548625461426269},
                                {0.861136311594052575224, 0.3478548451374538573731}};
static const double GL5[][2] = {{-0.9061798459386639927976, 0.2369268850561890875143},
                                {-0.5384693101056830910363, 0.4786286704993664680413},
                                {0., 0.5688888888888888888889},
                                {0.5384693101056830910363, 0.4786286704993664680413},
                                {0.9061798459386639927976, 0.2369268850561890875143}};
const double (*gl_rule_table(int order, int &n))[2] {
    switch (order) {
    case 1: n = 1; return GL1;
    case 2: n = 2; return GL2;
    case 3: n = 3; return GL3;
    case 4: n = 4; return GL4;
    case 5: n = 5; return GL5;
    default: n = 0; return nullptr;
    }
}

// Sub-triangles of a uniform subdivision in the order of include/integrator.hpp:24-51; each as the
// face barycentrics of its three corners.
static void subtriangles(int n, std::vector<std::array<double, 9>> &out) {
    auto bc = [&](double a, double b) { return std::array<double, 3>{1.0 - a - b, a, b}; };
    auto push = [&](std::array<double, 3> A, std::array<double, 3> B, std::array<double, 3> C) {
        out.push_back({A[0], A[1], A[2], B[0], B[1], B[2], C[0], C[1], C[2]});
    };
    const double h = 1.0 / n;
    push(bc(0, 0), bc(h, 0), bc(0, h));
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            if (!(i == 0 && j == 0) && i + j < n) push(bc(i * h, j * h), bc((i + 1) * h, j * h), bc(i * h, (j + 1) * h));
            if (i + j < n - 1)
                push(bc((i + 1) * h, (j + 1) * h), bc((i + 1) * h, j * h), bc(i * h, (j + 1) * h));
        }
}

int make_point_table(int order, int subdiv, PointTable &pt, PointTableD *ptd) {
    int nq = 0;
    const double(*rule)[4] = tri_rule_table(order, nq);
    SOD_REQUIRE(rule != nullptr, "triangle quadrature order must be 1..5 or 7 (13-point rule)");
    SOD_REQUIRE(subdiv >= 1 && subdiv <= 4, "quadrature subdivision must be 1..4");
    std::vector<std::array<double, 9>> st;
    subtriangles(subdiv, st);
    SOD_REQUIRE((int)st.size() * nq <= MAX_TRI_PTS, "too many quadrature points");
    pt.n = 0;
    if (ptd) ptd->n = 0;
    const double ws = 1.0 / ((double)subdiv * subdiv);
    for (const auto &t : st)
        for (int q = 0; q < nq; q++) {
            double l[3];
            for (int c = 0; c < 3; c++) l[c] = rule[q][0] * t[c] + rule[q][1] * t[3 + c] + rule[q][2] * t[6 + c];
            pt.p[pt.n++] = make_float4((float)l[0], (float)l[1], (float)l[2], (float)(rule[q][3] * ws));
            if (ptd) ptd->p[ptd->n++] = PointD{l[0], l[1], l[2], rule[q][3] * ws};
        }
    return SOD_OK;
}

int make_unit_gauss(int order, int subdiv, GaussTable &g) {
    int n = 0;
    const double(*r)[2] = gl_rule_table(order, n);
    SOD_REQUIRE(r != nullptr && subdiv >= 1 && n * subdiv <= 20, "bad 1-D Gauss order/subdivision");
    g.n = 0;
    for (int s = 0; s < subdiv; s++) {
        const double a = (double)s / subdiv, b = (double)(s + 1) / subdiv;
        for (int q = 0; q < n; q++) {
            g.x[g.n] = (b - a) * r[q][0] / 2. + (a + b) / 2.;
            g.w[g.n] = r[q][1] * (b - a) / 2.;
            g.n++;
        }
    }
    return SOD_OK;
}

KConst<double> make_kconst(double c1, double c2, double rho, double sr, double si) {
    KConst<double> k;
    k.ic1 = 1.0 / c1;
    k.ic2 = 1.0 / c2;
    k.ic1s = 1.0 / (c1 * c1);
    k.ic2s = 1.0 / (c2 * c2);
    k.kappa = (c2 * c2) / (c1 * c1);
    k.six_c2s = 6.0 * c2 * c2;
    k.inv4pirho = 1.0 / (4.0 * M_PI * rho);
    k.inv4pi = 1.0 / (4.0 * M_PI);
    k.sr = sr;
    k.si = si;
    const double d = sr * sr + si * si;
    k.isr = sr / d;
    k.isi = -si / d;
    k.sc1r = sr / c1, k.sc1i = si / c1;
    k.sc2r = sr / c2, k.sc2i = si / c2;
    k.is2r = k.isr * k.isr - k.isi * k.isi, k.is2i = 2.0 * k.isr * k.isi;
    k.c2sq = c2 * c2;
    return k;
}
KConst<float> to_float(const KConst<double> &k) {
    KConst<float> f;
    f.ic1 = (float)k.ic1, f.ic2 = (float)k.ic2, f.ic1s = (float)k.ic1s, f.ic2s = (float)k.ic2s;
    f.kappa = (float)k.kappa, f.six_c2s = (float)k.six_c2s, f.inv4pirho = (float)k.inv4pirho;
    f.inv4pi = (float)k.inv4pi, f.sr = (float)k.sr, f.si = (float)k.si, f.isr = (float)k.isr, f.isi = (float)k.isi;
    f.sc1r = (float)k.sc1r, f.sc1i = (float)k.sc1i, f.sc2r = (float)k.sc2r, f.sc2i = (float)k.sc2i;
    f.is2r = (float)k.is2r, f.is2i = (float)k.is2i, f.c2sq = (float)k.c2sq;
    return f;
}

static bool is_device_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

bool is_device_pointer(const void *p) { return is_device_ptr(p); }

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister, mapped into the
// device address space), or null for device, managed or pageable memory.
static void *mapped_host_ptr(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

template <class T> static int upload(DevBuf &b, const std::vector<T> &v) {
    SOD_TRY(b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1)));
    if (!v.empty()) SOD_CHECK_CUDA(cudaMemcpy(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return SOD_OK;
}

static int check_context(const sod_context *ctx) {
    if (!ctx) {
        set_error("null context");
        return SOD_ERR_INVALID_ARG;
    }
    return SOD_OK;
}

// Face records: 4 float4 = {y1, area}, {y2, nx}, {y3, ny}, {nz, j0, j1, j2 (int bits)}
static void face_record(const sod_mesh *m, int f, float4 *rec) {
    const int j[3] = {m->F[3 * f], m->F[3 * f + 1], m->F[3 * f + 2]};
    const double *a = &m->V[3 * j[0]], *b = &m->V[3 * j[1]], *c = &m->V[3 * j[2]];
    const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    const double vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
    const double cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    const float area = (float)(0.5 * std::sqrt(cx * cx + cy * cy + cz * cz));
    const double *n = &m->N[3 * f];
    int32_t bits[3];
    std::memcpy(bits, j, sizeof(bits));
    float fb[3];
    std::memcpy(fb, bits, sizeof(fb));
    rec[0] = make_float4((float)a[0], (float)a[1], (float)a[2], area);
    rec[1] = make_float4((float)b[0], (float)b[1], (float)b[2], (float)n[0]);
    rec[2] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)n[1]);
    rec[3] = make_float4((float)n[2], fb[0], fb[1], fb[2]);
}

}  // namespace sod

namespace {
// Colouring of the face conflict graph (faces sharing a vertex) with k colours of at most `cap` faces
// each, by min-conflicts local search with a tabu list: start from a random order, each face taking the
// least-conflicting colour with room, then take a conflicting face f and the best of: moving it to a
// colour with room, or swapping it with one of 16 random faces of a full colour (which keeps every
// colour's size, so k colours of exactly cap faces are reachable).  A move of f back to the colour it
// left is barred for 10-19 steps.  Deterministic for a given seed.  Returns false if conflicts remain
// after the iteration budget.
bool colour_search(const std::vector<std::vector<int>> &nbr, int nF, int k, int cap, uint64_t seed,
                   std::vector<int> &col, std::vector<int> &size) {
    if ((long long)k * cap < nF) return false;
    if ((size_t)nF * (size_t)k > ((size_t)1 << 24)) return false;  // host memory: 6 bytes per (face, colour)
    std::mt19937_64 rng(seed);
    col.assign(nF, -1);
    size.assign(k, 0);
    std::vector<int16_t> C((size_t)nF * k, 0);  // C[f k + c]: neighbours of f in colour c
    std::vector<std::vector<int>> members(k);
    std::vector<int> pos(nF, 0);
    std::vector<int> order(nF);
    std::iota(order.begin(), order.end(), 0);
    std::shuffle(order.begin(), order.end(), rng);
    long long conflicts = 0;
    auto place = [&](int f, int c) {
        col[f] = c;
        size[c]++;
        pos[f] = (int)members[c].size();
        members[c].push_back(f);
        for (int g : nbr[f]) C[(size_t)g * k + c]++;
    };
    auto take = [&](int f) {
        const int c = col[f];
        size[c]--;
        const int last = members[c].back();
        members[c][pos[f]] = last;
        pos[last] = pos[f];
        members[c].pop_back();
        for (int g : nbr[f]) C[(size_t)g * k + c]--;
    };
    for (int f : order) {
        int best = -1;
        for (int c = 0; c < k; c++) {
            if (size[c] >= cap) continue;
            if (best < 0 || C[(size_t)f * k + c] < C[(size_t)f * k + best] ||
                (C[(size_t)f * k + c] == C[(size_t)f * k + best] && size[c] < size[best]))
                best = c;
        }
        conflicts += C[(size_t)f * k + best];
        place(f, best);
    }
    auto adjacent = [&](int f, int g) { return std::binary_search(nbr[f].begin(), nbr[f].end(), g); };
    std::vector<int> tabu((size_t)nF * k, 0);  // iteration until which the move is barred
    std::vector<int> bad;
    const long long budget = 20LL * nF;  // feasible sizes converge in a few hundred steps
    for (long long it = 1; conflicts > 0 && it <= budget; it++) {
        if (bad.empty() || (it & 255) == 0) {
            bad.clear();
            for (int f = 0; f < nF; f++)
                if (C[(size_t)f * k + col[f]] > 0) bad.push_back(f);
            if (bad.empty()) break;
        }
        const size_t pick = (size_t)(rng() % bad.size());
        const int f = bad[pick];
        const int c0 = col[f];
        if (C[(size_t)f * k + c0] == 0) {  // stale entry
            bad[pick] = bad.back();
            bad.pop_back();
            continue;
        }
        int best = -1, bestg = -1;
        long long bestd = 0;
        for (int c = 0; c < k; c++) {
            if (c == c0 || tabu[(size_t)f * k + c] > it) continue;
            if (size[c] < cap) {
                const long long d = C[(size_t)f * k + c] - C[(size_t)f * k + c0];
                if (best < 0 || d < bestd) best = c, bestg = -1, bestd = d;
            } else {
                for (int t = 0; t < 16 && !members[c].empty(); t++) {
                    const int g = members[c][(size_t)(rng() % members[c].size())];
                    const int adj = adjacent(f, g) ? 1 : 0;
                    const long long d = (long long)C[(size_t)f * k + c] - C[(size_t)f * k + c0] +
                                        C[(size_t)g * k + c0] - C[(size_t)g * k + c] - 2 * adj;
                    if (best < 0 || d < bestd) best = c, bestg = g, bestd = d;
                }
            }
        }
        if (best < 0) continue;
        take(f);
        if (bestg >= 0) {
            take(bestg);
            place(bestg, c0);
        }
        place(f, best);
        conflicts += bestd;
        tabu[(size_t)f * k + c0] = (int)(it + 10 + (long long)(rng() % 10));
    }
    return conflicts == 0;
}
}  // namespace

namespace sod {
// Colouring of the faces (no two faces of a colour share a vertex, at most `threads` faces per
// colour): the balanced greedy pass, then, where it is two or more colours above ceil(nF / threads),
// the capacity search above.  Host-only; the mesh schedules and sod_face_colouring use it.
static void colour_faces_compute(const int *F, int nF, int nV, int threads, std::vector<int> &color,
                                 std::vector<int> &size) {
    std::vector<std::vector<int>> vf(nV);
    for (int f = 0; f < nF; f++)
        for (int k = 0; k < 3; k++) vf[F[3 * f + k]].push_back(f);
    color.assign(nF, -1);
    size.clear();
    std::vector<char> forbidden;
    for (int f = 0; f < nF; f++) {
        forbidden.assign(size.size(), 0);
        for (int k = 0; k < 3; k++)
            for (int g : vf[F[3 * f + k]])
                if (color[g] >= 0) forbidden[color[g]] = 1;
        int best = -1;
        for (int c = 0; c < (int)size.size(); c++)
            if (!forbidden[c] && size[c] < threads && (best < 0 || size[c] < size[best])) best = c;
        if (best < 0) {
            best = (int)size.size();
            size.push_back(0);
        }
        color[f] = best;
        size[best]++;
    }
    // lower bound: the faces around a vertex all conflict, so at least the largest valence
    int valence = 0;
    for (int v = 0; v < nV; v++) valence = std::max(valence, (int)vf[v].size());
    const int kb = std::max((nF + threads - 1) / threads, valence);
    if ((int)size.size() >= kb + 2) {  // the greedy pass is 2+ colours above the bound
        std::vector<std::vector<int>> nbr(nF);
        for (int f = 0; f < nF; f++) {
            for (int k = 0; k < 3; k++)
                for (int g : vf[F[3 * f + k]])
                    if (g != f) nbr[f].push_back(g);
            std::sort(nbr[f].begin(), nbr[f].end());
            nbr[f].erase(std::unique(nbr[f].begin(), nbr[f].end()), nbr[f].end());
        }
        const int k0 = kb;
        std::vector<int> col2, size2;
        for (int k = k0; k < (int)size.size() && k <= k0 + 2; k++)
            if (colour_search(nbr, nF, k, threads, 0x5eedull + (uint64_t)k, col2, size2)) {
                bool ok = true;  // independent check: no two faces of one colour share a vertex
                for (int f = 0; f < nF && ok; f++)
                    for (int g : nbr[f])
                        if (col2[g] == col2[f]) ok = false;
                std::vector<int> remap(size2.size(), -1), size3;  // drop empty colours
                for (int c = 0; c < (int)size2.size(); c++)
                    if (size2[c] > 0) remap[c] = (int)size3.size(), size3.push_back(size2[c]);
                for (int &c : col2) c = remap[c];
                if (ok && size3.size() < size.size()) {
                    color.swap(col2);
                    size.swap(size3);
                }
                break;
            }
    }
}

// The colouring depends only on the connectivity: objects of one topology (a request loop's spheres of
// one level, say) share it, so results are kept per (F, nV, capacity), up to 64 of them.
void colour_faces(const int *F, int nF, int nV, int threads, std::vector<int> &color, std::vector<int> &size) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the connectivity
    auto mix = [&h](uint64_t x) {
        for (int b = 0; b < 8; b++) {
            h ^= (x >> (8 * b)) & 0xff;
            h *= 1099511628211ull;
        }
    };
    mix((uint64_t)nV);
    mix((uint64_t)nF);
    mix((uint64_t)threads);
    for (int t = 0; t < 3 * nF; t++) mix((uint64_t)(uint32_t)F[t]);
    struct Entry {
        std::vector<int> F, color, size;
        int nV, threads;
    };
    static std::mutex mu;
    static std::map<uint64_t, Entry> cache;
    static std::vector<uint64_t> order;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find(h);
        if (it != cache.end() && it->second.nV == nV && it->second.threads == threads &&
            it->second.F.size() == (size_t)3 * nF && std::equal(it->second.F.begin(), it->second.F.end(), F)) {
            color = it->second.color;
            size = it->second.size;
            return;
        }
    }
    colour_faces_compute(F, nF, nV, threads, color, size);
    std::lock_guard<std::mutex> g(mu);
    if (!cache.count(h)) {
        if (order.size() >= 64) {
            cache.erase(order.front());
            order.erase(order.begin());
        }
        cache[h] = Entry{std::vector<int>(F, F + 3 * nF), color, size, nV, threads};
        order.push_back(h);
    }
}}  // namespace sod

using namespace sod;

// Colouring of faces such that faces of one colour share no vertex and no colour holds more than
// `threads` faces (one scatter round per colour, each thread one face).  A balanced greedy pass
// gives about 13 colours on a 5120-face sphere whatever the capacity above ~400 (each face conflicts
// with ~12 others); a min-conflicts search with k = ceil(nF / threads) colours (then k + 1, k + 2)
// usually reaches the capacity, so larger CTAs get fewer, fuller colours.  The fewer colours win.
int sod_mesh::coloured_for(int threads, const Coloured **out) {
    std::lock_guard<std::recursive_mutex> lock(sched_mu);
    auto it = coloured.find(threads);
    if (it != coloured.end()) {
        *out = it->second.get();
        return SOD_OK;
    }
    std::vector<int> color, size;
    colour_faces(F.data(), nF, nV, threads, color, size);
    auto C = std::make_unique<Coloured>();
    C->ncolors = (int)size.size();
    C->off.assign(C->ncolors + 1, 0);
    for (int c = 0; c < C->ncolors; c++) C->off[c + 1] = C->off[c] + size[c];
    // within a colour, faces follow the Morton order of their centroids: the lanes of a warp then
    // integrate nearby faces, so distance-dependent branches (the psi series) rarely diverge
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v = 0; v < nV; v++)
        for (int d = 0; d < 3; d++) lo[d] = std::min(lo[d], V[3 * v + d]), hi[d] = std::max(hi[d], V[3 * v + d]);
    auto spread = [](uint64_t x) {  // 10 bits -> every third bit
        x &= 0x3ff;
        x = (x | (x << 16)) & 0x30000ff;
        x = (x | (x << 8)) & 0x300f00f;
        x = (x | (x << 4)) & 0x30c30c3;
        x = (x | (x << 2)) & 0x9249249;
        return x;
    };
    std::vector<uint64_t> key(nF);
    for (int f = 0; f < nF; f++) {
        uint64_t q[3];
        for (int d = 0; d < 3; d++) {
            const double c = (V[3 * F[3 * f] + d] + V[3 * F[3 * f + 1] + d] + V[3 * F[3 * f + 2] + d]) / 3.0;
            const double t = hi[d] > lo[d] ? (c - lo[d]) / (hi[d] - lo[d]) : 0.0;
            q[d] = (uint64_t)std::min(1023.0, std::max(0.0, t * 1023.0));
        }
        key[f] = (((uint64_t)color[f]) << 32) | (spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2));
    }
    std::vector<int> order(nF);
    for (int f = 0; f < nF; f++) order[f] = f;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<float4> rec(4 * (size_t)nF);
    std::vector<int4> canon(has_vmap ? nF : 0);
    for (int p = 0; p < nF; p++) {
        const int f = order[p];
        face_record(this, f, &rec[4 * (size_t)p]);
        if (has_vmap) canon[p] = make_int4(vmap[F[3 * f]], vmap[F[3 * f + 1]], vmap[F[3 * f + 2]], 0);
    }
    SOD_TRY(upload(C->dFaces, rec));
    if (has_vmap) SOD_TRY(upload(C->dCanonF, canon));
    SOD_TRY(upload(C->dOff, C->off));
    *out = C.get();
    coloured[threads] = std::move(C);
    return SOD_OK;
}

extern "C" {

int sod_version(void) { return 1; }
const char *sod_last_error(void) { return g_last_error.c_str(); }

int sod_triangle_rule(int order, double *out, int *npts) {
    int n = 0;
    const double(*r)[4] = tri_rule_table(order, n);
    SOD_REQUIRE(r != nullptr && npts != nullptr, "unsupported triangle rule order");
    if (out) std::memcpy(out, r, sizeof(double) * 4 * n);
    *npts = n;
    return SOD_OK;
}

int sod_cq_frequencies(int bdf, double dt, int N, double *s_out, double *R_out, int *L_out) {
    SOD_REQUIRE(bdf == 1 || bdf == 2, "multistep method must be BDF1 or BDF2");
    SOD_REQUIRE(dt > 0 && N >= 1 && s_out && R_out && L_out, "bad CQ parameters");
    const double R = std::pow(1e-10, 1. / (2. * N));
    const int L = N + 1;
    for (int l = 0; l < L / 2 + 1; l++) {
        // R zeta^l with zeta = exp(2 pi i / L)
        const double ang = 2.0 * M_PI * (double)l / (double)L;
        const double wr = R * std::cos(ang), wi = R * std::sin(ang);
        double gr, gi;
        if (bdf == 1) {
            gr = 1.0 - wr, gi = -wi;
        } else {
            const double w2r = wr * wr - wi * wi, w2i = 2.0 * wr * wi;
            gr = 1.5 - 2.0 * wr + 0.5 * w2r, gi = -2.0 * wi + 0.5 * w2i;
        }
        s_out[2 * l] = gr / dt;
        s_out[2 * l + 1] = gi / dt;
    }
    *R_out = R;
    *L_out = L;
    return SOD_OK;
}

int sod_context_create(int device, sod_context **out) {
    SOD_REQUIRE(out != nullptr, "null output pointer");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return SOD_ERR_NO_DEVICE;
    }
    SOD_REQUIRE(device >= 0 && device < n, "device index out of range");
    cudaDeviceProp prop;
    SOD_CHECK_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) {
        set_error("device is not a Blackwell-class GPU (sm_103a build)");
        return SOD_ERR_NO_DEVICE;
    }
    SOD_CHECK_CUDA(cudaSetDevice(device));
    auto *ctx = new sod_context();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
        return SOD_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    if (ctx->dev_err.ensure(sizeof(int)) != SOD_OK || cudaMemset(ctx->dev_err.p, 0, sizeof(int)) != cudaSuccess) {
        cudaStreamDestroy(ctx->own_stream);
        delete ctx;
        set_error("could not allocate the context's device error word");
        return SOD_ERR_CUDA;
    }
    *out = ctx;
    return SOD_OK;
}


int sod_context_destroy(sod_context *ctx) {
    if (!ctx) return SOD_OK;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->own_stream);
        cudaStreamDestroy(ctx->own_stream);
    }
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    for (cudaEvent_t e : ctx->chunk_events) cudaEventDestroy(e);
    delete ctx;
    return SOD_OK;
}

int sod_context_set_stream(sod_context *ctx, void *stream) {
    SOD_TRY(check_context(ctx));
    ctx->stream = (cudaStream_t)stream;  // NULL: CUDA's default stream
    return SOD_OK;
}

int sod_context_synchronize(sod_context *ctx) {
    SOD_TRY(check_context(ctx));
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return take_device_error(ctx);
}

int sod_context_set_wait_test(sod_context *ctx, int stall) {
    SOD_TRY(check_context(ctx));
    ctx->wait_test = stall != 0;
    return SOD_OK;
}

int sod_context_set_tuning(sod_context *ctx, int coll_threads, int galerkin_threads) {
    SOD_TRY(check_context(ctx));
    SOD_REQUIRE(coll_threads == 0 || (coll_threads >= 32 && coll_threads <= 512 && coll_threads % 32 == 0),
                "collocation threads must be 0 or a multiple of 32 in [32, 512]");
    SOD_REQUIRE(galerkin_threads == 0 || (galerkin_threads >= 32 && galerkin_threads <= 1024 && galerkin_threads % 32 == 0),
                "Galerkin threads must be 0 or a multiple of 32 in [32, 1024]");
    ctx->coll_threads = coll_threads;
    ctx->gal_threads = galerkin_threads;
    return SOD_OK;
}

int sod_context_set_precision(sod_context *ctx, int precision) {
    SOD_TRY(check_context(ctx));
    SOD_REQUIRE(precision == SOD_PRECISION_AUTO || precision == SOD_PRECISION_FP32 ||
                    precision == SOD_PRECISION_COMPENSATED,
                "precision must be SOD_PRECISION_AUTO, _FP32 or _COMPENSATED");
    ctx->precision = precision;
    return SOD_OK;
}

int64_t sod_context_launch_count(const sod_context *ctx) { return ctx ? ctx->launches.load() : -1; }

int sod_mesh_create(sod_context *ctx, const double *V, int nV, const int *F, int nF, const double *N, const int *vmap,
                    sod_mesh **out) {
    SOD_TRY(check_context(ctx));
    SOD_REQUIRE(out && V && F, "null mesh array");
    SOD_REQUIRE(nV >= 3 && nF >= 1, "mesh needs at least 3 vertices and 1 face");
    *out = nullptr;
    auto m = std::make_unique<sod_mesh>();
    m->ctx = ctx;
    m->nV = nV;
    m->nF = nF;
    m->V.assign(V, V + 3 * (size_t)nV);
    m->F.assign(F, F + 3 * (size_t)nF);
    for (int t = 0; t < 3 * nF; t++) SOD_REQUIRE(m->F[t] >= 0 && m->F[t] < nV, "face index out of range");
    for (size_t t = 0; t < m->V.size(); t++) SOD_REQUIRE(std::isfinite(m->V[t]), "non-finite vertex coordinate");
    m->N.resize(3 * (size_t)nF);
    for (int f = 0; f < nF; f++) {
        const double *a = &m->V[3 * m->F[3 * f]], *b = &m->V[3 * m->F[3 * f + 1]], *c = &m->V[3 * m->F[3 * f + 2]];
        const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2], vx = c[0] - a[0], vy = c[1] - a[1],
                     vz = c[2] - a[2];
        double n[3] = {uy * vz - uz * vy, uz * vx - ux * vz, ux * vy - uy * vx};
        const double ln = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        SOD_REQUIRE(ln > 0.0, "degenerate (zero-area) face " + std::to_string(f));
        for (int d = 0; d < 3; d++) m->N[3 * f + d] = N ? N[3 * f + d] : n[d] / ln;
    }
    m->has_vmap = vmap != nullptr;
    if (vmap) {
        m->vmap.assign(vmap, vmap + nV);
        for (int v = 0; v < nV; v++)
            SOD_REQUIRE(m->vmap[v] >= 0 && m->vmap[v] < nV, "vertex_map_inverse entry outside [0, nV)");
    }
    auto canon = [&](int v) { return m->has_vmap ? m->vmap[v] : v; };
    // stars: for vertex i, the faces with a corner whose canonical id equals canon(i); singular
    // corner = first such corner (src/elastodynamics_cqbem_G_collocation.cu:79-88)
    std::map<int, std::vector<std::pair<int, int>>> by_canon;
    for (int f = 0; f < nF; f++) {
        std::set<int> seen;
        for (int k = 0; k < 3; k++) {
            const int c = canon(m->F[3 * f + k]);
            if (seen.insert(c).second) by_canon[c].push_back({f, k});
        }
    }
    m->star_off.assign(nV + 1, 0);
    m->nbr_off.assign(nV + 1, 0);
    size_t max_star = 0;
    for (int i = 0; i < nV; i++) {
        const auto &st = by_canon[canon(i)];
        max_star = std::max(max_star, st.size());
        std::vector<int> nb;
        for (auto &fc : st) {
            m->star_face.push_back(fc.first);
            m->star_corner.push_back(fc.second);
            for (int k = 0; k < 3; k++) nb.push_back(m->F[3 * fc.first + k]);
        }
        std::sort(nb.begin(), nb.end());
        nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
        const int base = (int)m->nbr_vert.size();
        for (auto &fc : st) {
            const int sc = fc.second;
            for (int c = 0; c < 3; c++) {
                const int j = m->F[3 * fc.first + (sc + c) % 3];
                m->star_slot.push_back(base + (int)(std::lower_bound(nb.begin(), nb.end(), j) - nb.begin()));
            }
        }
        m->nbr_vert.insert(m->nbr_vert.end(), nb.begin(), nb.end());
        m->star_off[i + 1] = (int)m->star_face.size();
        m->nbr_off[i + 1] = (int)m->nbr_vert.size();
    }
    if (max_star > 32) {
        set_error("vertex star with more than 32 faces is not supported");
        return SOD_ERR_UNSUPPORTED;
    }
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    std::vector<float> vf(m->V.begin(), m->V.end());
    std::vector<int> cv(nV);
    for (int v = 0; v < nV; v++) cv[v] = canon(v);
    SOD_TRY(upload(m->dV, m->V));
    SOD_TRY(upload(m->dN, m->N));
    SOD_TRY(upload(m->dF, m->F));
    SOD_TRY(upload(m->dVf, vf));
    SOD_TRY(upload(m->dCanon, cv));
    SOD_TRY(upload(m->dStarOff, m->star_off));
    SOD_TRY(upload(m->dStarFace, m->star_face));
    SOD_TRY(upload(m->dStarCorner, m->star_corner));
    SOD_TRY(upload(m->dStarSlot, m->star_slot));
    SOD_TRY(upload(m->dNbrOff, m->nbr_off));
    SOD_TRY(upload(m->dNbrVert, m->nbr_vert));
    std::vector<float4> rec(4 * (size_t)nF);
    std::vector<int4> cn(m->has_vmap ? nF : 0);
    for (int f = 0; f < nF; f++) {
        face_record(m.get(), f, &rec[4 * (size_t)f]);
        if (m->has_vmap) cn[f] = make_int4(canon(m->F[3 * f]), canon(m->F[3 * f + 1]), canon(m->F[3 * f + 2]), 0);
    }
    SOD_TRY(upload(m->dFacesNat, rec));
    if (m->has_vmap) SOD_TRY(upload(m->dCanonNat, cn));
    *out = m.release();
    return SOD_OK;
}

int sod_face_colouring(const int *F, int nF, int nV, int capacity, int *colour, int *ncolours) {
    SOD_REQUIRE(F && colour && ncolours && nF >= 1 && nV >= 3 && capacity >= 1, "bad face colouring arguments");
    for (int t = 0; t < 3 * nF; t++) SOD_REQUIRE(F[t] >= 0 && F[t] < nV, "face index out of range");
    std::vector<int> color, size;
    colour_faces(F, nF, nV, capacity, color, size);
    std::copy(color.begin(), color.end(), colour);
    *ncolours = (int)size.size();
    return SOD_OK;
}

int sod_mesh_destroy(sod_mesh *mesh) {
    if (mesh) {
        cudaSetDevice(mesh->ctx->device);
        delete mesh;
    }
    return SOD_OK;
}

static size_t kind_elems(int kind, int nV) {
    const size_t ncol = kind <= SOD_H ? 3 * (size_t)nV : (kind == SOD_B_TRANS ? 3 : 9);
    return 3 * (size_t)nV * ncol;
}

// Shared driver: validates, stages host outputs through device memory, launches, copies back.
// Collocation host outputs: large ones (>= 16 MB) are staged and copied in row chunks on a copy
// stream while later rows compute (the copy engine moves ~190 GB/s over the CPU-GPU link, about
// twice what kernel stores into host memory reach); small page-locked ones are written in place by
// the kernels through their device-mapped address (no copy launch at all).
}  // extern "C"

namespace sod {
int assemble_kinds(sod_context *ctx, const sod_mesh *mesh, int mask, int method, double c1, double c2, double rho,
                   const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, int parts,
                   void *const outs[4], int out_dtype, bool compensated) {
    SOD_TRY(check_context(ctx));
    SOD_REQUIRE(mesh && mesh->ctx == ctx, "mesh does not belong to this context");
    SOD_REQUIRE(out_dtype == SOD_C128 || out_dtype == SOD_C64, "output dtype must be complex128 or complex64");
    SOD_REQUIRE(parts >= 1 && parts <= 3, "parts must be regular (1), singular (2) or both (3)");
    SOD_REQUIRE(s != nullptr, "null frequency array");
    SOD_REQUIRE(nfreq >= 1 && nfreq <= 65535, "nfreq must be in [1, 65535]");
    SOD_REQUIRE(c1 > 0 && c2 > 0 && rho > 0 && std::isfinite(c1) && std::isfinite(c2) && std::isfinite(rho),
                "wave speeds and density must be positive and finite");
    for (int l = 0; l < nfreq; l++)
        SOD_REQUIRE(std::isfinite(s[2 * l]) && std::isfinite(s[2 * l + 1]) && (s[2 * l] != 0.0 || s[2 * l + 1] != 0.0),
                    "Laplace frequencies must be finite and non-zero");
    for (int kd = 0; kd < 4; kd++)
        if (mask & (1 << kd)) SOD_REQUIRE(outs[kd] != nullptr, "null output buffer");
    SOD_REQUIRE(method == SOD_COLLOCATION || method == SOD_GALERKIN, "method must be collocation or Galerkin");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t esz = out_dtype == SOD_C128 ? 16 : 8;
    CollLaunch L{};
    L.mesh = mesh;
    L.kind_mask = mask;
    L.nfreq = nfreq;
    // host outputs are staged in one device buffer, kinds back to back
    bool host_out[4] = {false, false, false, false};
    void *direct[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t staged = 0, off[4] = {0, 0, 0, 0};
    bool any_host = false;
    size_t host_bytes = 0;
    for (int kd = 0; kd < 4; kd++)
        if ((mask & (1 << kd)) && !is_device_ptr(outs[kd])) host_bytes += kind_elems(kd, mesh->nV) * nfreq * esz;
    const bool pipelined = method == SOD_COLLOCATION && host_bytes >= ((size_t)16 << 20);
    for (int kd = 0; kd < 4; kd++) {
        if (!(mask & (1 << kd))) continue;
        if (is_device_ptr(outs[kd])) continue;
        any_host = true;
        if (method == SOD_COLLOCATION && !pipelined) direct[kd] = mapped_host_ptr(outs[kd]);
        if (direct[kd]) continue;
        host_out[kd] = true;
        off[kd] = staged;
        staged += kind_elems(kd, mesh->nV) * nfreq * esz;
    }
    if (staged) SOD_TRY(ctx->staging.ensure(staged));
    for (int kd = 0; kd < 4; kd++) {
        L.freq_stride[kd] = (long long)kind_elems(kd, mesh->nV);
        if (!(mask & (1 << kd))) continue;
        L.out[kd] = direct[kd] ? direct[kd] : host_out[kd] ? ctx->staging.as<char>() + off[kd] : outs[kd];
    }
    std::vector<KConst<double>> kd(nfreq);
    for (int l = 0; l < nfreq; l++) kd[l] = make_kconst(c1, c2, rho, s[2 * l], s[2 * l + 1]);
    L.kc_host = kd.data();
    L.order = order;
    L.subdiv = subdiv;
    L.sorder = sorder;
    L.ssub = ssub;
    L.parts = parts;
    L.out_dtype = out_dtype;
    L.stream = ctx->stream;
    L.compensated = compensated && method == SOD_COLLOCATION;
    if (pipelined)
        for (int kd = 0; kd < 4; kd++) L.host[kd] = host_out[kd] ? outs[kd] : nullptr;
    SOD_TRY(method == SOD_GALERKIN ? launch_galerkin(ctx, L) : launch_collocation(ctx, L));
    if (any_host) {
        for (int kd2 = 0; kd2 < 4; kd2++)
            if (host_out[kd2] && !pipelined)
                SOD_CHECK_CUDA(cudaMemcpyAsync(outs[kd2], L.out[kd2], kind_elems(kd2, mesh->nV) * nfreq * esz,
                                               cudaMemcpyDeviceToHost, ctx->stream));
        SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
        SOD_TRY(take_device_error(ctx));
    }
    return SOD_OK;
}
}  // namespace sod

extern "C" {

int sod_cqbem_assemble_frequencies(sod_context *ctx, const sod_mesh *mesh, int kind, int method, double c1, double c2,
                                   double rho, const double *s, int nfreq, int order, int subdiv, int sorder, int ssub,
                                   int parts, void *out, int out_dtype) {
    SOD_REQUIRE(kind >= SOD_G && kind <= SOD_B_ANGULAR, "kind must be G, H, B_trans or B_angular");
    void *outs[4] = {nullptr, nullptr, nullptr, nullptr};
    outs[kind] = out;
    return assemble_kinds(ctx, mesh, 1 << kind, method, c1, c2, rho, s, nfreq, order, subdiv, sorder, ssub, parts,
                          outs, out_dtype, ctx && ctx->precision == SOD_PRECISION_COMPENSATED);
}

int sod_cqbem_assemble_all(sod_context *ctx, const sod_mesh *mesh, int method, double c1, double c2, double rho,
                           const double *s, int nfreq, int order, int subdiv, int sorder, int ssub, int parts,
                           void *out_G, void *out_H, void *out_B_trans, void *out_B_angular, int out_dtype) {
    void *outs[4] = {out_G, out_H, out_B_trans, out_B_angular};
    int mask = 0;
    for (int kd = 0; kd < 4; kd++)
        if (outs[kd]) mask |= 1 << kd;
    SOD_REQUIRE(mask != 0, "no output requested");
    return assemble_kinds(ctx, mesh, mask, method, c1, c2, rho, s, nfreq, order, subdiv, sorder, ssub, parts, outs,
                          out_dtype, ctx && ctx->precision == SOD_PRECISION_COMPENSATED);
}

int sod_cqbem_assemble(sod_context *ctx, const sod_mesh *mesh, int kind, int method, double c1, double c2, double rho,
                       double s_re, double s_im, int order, int subdiv, int sorder, int ssub, int parts, void *out,
                       int out_dtype) {
    const double s[2] = {s_re, s_im};
    return sod_cqbem_assemble_frequencies(ctx, mesh, kind, method, c1, c2, rho, s, 1, order, subdiv, sorder, ssub,
                                          parts, out, out_dtype);
}

int sod_cq_inverse_transform(sod_context *ctx, const void *Xhat, int in_dtype, int64_t M, int nfreq, int L, double R,
                             void *out, int out_dtype) {
    SOD_TRY(check_context(ctx));
    SOD_REQUIRE(Xhat && out, "null buffer");
    SOD_CHECK_CUDA(cudaSetDevice(ctx->device));
    const size_t isz = in_dtype == SOD_C128 ? 16 : 8, osz = out_dtype == SOD_F64 ? 8 : 4;
    const bool din = is_device_ptr(Xhat), dout = is_device_ptr(out);
    const void *x = Xhat;
    void *o = out;
    if (!din) {
        SOD_TRY(ctx->staging2.ensure(isz * (size_t)M * nfreq));
        SOD_CHECK_CUDA(cudaMemcpyAsync(ctx->staging2.p, Xhat, isz * (size_t)M * nfreq, cudaMemcpyHostToDevice, ctx->stream));
        x = ctx->staging2.p;
    }
    if (!dout) {
        SOD_TRY(ctx->staging.ensure(osz * (size_t)M * L));
        o = ctx->staging.p;
    }
    SOD_TRY(launch_inverse_transform(ctx, x, in_dtype, M, nfreq, L, R, o, out_dtype, ctx->stream));
    if (!dout) {
        SOD_CHECK_CUDA(cudaMemcpyAsync(out, o, osz * (size_t)M * L, cudaMemcpyDeviceToHost, ctx->stream));
        SOD_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return SOD_OK;
}

}  // extern "C"
