// Host side of the C ABI (include/sj.h): descriptor validation, the
// structure builder (class maps -> material combos, meep-form ADE
// coefficients, CPML profiles), source tables, probe stencils, device
// allocation, stepping and read-back.
//
// Reference counterparts: structure_from_settings (src/disp.cpp:482-550),
// the bound_geom constructor's source/monitor scan (src/disp.cpp:557-645),
// bound_geom::run (src/disp.cpp:690-749).
#include "sj_internal.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

using namespace sj;

namespace {

thread_local std::string g_create_error;

struct Fail {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& m) { throw Fail{code, m}; }

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) fail(SJ_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// ------------------------------------------------------------------ sources
// gaussian_src_time_phase (src/disp.cpp:378-400): omega = 2 pi f,
// phi = phase + pi, peak = (st + et)/2, cutoff = (et - st)/2 shrunk while the
// envelope there is below 1e-100 and rounded to float, amp = 1/(-i omega).
struct GaussParams {
    double omega, width, phi, peak, cutoff;
    std::complex<double> amp;
};

GaussParams gauss_params(const sj_source_desc& s) {
    GaussParams g;
    g.omega = 2 * M_PI * s.frequency;
    g.width = s.width;
    g.phi = s.phase + M_PI;
    g.peak = 0.5 * (s.start_time + s.end_time);
    g.cutoff = (s.end_time - s.start_time) * 0.5;
    g.amp = 1.0 / std::complex<double>(0, -g.omega);
    while (exp(-g.cutoff * g.cutoff / (2 * g.width * g.width)) < 1e-100) g.cutoff *= 0.9;
    g.cutoff = float(g.cutoff);
    return g;
}

std::complex<double> dipole(const sj_source_desc& s, double t) {
    if (s.kind == SJ_SRC_GAUSSIAN) {
        const GaussParams g = gauss_params(s);
        const double tt = t - g.peak;
        if (float(fabs(tt)) > g.cutoff) return 0.0;
        return exp(-tt * tt / (2 * g.width * g.width)) * std::polar(1.0, -g.omega * tt - g.phi) * g.amp;
    }
    // continuous source: e^{-i w t}/(-i w) with tanh turn-on/turn-off ramps of
    // width `width` and slowness 3 (meep's continuous_src_time)
    const float rt = float(t);
    if (rt < s.start_time || rt > s.end_time) return 0.0;
    const std::complex<double> iw(0, -2 * M_PI * s.frequency);
    if (s.width == 0.0) return std::exp(iw * t) / iw;
    const double slowness = 3.0;
    const double ts = (t - s.start_time) / s.width - slowness;
    const double te = (s.end_time - t) / s.width - slowness;
    return std::exp(iw * t) / iw * (1.0 + tanh(ts)) * (1.0 + tanh(te)) * 0.25;
}

std::complex<double> current(const sj_source_desc& s, double t, double dt) {
    return (dipole(s, t) - dipole(s, t - dt)) / dt;
}

double last_time(const sj_source_desc& s) {
    if (s.kind == SJ_SRC_GAUSSIAN) {
        const GaussParams g = gauss_params(s);
        return float(g.peak + g.cutoff);
    }
    return float(s.end_time);
}

// ------------------------------------------------------------------ helpers
const double kOff[6][3] = {{0.5, 0, 0}, {0, 0.5, 0}, {0, 0, 0.5},
                           {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0.5, 0}};

// one instance as the host sees it
template <typename real>
struct HostInst {
    sj_grid_desc grid{};
    int nx = 0, ny = 0, nz = 0, px = 0;
    double dx = 0, dt = 0;
    int save_span = 1;
    std::vector<sj_source_desc> srcs;
    std::vector<double*> d_tab;      // per source
    long long tab_cap = 0;
    std::vector<int> probe_flags;
    std::vector<int> dft_comp;       // component of each DFT row
    int n_mon = 0, n_dft = 0, n_freq = 0;
    double* d_mon = nullptr;
    long long mon_cap = 0;
    std::vector<uint32_t> keys;      // combo -> (cx | cy<<8 | cz<<16)
    std::vector<real> coef;          // combo coefficient table (host copy of I.coef)
    std::vector<real> prof[3];       // CPML profiles (host copies of I.prof)
    std::vector<double> des_eps;     // design region eps per voxel (empty: none)
    real* d_dinv = nullptr;          // its inverse on the device
    long long voxels = 0;
    double bytes_per_step = 0;
    double last_source_time = 0;
};

// dump_raw snapshots of one instance: a ring of `depth` slots, each a dense
// device staging copy and a pinned host copy of one component
struct Snapshots {
    int comp = -1, every = 0, depth = 0;
    std::vector<void*> dev, host;
    std::vector<cudaEvent_t> staged, done;  // staging copy made / host copy landed
    std::vector<long long> step;
    int head = 0, count = 0;                // oldest slot, slots holding a snapshot
};

}  // namespace

struct sj_sim {
    int precision = SJ_F64;
    int schedule = SJ_SCHED_SPLIT;
    int n_inst = 0;
    std::vector<HostInst<double>> hi64;
    std::vector<HostInst<float>> hi32;
    std::vector<InstDev<double>> h64;
    std::vector<InstDev<float>> h32;
    void* d_table = nullptr;           // InstDev[n] + split prefix[n+1]
    DevState* d_state = nullptr;
    double* d_scratch = nullptr;       // small reductions
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long t = 0;                   // host mirror of the step counter
    long long h2d = 0, d2h = 0;        // bytes copied across PCIe/C2C
    int cur = 0;                       // host mirror of the ping-pong buffer
    std::vector<void*> allocs;
    std::string err;
    // graph cache, by the parity the captured chunk starts at
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_chunk = 0;
    int graph_sched = -1;
    // TMA schedule: tiling, tensor maps, block prefixes
    int f_ty = 8, f_zs = 64, f_ring = 3;
    bool fused_ready = false;
    unsigned long long tma_wait_ns = 0;  // limit of a wait on a TMA copy (0 = the kernel's 100 ms)
    int test_stall = 0;                  // sj_set_test_stall
    FusedLaunch fl{};
    void* d_fpre = nullptr;
    void* d_tmaps = nullptr;
    // fused (lean) schedule: z-segment length (descriptors travel as kernel
    // parameters) and the side streams its kernels overlap on
    int l_zb = 16;
    int l_one_column = 0;              // 1: one column per thread in every tile kernel
    int lean_zb = -1;                  // z-segment length the tile lists were built for
    void* d_tiles = nullptr;           // tile lists of all instances and classes
    std::vector<LeanTiles> ltiles;     // per instance
    std::vector<LeanGroup> lgroups;    // instances sharing tile launches (every instance in one)
    std::vector<std::vector<int>> lmembers;  // per group: its instances, member order
    void* d_fix = nullptr;             // correction block tables (E sources, polarisations)
    LeanFix lfix{};
    void* d_gen = nullptr;             // general-launch block table
    LeanGen lgen{};
    void* d_parity = nullptr;          // every instance descriptor twice, by parity (LeanGen)
    cudaStream_t side[LEAN_STREAMS] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[LEAN_STREAMS] = {};
    std::vector<unsigned> h_tiles;     // host copy of the tile lists (prepare_lean)
    std::vector<long long> h_tile_off; // [instance][class] offset into h_tiles
    // queued launch of the fused schedule (SJ_LAUNCH_QUEUE)
    int l_launch = SJ_LAUNCH_GROUPED;
    LeanQueue<float> queue{};
    std::vector<LeanTable<float>> q_tabs;  // [dry][parity][group] descriptors (host; kernel parameters)
    void* d_qitems = nullptr;
    long long q_version = -1;          // table_version the queue tables were built from
    long long lists_version = 0;       // bumped whenever prepare_lean rebuilds the tile lists
    long long q_lists = -1;            // lists_version the queue items were built from
    // dump_raw snapshots (per instance) and the stream their host copies run on
    std::vector<Snapshots> snaps;
    cudaStream_t copy_stream = nullptr;
    // bumped whenever a descriptor changes; a graph holding parameter copies
    // of older descriptors is captured again
    long long table_version = 0;
    long long graph_version = -1;
    // divergence guard: bound, the device word electing the recorder and the
    // host-mapped record (host and device addresses)
    double guard_bound = 1000.0;
    int* d_guard_flag = nullptr;
    GuardRecord* h_guard = nullptr;
    GuardRecord* d_guard = nullptr;

    ~sj_sim() {
        if (stream) cudaStreamSynchronize(stream);
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (Snapshots& S : snaps) release(S);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        for (int q = 0; q < LEAN_STREAMS; ++q) {
            if (side[q]) cudaStreamSynchronize(side[q]), cudaStreamDestroy(side[q]);
            if (ev_join[q]) cudaEventDestroy(ev_join[q]);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        drop_graphs();
        for (void* p : allocs) cudaFree(p);
        if (h_guard) cudaFreeHost(h_guard);
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
    // frees a snapshot ring (its copies must have finished)
    void release(Snapshots& S) {
        for (void* h : S.host) cudaFreeHost(h);
        for (void* d : S.dev) dfree(d);
        for (cudaEvent_t e : S.staged) cudaEventDestroy(e);
        for (cudaEvent_t e : S.done) cudaEventDestroy(e);
        S = Snapshots{};
    }
    bool any_snapshots() const {
        for (const Snapshots& S : snaps)
            if (S.every > 0) return true;
        return false;
    }
    void drop_graphs() {
        for (int p = 0; p < 2; ++p)
            if (graph[p]) cudaGraphExecDestroy(graph[p]), graph[p] = nullptr;
    }
    void* dalloc(size_t bytes, bool zero = true) {
        void* p = nullptr;
        if (bytes == 0) return nullptr;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) fail(SJ_E_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
        allocs.push_back(p);
        if (zero) ck(cudaMemsetAsync(p, 0, bytes, stream), "cudaMemsetAsync");
        return p;
    }
    void dfree(void* p) {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p);
    }
    template <typename T>
    T* upload(const std::vector<T>& v) {
        if (v.empty()) return nullptr;
        T* p = (T*)dalloc(v.size() * sizeof(T), false);
        ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
        h2d += (long long)(v.size() * sizeof(T));
        return p;
    }
};

namespace {

// ------------------------------------------------------------------ validation
void check_scene(const sj_scene_desc* sc) {
    if (!sc) fail(SJ_E_INVALID, "material has neither class_map nor scene");
    if (sc->n_regions < 0 || sc->n_regions > SJ_MAX_REGIONS)
        fail(SJ_E_INVALID, "scene n_regions must be in [0, 8]");
    int total = 0;
    for (int r = 0; r < sc->n_regions; ++r) {
        const sj_region_desc& g = sc->regions[r];
        if (g.n_nodes < 1 || !g.nodes) fail(SJ_E_INVALID, "region without CSG nodes");
        int depth = 0;
        for (int q = 0; q < g.n_nodes; ++q) {
            const int op = g.nodes[q].op;
            if (op < 0) fail(SJ_E_INVALID, "negative CSG op");
            if (op <= SJ_CSG_PLANE || op == SJ_CSG_CONST || op == SJ_CSG_NOOP)
                ++depth;
            else if (op == SJ_CSG_UNION || op == SJ_CSG_INTERSECT) {
                if (depth < 2) fail(SJ_E_INVALID, "CSG program underflows its stack");
                --depth;
            } else if (op == SJ_CSG_PASS) {
                if (depth < 1) fail(SJ_E_INVALID, "CSG program underflows its stack");
            } else
                fail(SJ_E_INVALID, "unknown CSG op " + std::to_string(op));
            if (depth > 64) fail(SJ_E_INVALID, "CSG program deeper than 64");
        }
        if (depth != 1) fail(SJ_E_INVALID, "CSG program must leave exactly one value");
        if (g.n_poles < 0 || (g.n_poles > 0 && (!g.poles || !g.sigma)))
            fail(SJ_E_INVALID, "region poles/sigma missing");
        total += g.n_nodes;
    }
    if (total > SJ_MAX_CSG_NODES * SJ_MAX_REGIONS) fail(SJ_E_INVALID, "too many CSG nodes");
    if (sc->smooth_n < 0 || sc->smooth_n > SJ_MAX_SMOOTH_N) fail(SJ_E_INVALID, "scene smooth_n must be in [0, 31]");
    if (sc->smooth_n > 0) {
        if (!(sc->smooth_rad > 0) || !std::isfinite(sc->smooth_rad))
            fail(SJ_E_INVALID, "scene smooth_rad must be finite and > 0");
        if (sc->combine != SJ_EPS_SUM) fail(SJ_E_INVALID, "smoothing needs the SJ_EPS_SUM combine mode");
    }
}

void upload_scene(sj_sim* sim, const sj_scene_desc* sc, sj_csg_node** d_nodes, int** d_start) {
    std::vector<sj_csg_node> nodes;
    std::vector<int> start(1, 0);
    for (int r = 0; r < sc->n_regions; ++r) {
        const sj_region_desc& g = sc->regions[r];
        nodes.insert(nodes.end(), g.nodes, g.nodes + g.n_nodes);
        start.push_back((int)nodes.size());
    }
    if (nodes.empty()) nodes.push_back(sj_csg_node{});
    *d_nodes = sim->upload(nodes);
    *d_start = sim->upload(start);
}

// class table of a scene: class = bitmask of regions (src/disp.cpp:264-283)
void scene_classes(const sj_scene_desc* sc, std::vector<double>& eps, std::vector<sj_pole>& poles,
                   std::vector<double>& sigma, int& n_classes) {
    const int R = sc->n_regions;
    n_classes = 1 << R;
    poles.clear();
    std::vector<std::pair<int, double>> owner;  // (region, sigma)
    for (int r = 0; r < R; ++r)
        for (int q = 0; q < sc->regions[r].n_poles; ++q) {
            poles.push_back(sc->regions[r].poles[q]);
            owner.push_back({r, sc->regions[r].sigma[q]});
        }
    if ((int)poles.size() > SJ_MAX_POLES) fail(SJ_E_INVALID, "more than 8 susceptibilities in scene");
    if (sc->combine != SJ_EPS_SUM && sc->combine != SJ_EPS_FIRST) fail(SJ_E_INVALID, "bad scene combine mode");
    eps.assign(n_classes, 0.0);
    sigma.assign((size_t)n_classes * poles.size(), 0.0);
    const double def = sc->ambient_eps;
    for (int m = 0; m < n_classes; ++m) {
        int first = -1;  // first region containing the point (SJ_EPS_FIRST)
        for (int r = 0; r < R && first < 0; ++r)
            if ((m >> r) & 1) first = r;
        if (sc->combine == SJ_EPS_FIRST) {
            eps[m] = first >= 0 ? sc->regions[first].eps : def;
        } else if (R == 0) {
            eps[m] = def;
        } else {
            double ret = 0;
            for (int r = 0; r < R; ++r) {
                const double in = (m >> r) & 1;
                ret += def + (sc->regions[r].eps - def) * in / 1.0;
            }
            eps[m] = ret;
        }
        for (size_t p = 0; p < poles.size(); ++p) {
            double in = (m >> owner[p].first) & 1;
            if (sc->combine == SJ_EPS_FIRST && owner[p].first != first) in = 0;
            sigma[(size_t)m * poles.size() + p] = 0.0 + (owner[p].second - 0.0) * in / 1.0;
        }
    }
}

// Smoothing offsets: cgs_material_function::generate_smooth_pts
// (src/disp.cpp:56-112) as the constructors call it, with seed DEF_SEED
// (src/disp.hpp:34, the double 0xd9a28bf3).  Its seed_seq takes the seed's
// low 16 bits and (bits 16-31) >> 32, i.e. {0x8bf3, 0}.  Per draw: u, then
// phi = 2 pi u', then the radius r from N(0, smooth_rad); the point is
// (r sin(theta) cos(phi), the same for y, r cos(theta)) with cos(theta) =
// 1 - 2u, sin(theta) = 2 sqrt(u (1 - u)), and its 8 sign reflections follow
// with the x sign outermost.  libstdc++'s generators and distributions give
// the reference's sequence.
std::vector<double> smooth_points(int n, double rad) {
    std::seed_seq seeder{0x8bf3u, 0u};
    std::mt19937 gen(seeder);
    std::normal_distribution<double> radial(0.0, rad);
    std::uniform_real_distribution<double> unit(0.0, 1.0);
    std::vector<double> out;
    out.reserve((size_t)24 * n);
    for (int d = 0; d < n; ++d) {
        const double u = unit(gen);
        const double ct = 1 - 2 * u;
        const double st = 2 * std::sqrt(u * (1 - u));
        const double phi = 2 * M_PI * unit(gen);
        const double r = radial(gen);
        const double x = r * st * std::cos(phi), y = r * st * std::cos(phi), z = r * ct;
        for (int sx = -1; sx < 2; sx += 2)
            for (int sy = -1; sy < 2; sy += 2)
                for (int sz = -1; sz < 2; sz += 2) {
                    out.push_back(x * sx);
                    out.push_back(y * sy);
                    out.push_back(z * sz);
                }
    }
    return out;
}

// class table of a smoothed scene: class q = sorted key q, key = the point's
// counts 8 bits per region; in_bound's sum with this_ret = count over
// smooth_n + 1 = 8 n + 1 samples (src/disp.cpp:272-280), the susceptibility
// scale functions the same with def_ret 0 (src/disp.cpp:545)
void smooth_scene_classes(const sj_scene_desc* sc, const std::vector<unsigned long long>& keys,
                          std::vector<double>& eps, std::vector<sj_pole>& poles, std::vector<double>& sigma,
                          int& n_classes) {
    const int R = sc->n_regions;
    const double samples = (double)(8 * sc->smooth_n + 1);
    n_classes = (int)keys.size();
    poles.clear();
    std::vector<std::pair<int, double>> owner;
    for (int r = 0; r < R; ++r)
        for (int q = 0; q < sc->regions[r].n_poles; ++q) {
            poles.push_back(sc->regions[r].poles[q]);
            owner.push_back({r, sc->regions[r].sigma[q]});
        }
    if ((int)poles.size() > SJ_MAX_POLES) fail(SJ_E_INVALID, "more than 8 susceptibilities in scene");
    eps.assign(n_classes, 0.0);
    sigma.assign((size_t)n_classes * poles.size(), 0.0);
    const double def = sc->ambient_eps;
    for (int m = 0; m < n_classes; ++m) {
        if (R == 0) {
            eps[m] = def;
        } else {
            double ret = 0;
            for (int r = 0; r < R; ++r) {
                const double cnt = (double)((keys[m] >> (8 * r)) & 255);
                ret += def + (sc->regions[r].eps - def) * cnt / samples;
            }
            eps[m] = ret;
        }
        for (size_t p = 0; p < poles.size(); ++p) {
            const double cnt = (double)((keys[m] >> (8 * owner[p].first)) & 255);
            sigma[(size_t)m * poles.size() + p] = 0.0 + (owner[p].second - 0.0) * cnt / samples;
        }
    }
}

// Rasterise a smoothed scene into d_cls (pitched [3][cpitch]); returns the
// sorted distinct keys (the classes).
std::vector<unsigned long long> smooth_rasterize(sj_sim* sim, const sj_scene_desc* sc, const sj_grid_desc& g,
                                                 int px, const sj_csg_node* d_nodes, const int* d_start,
                                                 uint8_t* d_cls, long long cpitch, cudaStream_t st) {
    const std::vector<double> offs = smooth_points(sc->smooth_n, sc->smooth_rad);
    double* d_offs = sim->upload(offs);
    unsigned long long* d_keys = (unsigned long long*)sim->dalloc(3 * cpitch * sizeof(unsigned long long), false);
    unsigned long long* d_set = (unsigned long long*)sim->dalloc(SMOOTH_SET_CAP * sizeof(unsigned long long), false);
    int* d_over = (int*)sim->dalloc(sizeof(int));
    ck(cudaMemsetAsync(d_set, 0xff, SMOOTH_SET_CAP * sizeof(unsigned long long), st), "set clear");
    ck(launch_rasterize_counts(d_nodes, d_start, sc->n_regions, g.nx, g.ny, g.nz, g.dx, g.origin, d_offs,
                               (int)(offs.size() / 3), d_keys, cpitch, px, d_set, SMOOTH_SET_CAP, d_over, st),
       "rasterize counts");
    std::vector<unsigned long long> set(SMOOTH_SET_CAP);
    int over = 0;
    ck(cudaMemcpyAsync(set.data(), d_set, set.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st),
       "set read");
    ck(cudaMemcpyAsync(&over, d_over, sizeof(int), cudaMemcpyDeviceToHost, st), "overflow read");
    ck(cudaStreamSynchronize(st), "smoothing sync");
    sim->d2h += (long long)(set.size() * sizeof(unsigned long long) + sizeof(int));
    std::vector<unsigned long long> keys;
    for (unsigned long long k : set)
        if (k != ~0ull) keys.push_back(k);
    std::sort(keys.begin(), keys.end());
    if (over || keys.size() > 256)
        fail(SJ_E_INVALID, "smoothing gives more than 256 distinct point classes (lower smooth_n or smooth_rad)");
    unsigned long long* d_sorted = sim->upload(keys);
    ck(launch_class_assign(d_keys, cpitch, g.nx, g.ny, g.nz, px, d_sorted, (int)keys.size(), d_cls, st),
       "class assign");
    ck(cudaStreamSynchronize(st), "smoothing sync");
    sim->dfree(d_sorted);
    sim->dfree(d_over);
    sim->dfree(d_set);
    sim->dfree(d_keys);
    sim->dfree(d_offs);
    return keys;
}

// ------------------------------------------------------------------ builder
template <typename real>
void build_instance(sj_sim* sim, const sj_instance_desc& d, HostInst<real>& H, InstDev<real>& I) {
    cudaStream_t st = sim->stream;
    memset(&I, 0, sizeof(I));
    const sj_grid_desc& g = d.grid;
    if (g.nx < 1 || g.ny < 1 || g.nz < 1) fail(SJ_E_INVALID, "grid dimensions must be >= 1");
    if (!(g.dx > 0)) fail(SJ_E_INVALID, "grid dx must be > 0");
    if ((long long)g.nx * g.ny * g.nz > (1ll << 40)) fail(SJ_E_INVALID, "grid too large");
    H.grid = g;
    H.nx = g.nx, H.ny = g.ny, H.nz = g.nz;
    H.px = (g.nx + PITCH_ALIGN - 1) / PITCH_ALIGN * PITCH_ALIGN;
    H.dx = g.dx;
    H.dt = g.dt > 0 ? g.dt : 0.5 * g.dx;
    H.save_span = d.save_span > 0 ? d.save_span : 1;
    const int nx = H.nx, ny = H.ny, nz = H.nz, px = H.px;
    const long long plane = (long long)px * ny, vol = plane * nz;
    I.nx = nx, I.ny = ny, I.nz = nz, I.px = px;
    I.plane = plane, I.vol = vol;
    I.S = (real)(H.dt / H.dx);
    I.dt = H.dt;
    I.save_span = H.save_span;
    H.voxels = (long long)nx * ny * nz;

    // ---- fields, both ping-pong buffers
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 6; ++c) I.F[b][c] = (real*)sim->dalloc(vol * sizeof(real));

    // ---- material classes per E-component point (pitched [3][nz][ny][px])
    const sj_material_desc& m = d.material;
    std::vector<double> eps;
    std::vector<sj_pole> poles;
    std::vector<double> sigma;
    int n_classes = 0;
    const long long cpitch = vol;
    uint8_t* d_cls = (uint8_t*)sim->dalloc(3 * cpitch, false);
    if (m.class_map) {
        if (m.n_classes < 1 || m.n_classes > 255) fail(SJ_E_INVALID, "n_classes must be in [1, 255]");
        if (!m.eps_inf) fail(SJ_E_INVALID, "eps_inf missing");
        if (m.n_poles < 0 || m.n_poles > SJ_MAX_POLES) fail(SJ_E_INVALID, "n_poles must be in [0, 8]");
        if (m.n_poles > 0 && (!m.poles || !m.sigma)) fail(SJ_E_INVALID, "poles/sigma missing");
        n_classes = m.n_classes;
        eps.assign(m.eps_inf, m.eps_inf + n_classes);
        poles.assign(m.poles, m.poles + m.n_poles);
        sigma.assign(m.sigma, m.sigma + (size_t)n_classes * m.n_poles);
        for (int c = 0; c < 3; ++c)
            ck(cudaMemcpy2D(d_cls + c * cpitch, px, m.class_map + (size_t)c * nx * ny * nz, nx, nx,
                            (size_t)ny * nz, cudaMemcpyHostToDevice),
               "class map upload");
        sim->h2d += 3ll * nx * ny * nz;
    } else {
        check_scene(m.scene);
        sj_csg_node* d_nodes;
        int* d_start;
        upload_scene(sim, m.scene, &d_nodes, &d_start);
        if (m.scene->smooth_n > 0) {
            const std::vector<unsigned long long> keys =
                smooth_rasterize(sim, m.scene, g, px, d_nodes, d_start, d_cls, cpitch, st);
            smooth_scene_classes(m.scene, keys, eps, poles, sigma, n_classes);
        } else {
            scene_classes(m.scene, eps, poles, sigma, n_classes);
            ck(launch_rasterize(d_nodes, d_start, m.scene->n_regions, nx, ny, nz, H.dx, g.origin, d_cls,
                                cpitch, px, st),
               "rasterize");
        }
    }
    for (int c = 0; c < n_classes; ++c)
        if (!(eps[c] != 0.0) || !std::isfinite(eps[c])) fail(SJ_E_INVALID, "eps_inf must be finite and nonzero");

    // ---- combos: distinct (class_x, class_y, class_z) triples
    {
        // one bit per (cx, cy, cz) triple present, compacted on the device to
        // at most 257 keys (count first), so only those cross to the host
        constexpr int KCAP = 257;
        const int n_words = (1 << 24) / 32;
        uint32_t* d_bitmap = (uint32_t*)sim->dalloc((size_t)n_words * 4 + (KCAP + 1) * 4);
        uint32_t* d_found = d_bitmap + n_words;  // [0] = count, then the keys
        ck(launch_combo_mark(d_cls, cpitch, nx, ny, nz, px, d_bitmap, st), "combo mark");
        ck(launch_combo_compact(d_bitmap, n_words, d_found + 1, KCAP, reinterpret_cast<int*>(d_found), st),
           "combo compact");
        std::vector<uint32_t> found(KCAP + 1);
        ck(cudaMemcpyAsync(found.data(), d_found, found.size() * 4, cudaMemcpyDeviceToHost, st), "combo keys");
        sim->d2h += (long long)found.size() * 4;
        ck(cudaStreamSynchronize(st), "combo sync");
        sim->dfree(d_bitmap);
        const int n_found = (int)found[0];
        if (n_found > 256) fail(SJ_E_INVALID, "more than 256 distinct material combos");
        H.keys.assign(found.begin() + 1, found.begin() + 1 + n_found);
        std::sort(H.keys.begin(), H.keys.end());
        for (uint32_t k : H.keys)
            for (int c = 0; c < 3; ++c)
                if ((int)((k >> (8 * c)) & 255) >= n_classes)
                    fail(SJ_E_INVALID, "class map holds a class index >= n_classes");
        uint32_t* d_keys = sim->upload(H.keys);
        uint8_t* d_combo = (uint8_t*)sim->dalloc(vol);
        ck(launch_combo_assign(d_cls, cpitch, nx, ny, nz, px, d_keys, (int)H.keys.size(), d_combo, st),
           "combo assign");
        ck(cudaStreamSynchronize(st), "combo sync");
        sim->dfree(d_keys);
        sim->dfree(d_cls);
        I.combo = d_combo;
    }

    // ---- meep-form ADE coefficients (lorentzian_susceptibility::update_P)
    const int np = (int)poles.size();
    I.n_poles = np;
    std::vector<double> Cp(np);
    for (int p = 0; p < np; ++p) {
        const double w = 2 * M_PI * poles[p].omega_0, gm = 2 * M_PI * poles[p].gamma;
        const double dt = H.dt;
        const double den = 1 + gm * dt / 2;
        const double L = poles[p].drude ? 0.0 : 1.0;
        I.A[p] = (real)((2 - w * w * dt * dt * L) / den);
        I.B[p] = (real)(-(1 - gm * dt / 2) / den);
        Cp[p] = w * w * dt * dt / den;
    }
    const int nk = (int)H.keys.size();
    I.n_combos = nk;
    I.ncoef = 6 + 3 * np;
    std::vector<real> coef((size_t)nk * I.ncoef);
    std::vector<uint8_t> cflag(nk, 0);
    std::vector<uint32_t> pmask(nk, 0);
    for (int q = 0; q < nk; ++q) {
        for (int c = 0; c < 3; ++c) {
            const int cl = (H.keys[q] >> (8 * c)) & 255;
            coef[(size_t)q * I.ncoef + c] = (real)(1.0 / eps[cl]);
            for (int p = 0; p < np; ++p) {
                const double cs = Cp[p] * sigma[(size_t)cl * np + p];
                coef[(size_t)q * I.ncoef + 3 + 3 * p + c] = (real)cs;
                if (cs != 0.0) cflag[q] |= 1;
                if ((real)cs != real(0)) pmask[q] |= 1u << (8 * c + p);
            }
            // S eps_inf^-1, the product the fused E update scales curl H by
            // (a product of two `real`s: the bits of the device's I.S * inv)
            coef[(size_t)q * I.ncoef + 3 + 3 * np + c] = I.S * coef[(size_t)q * I.ncoef + c];
        }
    }
    I.coef = sim->upload(coef);
    I.cflag = sim->upload(cflag);
    I.pmask = sim->upload(pmask);
    H.coef = coef;

    // ---- dispersive bounding box and polarisation storage
    {
        std::vector<unsigned long long> hist(256);
        unsigned long long* d_hist = (unsigned long long*)sim->dalloc(256 * 8);
        ck(launch_combo_hist(I.combo, nx, ny, nz, px, d_hist, st), "combo hist");
        ck(cudaMemcpyAsync(hist.data(), d_hist, 256 * 8, cudaMemcpyDeviceToHost, st), "hist");
        int box[6] = {INT_MAX, INT_MAX, INT_MAX, -1, -1, -1};
        bool any = false;
        for (int q = 0; q < nk; ++q) any |= (cflag[q] & 1) != 0;
        int* d_box = nullptr;
        if (any) {
            d_box = (int*)sim->dalloc(sizeof(box), false);
            ck(cudaMemcpyAsync(d_box, box, sizeof(box), cudaMemcpyHostToDevice, st), "box");
            ck(launch_disp_bbox(I.combo, I.cflag, nx, ny, nz, px, d_box, st), "bbox");
            ck(cudaMemcpyAsync(box, d_box, sizeof(box), cudaMemcpyDeviceToHost, st), "box");
        }
        ck(cudaStreamSynchronize(st), "bbox sync");
        sim->dfree(d_hist);
        sim->dfree(d_box);
        long long n_disp_pole = 0;  // sum over poles of voxels carrying the pole
        for (int q = 0; q < nk; ++q)
            for (int p = 0; p < np; ++p) {
                bool on = false;
                for (int c = 0; c < 3; ++c) on |= coef[(size_t)q * I.ncoef + 3 + 3 * p + c] != 0;
                if (on) n_disp_pole += (long long)hist[q];
            }
        if (any && box[3] >= 0) {
            for (int a = 0; a < 3; ++a) {
                I.dlo[a] = box[a];
                I.dn[a] = box[3 + a] - box[a] + 1;
            }
            I.dvol = (long long)I.dn[0] * I.dn[1] * I.dn[2];
            I.P = (real*)sim->dalloc((size_t)np * 6 * I.dvol * sizeof(real));
        }
        H.bytes_per_step = (double)H.voxels * (12.0 * sizeof(real) + 1) + (double)n_disp_pole * 12.0 * sizeof(real);
    }

    // ---- CPML profiles and slabs
    const sj_pml_desc& pm = d.pml;
    const double R = pm.r_asymptotic > 0 ? pm.r_asymptotic : 1e-15;
    const double pw = pm.power > 0 ? pm.power : 2.0;
    for (int a = 0; a < 3; ++a) {
        const int n = a == 0 ? nx : (a == 1 ? ny : nz);
        const double o = g.origin[a], L = n * H.dx;
        const double dlo = pm.thickness[a][0], dhi = pm.thickness[a][1];
        if (dlo < 0 || dhi < 0) fail(SJ_E_INVALID, "PML thickness must be >= 0");
        auto sigma_at = [&](double q) {
            double s = 0;
            if (dlo > 0 && q < o + dlo) {
                const double u = (o + dlo - q) / dlo;
                s += -(pw + 1) * log(R) / (2 * dlo) * pow(u, pw);
            }
            if (dhi > 0 && q > o + L - dhi) {
                const double u = (q - (o + L - dhi)) / dhi;
                s += -(pw + 1) * log(R) / (2 * dhi) * pow(u, pw);
            }
            return s;
        };
        std::vector<real> prof(4 * (size_t)n);
        std::vector<char> on(n, 0);
        for (int i = 0; i < n; ++i) {
            for (int h = 0; h < 2; ++h) {
                const double q = o + (i + 0.5 * h) * H.dx;
                const double s = sigma_at(q);
                const double b = exp(-(s + pm.alpha) * H.dt);
                const double c = s > 0 ? s / (s + pm.alpha) * (b - 1) : 0.0;
                prof[(2 * h) * n + i] = (real)b;
                prof[(2 * h + 1) * n + i] = (real)c;
                if (s > 0) on[i] = 1;
            }
        }
        int pl = 0, ph = 0;
        while (pl < n && on[pl]) ++pl;
        while (ph < n - pl && on[n - 1 - ph]) ++ph;
        for (int i = pl; i < n - ph; ++i)
            if (on[i]) fail(SJ_E_INVALID, "PML profile is not confined to the faces");
        I.pl[a] = pl, I.ph[a] = ph;
        I.prof[a] = sim->upload(prof);
        H.prof[a] = prof;
        const long long w = pl + ph;
        if (w > 0) {  // full-grid layout; only the slab voxels are ever touched
            I.psiE[a] = (real*)sim->dalloc(2 * vol * sizeof(real));
            I.psiH[0][a] = (real*)sim->dalloc(2 * vol * sizeof(real));
            I.psiH[1][a] = (real*)sim->dalloc(2 * vol * sizeof(real));
        }
        const long long slab_vox = a == 0 ? (long long)nz * ny * w : (a == 1 ? (long long)nz * w * nx : w * (long long)ny * nx);
        H.bytes_per_step += (double)slab_vox * 4 * 2 * sizeof(real);
    }

    // ---- sources: separable weights on the component's own grid
    if (d.n_sources < 0 || d.n_sources > SJ_MAX_SOURCES) fail(SJ_E_INVALID, "n_sources must be in [0, 4]");
    I.n_src = d.n_sources;
    H.srcs.assign(d.sources, d.sources + d.n_sources);
    H.last_source_time = 0;
    for (int s = 0; s < d.n_sources; ++s) {
        const sj_source_desc& sd = d.sources[s];
        if (sd.component < 0 || sd.component > 5) fail(SJ_E_INVALID, "source component out of range");
        if (sd.kind != SJ_SRC_GAUSSIAN && sd.kind != SJ_SRC_CONTINUOUS) fail(SJ_E_INVALID, "bad source kind");
        if (sd.kind == SJ_SRC_GAUSSIAN && !(sd.width > 0)) fail(SJ_E_INVALID, "Gaussian width must be > 0");
        if (!(sd.frequency > 0)) fail(SJ_E_INVALID, "source frequency must be > 0");
        SrcDev<real>& sv = I.src[s];
        sv.comp = sd.component;
        for (int a = 0; a < 3; ++a) {
            const int n = a == 0 ? nx : (a == 1 ? ny : nz);
            const double lo = std::min(sd.lo[a], sd.hi[a]), hi = std::max(sd.lo[a], sd.hi[a]);
            const double off = kOff[sd.component][a];
            std::vector<double> w(n, 0.0);
            if (hi - lo <= 1e-9 * H.dx) {
                // zero extent: linear interpolation onto the two nearest points, / dx
                const double u = (lo - g.origin[a]) / H.dx - off;
                const double i0 = floor(u);
                const double f = u - i0;
                const long long a0 = (long long)i0;
                if (a0 >= 0 && a0 < n) w[a0] += (1 - f) / H.dx;
                if (a0 + 1 >= 0 && a0 + 1 < n) w[a0 + 1] += f / H.dx;
            } else {
                // finite extent: overlap of each point's dual cell with [lo, hi], / dx
                for (int i = 0; i < n; ++i) {
                    const double q = g.origin[a] + (i + off) * H.dx;
                    const double ov = std::min(hi, q + 0.5 * H.dx) - std::max(lo, q - 0.5 * H.dx);
                    if (ov > 0) w[i] = ov / H.dx;
                }
            }
            int first = -1, last = -1;
            for (int i = 0; i < n; ++i)
                if (w[i] != 0.0) {
                    if (first < 0) first = i;
                    last = i;
                }
            if (first < 0) {  // outside the grid: empty stencil
                first = 0;
                last = -1;
            }
            sv.lo[a] = first;
            sv.n[a] = last - first + 1;
            std::vector<real> wr(std::max(1, sv.n[a]));
            for (int i = 0; i < sv.n[a]; ++i) wr[i] = (real)w[first + i];
            sv.w[a] = sim->upload(wr);
        }
        H.last_source_time = std::max(H.last_source_time, last_time(sd));
    }
    H.d_tab.assign(d.n_sources, nullptr);
    H.tab_cap = 0;

    // ---- probes: trilinear stencils on the component's grid
    if (d.n_probes < 0) fail(SJ_E_INVALID, "n_probes < 0");
    if (d.n_freqs < 0 || d.n_freqs > 256) fail(SJ_E_INVALID, "n_freqs must be in [0, 256]");
    I.n_probe = d.n_probes;
    std::vector<int> pcomp(d.n_probes), pmon(d.n_probes, -1), pdft(d.n_probes, -1);
    std::vector<long long> pidx(8 * (size_t)d.n_probes, -1);
    std::vector<double> pw8(8 * (size_t)d.n_probes, 0.0);
    for (int p = 0; p < d.n_probes; ++p) {
        const sj_probe_desc& pd = d.probes[p];
        if (pd.component < 0 || pd.component > 5) fail(SJ_E_INVALID, "probe component out of range");
        pcomp[p] = pd.component;
        if (pd.flags & SJ_PROBE_MONITOR) pmon[p] = H.n_mon++;
        if (pd.flags & SJ_PROBE_DFT) {
            pdft[p] = H.n_dft++;
            H.dft_comp.push_back(pd.component);
        }
        long long i0[3];
        double f[3];
        for (int a = 0; a < 3; ++a) {
            const double u = (pd.pos[a] - g.origin[a]) / H.dx - kOff[pd.component][a];
            const double fl = floor(u);
            i0[a] = (long long)fl;
            f[a] = u - fl;
        }
        for (int m8 = 0; m8 < 8; ++m8) {
            const int di = m8 & 1, dj = (m8 >> 1) & 1, dk = (m8 >> 2) & 1;
            const long long ii = i0[0] + di, jj = i0[1] + dj, kk = i0[2] + dk;
            const double w = (di ? f[0] : 1 - f[0]) * (dj ? f[1] : 1 - f[1]) * (dk ? f[2] : 1 - f[2]);
            if (ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz) {
                pidx[8 * (size_t)p + m8] = kk * plane + jj * px + ii;
                pw8[8 * (size_t)p + m8] = w;
            }
        }
    }
    I.n_mon = H.n_mon, I.n_dft = H.n_dft, I.n_freq = d.n_freqs;
    H.n_freq = d.n_freqs;
    I.probe_comp = sim->upload(pcomp);
    I.probe_idx = sim->upload(pidx);
    I.probe_w = sim->upload(pw8);
    I.probe_mon = sim->upload(pmon);
    I.probe_dft = sim->upload(pdft);
    if (d.n_freqs > 0) I.freqs = sim->upload(std::vector<double>(d.freqs, d.freqs + d.n_freqs));
    if (H.n_dft > 0 && d.n_freqs > 0)
        I.dft = (double2*)sim->dalloc((size_t)H.n_dft * d.n_freqs * sizeof(double2));
    I.mon = nullptr;
    I.mon_cap = 0;
}

// ------------------------------------------------------------------ stepping support
template <typename real>
std::vector<HostInst<real>>& hostv(sj_sim* s);
template <>
std::vector<HostInst<double>>& hostv<double>(sj_sim* s) { return s->hi64; }
template <>
std::vector<HostInst<float>>& hostv<float>(sj_sim* s) { return s->hi32; }
template <typename real>
std::vector<InstDev<real>>& devv(sj_sim* s);
template <>
std::vector<InstDev<double>>& devv<double>(sj_sim* s) { return s->h64; }
template <>
std::vector<InstDev<float>>& devv<float>(sj_sim* s) { return s->h32; }

long long split_blocks(const InstDev<double>& I) { return split_block_count_f64(I); }
long long split_blocks(const InstDev<float>& I) { return split_block_count_f32(I); }

template <typename real>
void upload_table(sj_sim* sim) {
    auto& dv = devv<real>(sim);
    const int n = sim->n_inst;
    std::vector<char> buf(n * sizeof(InstDev<real>) + (n + 1) * sizeof(long long));
    memcpy(buf.data(), dv.data(), n * sizeof(InstDev<real>));
    long long* pre = reinterpret_cast<long long*>(buf.data() + n * sizeof(InstDev<real>));
    pre[0] = 0;
    for (int q = 0; q < n; ++q) pre[q + 1] = pre[q] + split_blocks(dv[q]);
    if (!sim->d_table) sim->d_table = sim->dalloc(buf.size(), false);
    ck(cudaStreamSynchronize(sim->stream), "sync before table upload");
    ck(cudaMemcpy(sim->d_table, buf.data(), buf.size(), cudaMemcpyHostToDevice), "table upload");
    sim->h2d += (long long)buf.size();
    // by parity: entry cur * n + q has slot 0 = buffer cur (fields, H-side psi)
    std::vector<InstDev<real>> par(2 * (size_t)n);
    for (int q = 0; q < n; ++q) {
        par[q] = dv[q];
        InstDev<real>& t = par[n + q];
        t = dv[q];
        for (int c = 0; c < 6; ++c) std::swap(t.F[0][c], t.F[1][c]);
        for (int a = 0; a < 3; ++a) std::swap(t.psiH[0][a], t.psiH[1][a]);
    }
    if (!sim->d_parity) sim->d_parity = sim->dalloc(par.size() * sizeof(InstDev<real>), false);
    ck(cudaMemcpy(sim->d_parity, par.data(), par.size() * sizeof(InstDev<real>), cudaMemcpyHostToDevice),
       "parity table upload");
    sim->h2d += (long long)(par.size() * sizeof(InstDev<real>));
    sim->table_version += 1;
}

// Make sure source tables and monitor buffers cover steps [0, t_end).
template <typename real>
void ensure_capacity(sj_sim* sim, long long t_end) {
    auto& hv = hostv<real>(sim);
    auto& dv = devv<real>(sim);
    bool changed = false;
    for (int q = 0; q < sim->n_inst; ++q) {
        HostInst<real>& H = hv[q];
        InstDev<real>& I = dv[q];
        if (!H.srcs.empty() && H.tab_cap < t_end) {
            const long long cap = std::max(t_end, 2 * H.tab_cap);
            ck(cudaStreamSynchronize(sim->stream), "sync");
            for (size_t s = 0; s < H.srcs.size(); ++s) {
                std::vector<double> tab(cap);
                const sj_source_desc& sd = H.srcs[s];
                const double half = sd.component < 3 ? 0.5 : 0.0;
                for (long long nn = 0; nn < cap; ++nn) {
                    const double tt = ((double)nn + half) * H.dt;
                    const std::complex<double> a(sd.amplitude[0], sd.amplitude[1]);
                    tab[nn] = H.dt * std::real(a * current(sd, tt, H.dt));
                }
                sim->dfree(H.d_tab[s]);
                H.d_tab[s] = sim->upload(tab);
                I.src[s].tab = H.d_tab[s];
            }
            H.tab_cap = cap;
            changed = true;
        }
        if (H.n_mon > 0) {
            const long long need = (t_end + H.save_span - 1) / H.save_span;
            if (H.mon_cap < need) {
                const long long cap = std::max(need, 2 * H.mon_cap);
                double* nb = (double*)sim->dalloc((size_t)cap * H.n_mon * sizeof(double));
                ck(cudaStreamSynchronize(sim->stream), "sync");
                if (H.d_mon)
                    ck(cudaMemcpy(nb, H.d_mon, (size_t)H.mon_cap * H.n_mon * sizeof(double),
                                  cudaMemcpyDeviceToDevice),
                       "mon grow");
                sim->dfree(H.d_mon);
                H.d_mon = nb;
                H.mon_cap = cap;
                I.mon = nb;
                I.mon_cap = cap;
                changed = true;
            }
        }
    }
    if (changed) upload_table<real>(sim);
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        ck(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
           "cuTensorMapEncodeTiled lookup");
        if (q != cudaDriverEntryPointSuccess || !p) fail(SJ_E_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// Tensor maps, tiling and block prefixes of the fused schedule.
template <typename real>
void prepare_fused(sj_sim* sim) {
    if (sim->fused_ready) return;
    auto& dv = devv<real>(sim);
    const int n = sim->n_inst, ty = sim->f_ty;
    auto encode = tensor_map_encoder();
    const int nmaps = fused_tensor_maps();
    std::vector<CUtensorMap> maps((size_t)n * nmaps);
    std::vector<long long> pre(2 * (n + 1), 0);
    const int thr = fused_block_threads(ty);
    for (int q = 0; q < n; ++q) {
        InstDev<real>& I = dv[q];
        const cuuint64_t dims[3] = {(cuuint64_t)I.nx, (cuuint64_t)I.ny, (cuuint64_t)I.nz};
        const cuuint32_t es[3] = {1, 1, 1};
        auto enc = [&](CUtensorMap* m, CUtensorMapDataType dt, void* base, size_t esize, cuuint32_t bx,
                       cuuint32_t by) {
            const cuuint64_t strides[2] = {(cuuint64_t)I.px * esize, (cuuint64_t)I.plane * esize};
            const cuuint32_t box[3] = {bx, by, 1};
            CUresult r = encode(m, dt, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) fail(SJ_E_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        };
        const CUtensorMapDataType fdt =
            sizeof(real) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
        const cuuint32_t bx = (cuuint32_t)fused_box_width<real>();
        // slots: [0..5] E[b][c] (halo box), [6..11] H[b][c] (halo box), [12] combo (own box),
        // [13..18] psi_E[a][pair] (own box), [19..30] psi_H[b][a][pair] (own box)
        CUtensorMap* m = &maps[(size_t)q * nmaps];
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 3; ++c) {
                enc(m + b * 3 + c, fdt, I.F[b][c], sizeof(real), bx, (cuuint32_t)(ty + 2));      // E
                enc(m + 6 + b * 3 + c, fdt, I.F[b][3 + c], sizeof(real), bx, (cuuint32_t)(ty + 1));  // H
            }
        enc(m + 12, CU_TENSOR_MAP_DATA_TYPE_UINT8, const_cast<uint8_t*>(I.combo), 1, 32, (cuuint32_t)ty);
        for (int a = 0; a < 3; ++a)
            for (int pp = 0; pp < 2; ++pp) {
                // axes without a slab never issue these loads; encode a valid placeholder
                real* pe = I.psiE[a] ? I.psiE[a] + (size_t)pp * I.vol : I.F[0][0];
                enc(m + 13 + a * 2 + pp, fdt, pe, sizeof(real), 32, (cuuint32_t)ty);
                for (int b = 0; b < 2; ++b) {
                    real* ph = I.psiH[b][a] ? I.psiH[b][a] + (size_t)pp * I.vol : I.F[0][3];
                    enc(m + 19 + b * 6 + a * 2 + pp, fdt, ph, sizeof(real), 32, (cuuint32_t)ty);
                }
            }
        I.f_ntx = (I.nx + 31) / 32;
        I.f_nty = (I.ny + ty - 1) / ty;
        I.f_zs = std::max(1, std::min(sim->f_zs, I.nz));
        I.f_nzs = (I.nz + I.f_zs - 1) / I.f_zs;
        pre[q + 1] = pre[q] + (long long)I.f_ntx * I.f_nty * I.f_nzs;
        pre[n + 1 + q + 1] = pre[n + 1 + q] + (I.n_probe + thr - 1) / thr;
    }
    sim->dfree(sim->d_tmaps);
    sim->dfree(sim->d_fpre);
    sim->d_tmaps = sim->upload(maps);
    sim->d_fpre = sim->upload(pre);
    for (int q = 0; q < n; ++q) dv[q].tmap = reinterpret_cast<const CUtensorMap*>(sim->d_tmaps) + (size_t)q * nmaps;
    FusedLaunch& fl = sim->fl;
    fl.ty = ty;
    fl.ring = sim->f_ring;
    fl.n_items = pre[n];
    fl.n_probe_blocks = pre[2 * n + 1];
    fl.d_item_pre = reinterpret_cast<const long long*>(sim->d_fpre);
    fl.d_probe_pre = reinterpret_cast<const long long*>(sim->d_fpre) + (n + 1);
    fl.dry = 0;
    fl.wait_ns = sim->tma_wait_ns;
    fl.stall = sim->test_stall;
    upload_table<real>(sim);
    sim->fused_ready = true;
}

// Tile lists of the fused schedule for the current z-segment length: every
// instance's tiles by class, in one device buffer.
template <typename real>
void prepare_lean(sj_sim* sim) {
    if (sim->lean_zb == sim->l_zb && sim->d_tiles) return;
    auto& dv = devv<real>(sim);
    std::vector<unsigned> all;
    std::vector<long long> off((size_t)sim->n_inst * LEAN_CLASSES);
    std::vector<unsigned> lists[LEAN_CLASSES];
    std::vector<std::vector<unsigned>> general(sim->n_inst);
    sim->ltiles.assign(sim->n_inst, LeanTiles{});
    for (int q = 0; q < sim->n_inst; ++q) {
        if (2 * dv[q].vol >= (1LL << 32))
            fail(SJ_E_INVALID, "grid too large for the fused schedule's 32-bit offsets (use split or tma)");
        if (lean_classify<real>(dv[q], sim->l_zb, lists) != 0)
            fail(SJ_E_INVALID, "grid too large for the fused schedule's tile codes");
        for (int c = 0; c < LEAN_CLASSES; ++c) {
            off[(size_t)q * LEAN_CLASSES + c] = (long long)all.size();
            sim->ltiles[q].count[c] = (long long)lists[c].size();
            all.insert(all.end(), lists[c].begin(), lists[c].end());
        }
        general[q] = lists[LEAN_GENERAL];
    }
    // Launch groups: a group's launches use its lead's plain, slab and multi
    // lists, so a packed group splits into runs of consecutive members whose
    // lists are equal (a design region turns tiles general in one member
    // only); a run keeps the fixed stride from its own first member.
    auto same_lists = [&](int a, int b) {
        for (int c = 0; c < LEAN_CLASSES; ++c) {
            if (c == LEAN_GENERAL) continue;
            const long long n = sim->ltiles[a].count[c];
            if (sim->ltiles[b].count[c] != n) return false;
            if (n && memcmp(all.data() + off[(size_t)a * LEAN_CLASSES + c],
                            all.data() + off[(size_t)b * LEAN_CLASSES + c], n * sizeof(unsigned)) != 0)
                return false;
        }
        return true;
    };
    sim->lgroups.clear();
    for (const auto& mem : sim->lmembers) {
        size_t first = 0;
        for (size_t r = 1; r <= mem.size(); ++r)
            if (r == mem.size() || !same_lists(mem[first], mem[r])) {
                sim->lgroups.push_back(LeanGroup{mem[first], (int)(r - first)});
                first = r;
            }
    }
    sim->h_tiles = all;
    sim->h_tile_off = off;
    sim->lists_version += 1;
    sim->dfree(sim->d_tiles);
    sim->d_tiles = sim->upload(all);
    const unsigned* base = reinterpret_cast<const unsigned*>(sim->d_tiles);
    for (int q = 0; q < sim->n_inst; ++q)
        for (int c = 0; c < LEAN_CLASSES; ++c)
            sim->ltiles[q].list[c] = base + off[(size_t)q * LEAN_CLASSES + c];
    // the general launch's blocks
    std::vector<int4> gblk;
    lean_gen_blocks<real>(dv.data(), general.data(), sim->n_inst, gblk, sim->lgen.n_tiles);
    sim->lgen.n_all = (long long)gblk.size();
    sim->dfree(sim->d_gen);
    sim->d_gen = sim->upload(gblk);
    sim->lgen.blk = reinterpret_cast<const int4*>(sim->d_gen);
    // correction passes (independent of the tiling)
    std::vector<int2> passes[LEAN_FIX_PASSES];
    lean_fix_blocks<real>(dv.data(), sim->n_inst, passes);
    std::vector<int2> fall;
    long long foff[LEAN_FIX_PASSES];
    for (int p = 0; p < LEAN_FIX_PASSES; ++p) {
        foff[p] = (long long)fall.size();
        sim->lfix.count[p] = (long long)passes[p].size();
        fall.insert(fall.end(), passes[p].begin(), passes[p].end());
    }
    sim->dfree(sim->d_fix);
    sim->d_fix = sim->upload(fall);
    for (int p = 0; p < LEAN_FIX_PASSES; ++p)
        sim->lfix.blk[p] = reinterpret_cast<const int2*>(sim->d_fix) + foff[p];
    sim->lean_zb = sim->l_zb;
}

// Can the fused schedule's tiles run as one queued launch?  FP32, two
// columns per thread, every instance with whole 32-column rows.
template <typename real>
bool queue_eligible(sj_sim* sim) {
    if (sizeof(real) != 4 || sim->l_one_column) return false;
    for (const auto& I : devv<real>(sim))
        if (I.nx % 32 != 0) return false;
    return true;
}

// The queued launch's descriptor tables and items for the current tile lists
// and descriptors (rebuilt when either changes); nullptr when the grouped
// launches run.
template <typename real>
const LeanQueue<real>* prepare_queue(sj_sim* sim) {
    if constexpr (sizeof(real) != 4) {
        return nullptr;
    } else {
        if (sim->l_launch != SJ_LAUNCH_QUEUE || !queue_eligible<real>(sim)) return nullptr;
        if (sim->q_version == sim->table_version && sim->q_lists == sim->lists_version) return &sim->queue;
        const auto& dv = devv<float>(sim);
        const int ng = (int)sim->lgroups.size();
        // [dry][parity][group]
        if (ng > LEAN_QUEUE_GROUPS) return nullptr;  // more groups than one launch's parameters hold
        std::vector<LeanTable<float>>& tabs = sim->q_tabs;
        tabs.assign(4 * (size_t)ng, LeanTable<float>{});
        for (int dry = 0; dry < 2; ++dry)
            for (int par = 0; par < 2; ++par)
                for (int g = 0; g < ng; ++g) {
                    LeanTable<float>& t = tabs[((size_t)dry * 2 + par) * ng + g];
                    memset(&t, 0, sizeof(t));
                    t.inst = dv[sim->lgroups[g].lead];
                    if (par) {
                        for (int c = 0; c < 6; ++c) std::swap(t.inst.F[0][c], t.inst.F[1][c]);
                        for (int a = 0; a < 3; ++a) std::swap(t.inst.psiH[0][a], t.inst.psiH[1][a]);
                    }
                    t.dry = dry;
                    t.qvol = (unsigned)t.inst.vol;
                }
        sim->queue.tabs = tabs.data();
        sim->q_version = sim->table_version;
        if (sim->q_lists == sim->lists_version) return &sim->queue;  // the items still hold
        // items: multi-slab tiles of every group, then single-slab, then plain;
        // groups of larger grids first, members in order
        std::vector<int> order(ng);
        for (int g = 0; g < ng; ++g) order[g] = g;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return dv[sim->lgroups[a].lead].vol > dv[sim->lgroups[b].lead].vol; });
        std::vector<uint4> items;
        for (int cls : {LEAN_MULTI, LEAN_SLAB, LEAN_PLAIN})
            for (int g : order) {
                const int lead = sim->lgroups[g].lead;
                const long long o = sim->h_tile_off[(size_t)lead * LEAN_CLASSES + cls];
                const long long n = sim->ltiles[lead].count[cls];
                for (int r = 0; r < sim->lgroups[g].n; ++r)
                    for (long long t = 0; t < n; ++t)
                        items.push_back(make_uint4((unsigned)g, (unsigned)r, sim->h_tiles[(size_t)(o + t)], 0u));
            }
        if (items.size() >= (1ull << 32)) fail(SJ_E_INVALID, "too many tiles for the queued launch");
        sim->dfree(sim->d_qitems);
        sim->d_qitems = items.empty() ? nullptr : sim->upload(items);
        if (!sim->queue.ctr) sim->queue.ctr = (unsigned*)sim->dalloc(sizeof(unsigned));
        int dev = 0, sms = 0;
        ck(cudaGetDevice(&dev), "device");
        ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
        const int nb = lean_queue_blocks_per_sm(sim->lean_zb);
        if (nb < 1) fail(SJ_E_CUDA, "queued tile kernel cannot be resident");
        sim->queue.items = reinterpret_cast<const uint4*>(sim->d_qitems);
        sim->queue.n_items = (unsigned)items.size();
        sim->queue.n_groups = ng;
        sim->queue.grid = nb * sms;
        sim->q_lists = sim->lists_version;
        return &sim->queue;
    }
}

template <typename real>
void prepare_schedule(sj_sim* sim) {
    if (sim->schedule == SJ_SCHED_TMA) prepare_fused<real>(sim);
    if (sim->schedule == SJ_SCHED_FUSED) {
        prepare_lean<real>(sim);
        prepare_queue<real>(sim);
    }
}

// Side streams and events of the fused schedule, created on first use.
LeanStreams lean_streams(sj_sim* sim) {
    if (!sim->ev_fork) {
        for (int q = 0; q < LEAN_STREAMS; ++q) {
            ck(cudaStreamCreateWithFlags(&sim->side[q], cudaStreamNonBlocking), "side stream");
            ck(cudaEventCreateWithFlags(&sim->ev_join[q], cudaEventDisableTiming), "event");
        }
        ck(cudaEventCreateWithFlags(&sim->ev_fork, cudaEventDisableTiming), "event");
    }
    LeanStreams ls;
    ls.main = sim->stream;
    ls.fork = sim->ev_fork;
    for (int q = 0; q < LEAN_STREAMS; ++q) ls.side[q] = sim->side[q], ls.join[q] = sim->ev_join[q];
    return ls;
}

template <typename real>
const InstDev<real>* parity_table(sj_sim* sim) {
    return reinterpret_cast<const InstDev<real>*>(sim->d_parity);
}

// One step.  The single-pass schedules alternate the ping-pong buffers; the
// host mirror of the parity (sim->cur) flips with every launched step.
template <typename real>
cudaError_t launch_one(sj_sim* sim) {
    auto& dv = devv<real>(sim);
    const InstDev<real>* d = reinterpret_cast<const InstDev<real>*>(sim->d_table);
    cudaError_t e;
    if (sim->schedule == SJ_SCHED_FUSED) {
        prepare_lean<real>(sim);
        const LeanQueue<real>* q = prepare_queue<real>(sim);
        e = launch_lean_step<real>(dv.data(), d, parity_table<real>(sim), sim->ltiles.data(), sim->lgroups.data(),
                                   (int)sim->lgroups.size(), sim->lgen, sim->lfix, sim->n_inst, sim->l_zb, 0, sim->cur,
                                   sim->d_state, lean_streams(sim), sim->l_one_column, q);
    } else if (sim->schedule == SJ_SCHED_TMA) {
        prepare_fused<real>(sim);
        e = launch_fused_step<real>(d, sim->n_inst, sim->d_state, sim->fl, sim->stream);
    } else {
        return launch_split_step<real>(d, dv.data(), sim->n_inst, sim->d_state, sim->stream);
    }
    sim->cur ^= 1;
    return e;
}

// Time `steps` dry launches (no state change) of every tiling candidate and
// keep the fastest: the project's own autotuner for the fused schedule.
// Lean-schedule autotuner: z-segment length by timing dry launches.
template <typename real>
void autotune_lean(sj_sim* sim, int steps, int* best_zs, float* best_ms) {
    const int zbs[3] = {8, 16, 32};
    float best = 1e30f;
    int bzb = sim->l_zb;
    // the queued launch is a candidate where it applies
    const bool try_queue = queue_eligible<real>(sim);
    int blaunch = sim->l_launch;
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    ensure_capacity<real>(sim, sim->t + 1);
    const auto& dv = devv<real>(sim);
    const LeanStreams ls = lean_streams(sim);
    for (int mode = 0; mode < (try_queue ? 2 : 1); ++mode)
    for (int zb : zbs) {
        sim->l_zb = zb;
        if (try_queue) sim->l_launch = mode;
        prepare_lean<real>(sim);
        const LeanQueue<real>* qu = prepare_queue<real>(sim);
        const LeanTiles* lt = sim->ltiles.data();
        const InstDev<real>* d = reinterpret_cast<const InstDev<real>*>(sim->d_table);
        ck(launch_lean_step<real>(dv.data(), d, parity_table<real>(sim), lt, sim->lgroups.data(),
                                  (int)sim->lgroups.size(), sim->lgen, sim->lfix, sim->n_inst, zb, 1, sim->cur,
                                  sim->d_state, ls, sim->l_one_column, qu),
           "autotune");
        ck(cudaEventRecord(e0, sim->stream), "event");
        for (int q = 0; q < steps; ++q)
            ck(launch_lean_step<real>(dv.data(), d, parity_table<real>(sim), lt, sim->lgroups.data(),
                                      (int)sim->lgroups.size(), sim->lgen, sim->lfix, sim->n_inst, zb, 1, sim->cur,
                                      sim->d_state, ls, sim->l_one_column, qu),
               "autotune");
        ck(cudaEventRecord(e1, sim->stream), "event");
        ck(cudaEventSynchronize(e1), "event");
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, e0, e1), "event");
        if (ms < best) {
            best = ms;
            bzb = zb;
            blaunch = sim->l_launch;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sim->l_zb = bzb;
    sim->l_launch = blaunch;
    sim->drop_graphs();
    prepare_lean<real>(sim);
    prepare_queue<real>(sim);
    if (best_zs) *best_zs = bzb;
    if (best_ms) *best_ms = best / steps;
}

template <typename real>
void autotune(sj_sim* sim, int steps, int* best_ty, int* best_ring, int* best_zs, float* best_ms) {
    if (sim->schedule == SJ_SCHED_FUSED) {
        autotune_lean<real>(sim, steps, best_zs, best_ms);
        if (best_ty) *best_ty = 8;
        if (best_ring) *best_ring = 0;
        return;
    }
    int nzmax = 1;
    for (auto& I : devv<real>(sim)) nzmax = std::max(nzmax, I.nz);
    const int tilings[5][2] = {{4, 3}, {8, 3}, {16, 3}, {4, 4}, {8, 4}};
    const int zss[3] = {32, 64, nzmax};
    float best = 1e30f;
    int bty = sim->f_ty, bzs = sim->f_zs, bring = sim->f_ring;
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    ensure_capacity<real>(sim, sim->t + 1);
    for (const auto& tl : tilings)
        for (int zs : zss) {
            const int ty = tl[0], ring = tl[1];
            const int sb = fused_smem_bytes<real>(ty, ring);
            if (sb < 0 || sb > FUSED_MAX_SMEM) continue;  // does not fit one SM
            sim->f_ty = ty;
            sim->f_zs = zs;
            sim->f_ring = ring;
            sim->fused_ready = false;
            prepare_fused<real>(sim);
            FusedLaunch fl = sim->fl;
            fl.dry = 1;
            const InstDev<real>* d = reinterpret_cast<const InstDev<real>*>(sim->d_table);
            ck(launch_fused_step<real>(d, sim->n_inst, sim->d_state, fl, sim->stream), "autotune");
            ck(cudaEventRecord(e0, sim->stream), "event");
            for (int q = 0; q < steps; ++q)
                ck(launch_fused_step<real>(d, sim->n_inst, sim->d_state, fl, sim->stream), "autotune");
            ck(cudaEventRecord(e1, sim->stream), "event");
            ck(cudaEventSynchronize(e1), "event");
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, e0, e1), "event");
            if (ms < best) {
                best = ms;
                bty = ty;
                bzs = zs;
                bring = ring;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sim->f_ty = bty;
    sim->f_zs = bzs;
    sim->f_ring = bring;
    sim->fused_ready = false;
    prepare_fused<real>(sim);
    if (best_ty) *best_ty = bty;
    if (best_zs) *best_zs = bzs;
    if (best_ring) *best_ring = bring;
    if (best_ms) *best_ms = best / steps;
}

// Start the snapshot of instance q due before step sim->t: a dense copy
// into the next free staging slot on the stepping stream (the step after
// next overwrites this buffer), then its host copy on the copy stream.
template <typename real>
void take_snapshot_async(sj_sim* sim, int q) {
    Snapshots& S = sim->snaps[q];
    if (S.count == S.depth)
        fail(SJ_E_RANGE, "snapshot ring full at step " + std::to_string(sim->t) + ": take snapshots first");
    const HostInst<real>& H = hostv<real>(sim)[q];
    const InstDev<real>& I = devv<real>(sim)[q];
    const int slot = (S.head + S.count) % S.depth;
    const size_t row = (size_t)H.nx * sizeof(real);
    ck(cudaMemcpy2DAsync(S.dev[slot], row, I.F[sim->cur][S.comp], (size_t)H.px * sizeof(real), row,
                         (size_t)H.ny * H.nz, cudaMemcpyDeviceToDevice, sim->stream),
       "snapshot staging copy");
    ck(cudaEventRecord(S.staged[slot], sim->stream), "event");
    ck(cudaStreamWaitEvent(sim->copy_stream, S.staged[slot], 0), "event wait");
    ck(cudaMemcpyAsync(S.host[slot], S.dev[slot], row * H.ny * H.nz, cudaMemcpyDeviceToHost, sim->copy_stream),
       "snapshot host copy");
    ck(cudaEventRecord(S.done[slot], sim->copy_stream), "event");
    S.step[slot] = sim->t;
    S.count += 1;
    sim->d2h += (long long)(row * H.ny * H.nz);
}

template <typename real>
void do_steps(sj_sim* sim, long long n) {
    ensure_capacity<real>(sim, sim->t + n);
    if (!sim->any_snapshots()) {
        for (long long q = 0; q < n; ++q) ck(launch_one<real>(sim), "step launch");
        sim->t += n;
        return;
    }
    // with snapshots: step by step, the counter current at every save point
    for (long long q = 0; q < n; ++q) {
        for (int i = 0; i < sim->n_inst; ++i) {
            const Snapshots& S = sim->snaps[i];
            if (S.every > 0 && sim->t % S.every == 0) take_snapshot_async<real>(sim, i);
        }
        ck(launch_one<real>(sim), "step launch");
        sim->t += 1;
    }
}

// Steps in graph replays of `chunk` steps.  The single-pass schedules bake
// the parity into their launches, so a chunk is captured once per starting
// parity it is replayed at (one graph for even chunks, two for odd ones).
template <typename real>
void do_steps_graph(sj_sim* sim, long long n, int chunk) {
    if (chunk < 1) fail(SJ_E_INVALID, "chunk must be >= 1");
    if (sim->any_snapshots()) return do_steps<real>(sim, n);  // save points fall inside chunks
    ensure_capacity<real>(sim, sim->t + n);
    // everything that allocates or copies happens before the capture
    prepare_schedule<real>(sim);
    if (sim->graph_chunk != chunk || sim->graph_sched != sim->schedule || sim->graph_version != sim->table_version)
        sim->drop_graphs();
    sim->graph_chunk = chunk;
    sim->graph_sched = sim->schedule;
    sim->graph_version = sim->table_version;
    const bool flips = sim->schedule != SJ_SCHED_SPLIT;
    long long left = n;
    while (left >= chunk) {
        const int p = flips ? sim->cur : 0;
        if (!sim->graph[p]) {
            cudaStream_t cs;
            ck(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
            cudaStream_t saved = sim->stream;
            const int saved_cur = sim->cur;
            sim->stream = cs;
            cudaGraph_t gr = nullptr;
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                try {
                    for (int q = 0; q < chunk && e == cudaSuccess; ++q) e = launch_one<real>(sim);
                } catch (...) {
                    e = cudaErrorStreamCaptureInvalidated;
                }
                cudaError_t e2 = cudaStreamEndCapture(cs, &gr);
                if (e == cudaSuccess) e = e2;
            }
            sim->stream = saved;
            sim->cur = saved_cur;  // capturing ran nothing
            cudaStreamDestroy(cs);
            if (e != cudaSuccess && gr) cudaGraphDestroy(gr);
            ck(e, "graph capture");
            e = cudaGraphInstantiate(&sim->graph[p], gr, 0);
            cudaGraphDestroy(gr);
            ck(e, "graph instantiate");
        }
        ck(cudaGraphLaunch(sim->graph[p], sim->stream), "graph launch");
        if (flips && (chunk & 1)) sim->cur ^= 1;
        left -= chunk;
    }
    for (long long q = 0; q < left; ++q) ck(launch_one<real>(sim), "step launch");
    sim->t += n;
}

int finish(sj_sim* sim, int code, const std::string& msg) {
    if (sim)
        sim->err = msg;
    else
        g_create_error = msg;
    return code;
}

#define SJ_TRY(sim) try {
#define SJ_CATCH(sim)                                              \
    }                                                              \
    catch (const Fail& f) {                                        \
        return finish(sim, f.code, f.msg);                         \
    }                                                              \
    catch (const std::exception& ex) {                             \
        return finish(sim, SJ_E_INVALID, ex.what());               \
    }                                                              \
    return SJ_OK;

// The divergence record as the host sees it (no synchronisation: the probe
// that trips the guard writes it through host-mapped memory, flag last).
bool diverged(const sj_sim* sim) {
    return sim->h_guard && *reinterpret_cast<const volatile int*>(&sim->h_guard->flag) != 0;
}

void fail_if_diverged(const sj_sim* sim) {
    if (!diverged(sim)) return;
    const volatile GuardRecord* g = sim->h_guard;
    char buf[200];
    snprintf(buf, sizeof buf, "divergence at step %lld: instance %d monitor %d sampled %g (guard %g)",
             (long long)g->step, g->inst, g->monitor, (double)g->value, sim->guard_bound);
    fail(SJ_E_DIVERGED, buf);
}

template <typename real>
void set_guard_t(sj_sim* sim, double bound) {
    ck(cudaStreamSynchronize(sim->stream), "sync");
    sim->guard_bound = bound;
    for (auto& I : devv<real>(sim)) I.guard_bound = bound;
    ck(cudaMemset(sim->d_guard_flag, 0, sizeof(int)), "guard reset");
    memset(sim->h_guard, 0, sizeof(GuardRecord));
    sim->drop_graphs();
    upload_table<real>(sim);
}

int check_status(sj_sim* sim) {
    DevState st;
    ck(cudaStreamSynchronize(sim->stream), "sync");
    ck(cudaMemcpy(&st, sim->d_state, sizeof(st), cudaMemcpyDeviceToHost), "state");
    if (st.status != 0) fail(st.status, "a kernel reported status " + std::to_string(st.status));
    if (st.step != sim->t) fail(SJ_E_CUDA, "device step counter disagrees with host");
    return 0;
}

template <typename real>
void read_field_t(sj_sim* sim, int inst, int comp, double* out) {
    auto& hv = hostv<real>(sim);
    auto& dv = devv<real>(sim);
    const HostInst<real>& H = hv[inst];
    const InstDev<real>& I = dv[inst];
    std::vector<real> tmp((size_t)H.nx * H.ny * H.nz);
    ck(cudaStreamSynchronize(sim->stream), "sync");
    ck(cudaMemcpy2D(tmp.data(), H.nx * sizeof(real), I.F[sim->cur][comp], H.px * sizeof(real),
                    H.nx * sizeof(real), (size_t)H.ny * H.nz, cudaMemcpyDeviceToHost),
       "field read");
    for (size_t q = 0; q < tmp.size(); ++q) out[q] = (double)tmp[q];
}

template <typename real>
void write_field_t(sj_sim* sim, int inst, int comp, const double* in) {
    auto& hv = hostv<real>(sim);
    auto& dv = devv<real>(sim);
    const HostInst<real>& H = hv[inst];
    const InstDev<real>& I = dv[inst];
    std::vector<real> tmp((size_t)H.nx * H.ny * H.nz);
    for (size_t q = 0; q < tmp.size(); ++q) tmp[q] = (real)in[q];
    ck(cudaStreamSynchronize(sim->stream), "sync");
    ck(cudaMemcpy2D(I.F[sim->cur][comp], H.px * sizeof(real), tmp.data(), H.nx * sizeof(real),
                    H.nx * sizeof(real), (size_t)H.ny * H.nz, cudaMemcpyHostToDevice),
       "field write");
}

// ------------------------------------------------------------------ adjoint
template <typename real>
bool any_design(sj_sim* sim) {
    for (const auto& H : hostv<real>(sim))
        if (!H.des_eps.empty()) return true;
    return false;
}

template <typename real>
void set_design_t(sj_sim* sim, int q, const sj_design_desc* d) {
    HostInst<real>& H = hostv<real>(sim)[q];
    InstDev<real>& I = devv<real>(sim)[q];
    long long nd = 1;
    if (d) {
        const int n3[3] = {H.nx, H.ny, H.nz};
        for (int a = 0; a < 3; ++a) {
            if (d->n[a] < 1 || d->lo[a] < 0 || (long long)d->lo[a] + d->n[a] > n3[a])
                fail(SJ_E_INVALID, "design box outside the grid");
            nd *= d->n[a];
        }
        if (!d->eps) fail(SJ_E_INVALID, "design eps is NULL");
        for (long long k = 0; k < nd; ++k)
            if (!(d->eps[k] > 0) || !std::isfinite(d->eps[k])) fail(SJ_E_INVALID, "design eps must be finite and > 0");
    }
    ck(cudaStreamSynchronize(sim->stream), "sync");
    sim->dfree(H.d_dinv);
    H.d_dinv = nullptr;
    H.des_eps.clear();
    I.dinv = nullptr;
    for (int a = 0; a < 3; ++a) I.des_lo[a] = I.des_n[a] = 0;
    if (d) {
        H.des_eps.assign(d->eps, d->eps + nd);
        std::vector<real> inv(nd);
        for (long long k = 0; k < nd; ++k) inv[k] = (real)(1.0 / d->eps[k]);
        H.d_dinv = sim->upload(inv);
        I.dinv = H.d_dinv;
        for (int a = 0; a < 3; ++a) I.des_lo[a] = d->lo[a], I.des_n[a] = d->n[a];
        // the per-voxel eps is applied by the split schedule's E update and by
        // the fused schedule's general tiles; the TMA schedule has neither
        if (sim->schedule == SJ_SCHED_TMA) sim->schedule = SJ_SCHED_FUSED;
    }
    sim->drop_graphs();
    sim->lean_zb = -1;  // the design's tiles move to the general class
    upload_table<real>(sim);
    if (sim->schedule == SJ_SCHED_FUSED) prepare_lean<real>(sim);
}

template <typename real>
void set_dev_step(sj_sim* sim, long long step) {
    DevState st{};
    st.step = step;
    st.done = 0;
    st.cur = sim->cur;
    st.status = 0;
    ck(cudaMemcpyAsync(sim->d_state, &st, sizeof(st), cudaMemcpyHostToDevice, sim->stream), "state");
    ck(cudaStreamSynchronize(sim->stream), "sync");
}

template <typename real>
void adjoint_t(sj_sim* sim, const sj_objective_desc* objs, long long N, long long K, double* grad, size_t cap,
               double* objv, bool backward = true) {
    auto& hv = hostv<real>(sim);
    auto& dv = devv<real>(sim);
    const int ni = sim->n_inst;
    if (N < 1) fail(SJ_E_INVALID, "n_steps must be >= 1");
    if (!objs || !objv) fail(SJ_E_INVALID, "objectives and obj must not be NULL");
    if (K < 1 || K > N) K = N;
    long long total_d = 0;
    for (int q = 0; q < ni; ++q) {
        const sj_objective_desc& ob = objs[q];
        if (ob.n_cells < 0 || (ob.n_cells > 0 && !ob.cells)) fail(SJ_E_INVALID, "bad objective cells");
        if (ob.comp_mask < 1 || ob.comp_mask > 7) fail(SJ_E_INVALID, "objective comp_mask must be in 1..7");
        for (int c = 0; c < ob.n_cells; ++c) {
            const int* x = ob.cells + 3 * c;
            if (x[0] < 0 || x[1] < 0 || x[2] < 0 || x[0] >= hv[q].nx || x[1] >= hv[q].ny || x[2] >= hv[q].nz)
                fail(SJ_E_INVALID, "objective cell outside the grid");
        }
        total_d += (long long)hv[q].des_eps.size();
    }
    if (backward && total_d > 0 && (!grad || (size_t)total_d > cap))
        fail(SJ_E_RANGE, "d_obj_d_eps too small for the design voxels");
    if (!backward) K = N;  // the final state is the only one kept
    if (sim->schedule == SJ_SCHED_TMA) fail(SJ_E_INVALID, "the adjoint steps with the fused or split schedule");
    for (int q = 0; q < ni; ++q)  // the adjoint kernels address an instance with 32-bit offsets
        if ((unsigned long long)dv[q].vol >= (1ull << 31))
            fail(SJ_E_INVALID, "the adjoint takes grids of fewer than 2^31 voxels (row pitch included)");
    ensure_capacity<real>(sim, N);
    prepare_schedule<real>(sim);
    cudaStream_t st = sim->stream;
    std::vector<void*> temps;  // freed at the end
    auto tmp = [&](size_t bytes) {
        void* p = sim->dalloc(bytes);
        temps.push_back(p);
        return p;
    };
    // ---- the state one step needs: fields, psi, polarisations
    struct Arr {
        void* p;
        size_t bytes;
    };
    // the arrays holding the state while the ping-pong parity is p (the
    // fused schedule flips it every step; the split one stays in place)
    auto state_of = [&](int p) {
        std::vector<Arr> v;
        for (int q = 0; q < ni; ++q) {
            const InstDev<real>& I = dv[q];
            const size_t vb = (size_t)I.vol * sizeof(real);
            for (int c = 0; c < 6; ++c) v.push_back({I.F[p][c], vb});
            for (int a = 0; a < 3; ++a)
                if (I.psiE[a]) v.push_back({I.psiE[a], 2 * vb}), v.push_back({I.psiH[p][a], 2 * vb});
            if (I.P) v.push_back({I.P, (size_t)I.n_poles * 6 * I.dvol * sizeof(real)});
        }
        return v;
    };
    size_t sbytes = 0;
    for (const Arr& a : state_of(0)) sbytes += a.bytes;
    const long long nseg = (N + K - 1) / K;
    {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && (size_t)(nseg + 1) * sbytes > free_b) {
            char buf[240];
            snprintf(buf, sizeof buf,
                     "the %lld checkpoints of %.2f GB each need %.1f GB, %.1f GB are free: use a larger "
                     "checkpoint_every (<= 0: one segment)",
                     nseg + 1, sbytes / 1e9, (nseg + 1) * (double)sbytes / 1e9, free_b / 1e9);
            fail(SJ_E_NOMEM, buf);
        }
    }
    char* arena = (char*)tmp((size_t)(nseg + 1) * sbytes);
    std::vector<int> slot_cur(nseg + 1, 0);  // the parity each checkpoint was taken at
    auto save = [&](long long slot) {
        size_t off = (size_t)slot * sbytes;
        for (const Arr& a : state_of(sim->cur)) {
            ck(cudaMemcpyAsync(arena + off, a.p, a.bytes, cudaMemcpyDeviceToDevice, st), "checkpoint");
            off += a.bytes;
        }
        slot_cur[slot] = sim->cur;
    };
    auto restore = [&](long long slot) {
        sim->cur = slot_cur[slot];
        size_t off = (size_t)slot * sbytes;
        for (const Arr& a : state_of(sim->cur)) {
            ck(cudaMemcpyAsync(a.p, arena + off, a.bytes, cudaMemcpyDeviceToDevice, st), "restore");
            off += a.bytes;
        }
    };
    // ---- objective cells and DFT sums
    std::vector<int*> d_cells(ni, nullptr);
    std::vector<double2*> d_D(ni, nullptr);
    for (int q = 0; q < ni; ++q) {
        const int nc = objs[q].n_cells;
        if (nc == 0) continue;
        d_cells[q] = (int*)tmp((size_t)nc * 3 * sizeof(int));
        ck(cudaMemcpyAsync(d_cells[q], objs[q].cells, (size_t)nc * 3 * sizeof(int), cudaMemcpyHostToDevice, st),
           "cells");
        d_D[q] = (double2*)tmp((size_t)nc * 3 * sizeof(double2));
    }
    // ---- forward from rest, keeping the state every K steps and at the end
    for (const Arr& a : state_of(sim->cur)) ck(cudaMemsetAsync(a.p, 0, a.bytes, st), "reset");
    for (int q = 0; q < ni; ++q)
        if (dv[q].dft) ck(cudaMemsetAsync(dv[q].dft, 0, (size_t)hv[q].n_dft * hv[q].n_freq * sizeof(double2), st), "reset");
    sim->t = 0;
    set_dev_step<real>(sim, 0);
    for (long long n = 0; n < N; ++n) {
        if (n % K == 0) save(n / K);
        for (int q = 0; q < ni; ++q)
            ck(launch_objective<real>(dv[q], sim->cur, d_cells[q], objs[q].n_cells, objs[q].comp_mask,
                                      objs[q].frequency, d_D[q], n, true, nullptr, st),
               "objective");
        ck(launch_one<real>(sim), "step launch");
    }
    save(nseg);
    std::vector<std::vector<double2>> dft_keep(ni);
    ck(cudaStreamSynchronize(st), "sync");
    for (int q = 0; q < ni; ++q) {
        if (dv[q].dft) {
            dft_keep[q].resize((size_t)hv[q].n_dft * hv[q].n_freq);
            ck(cudaMemcpy(dft_keep[q].data(), dv[q].dft, dft_keep[q].size() * sizeof(double2), cudaMemcpyDeviceToHost),
               "dft");
        }
        double F = 0;
        if (objs[q].n_cells) {
            std::vector<double2> D((size_t)objs[q].n_cells * 3);
            ck(cudaMemcpy(D.data(), d_D[q], D.size() * sizeof(double2), cudaMemcpyDeviceToHost), "objective");
            for (const double2& v : D) F += v.x * v.x + v.y * v.y;
        }
        objv[q] = F;
    }
    if (!backward) {
        sim->t = N;  // the device counter advanced with the steps
        for (void* p : temps) sim->dfree(p);
        return;
    }
    // ---- adjoint buffers
    std::vector<AdjDev<real>> A(ni);
    for (int q = 0; q < ni; ++q) {
        const InstDev<real>& I = dv[q];
        AdjDev<real>& a = A[q];
        memset(&a, 0, sizeof(a));
        a.I = I;
        const size_t vb = (size_t)I.vol * sizeof(real);
        for (int c = 0; c < 3; ++c) {
            a.eb[c] = (real*)tmp(vb);
            a.hb[c] = (real*)tmp(vb);
            a.t1[c] = (real*)tmp(vb);
            a.t2[c] = (real*)tmp(vb);
            a.t3[c] = (real*)tmp(vb);
            a.t4[c] = (real*)tmp(vb);
        }
        for (int ax = 0; ax < 3; ++ax)
            if (I.psiE[ax]) a.psEb[ax] = (real*)tmp(2 * vb), a.psHb[ax] = (real*)tmp(2 * vb);
        if (I.P) a.pb = (real*)tmp((size_t)I.n_poles * 6 * I.dvol * sizeof(real));
        const long long nd = (long long)hv[q].des_eps.size();
        if (nd) {
            a.rec = (const real*)tmp((size_t)K * nd * 3 * sizeof(real));
            a.g = (double*)tmp((size_t)nd * 3 * sizeof(double));
        }
    }
    // ---- backwards, one segment at a time: re-run it forward recording acc
    // at the design points, then its transposed steps in reverse
    bool first = true;  // the sweep's first transposed step has no gather to fold in
    for (long long seg = nseg - 1; seg >= 0; --seg) {
        const long long t0 = seg * K, t1 = std::min(N, t0 + K);
        restore(seg);
        sim->t = t0;
        set_dev_step<real>(sim, t0);
        for (int q = 0; q < ni; ++q)
            if (A[q].rec) dv[q].rec_acc = const_cast<real*>(A[q].rec), dv[q].rec_t0 = t0, dv[q].rec_len = t1 - t0;
        upload_table<real>(sim);
        for (long long n = t0; n < t1; ++n) ck(launch_one<real>(sim), "step launch");
        for (int q = 0; q < ni; ++q) dv[q].rec_acc = nullptr, dv[q].rec_len = 0;
        upload_table<real>(sim);
        for (long long n = t1 - 1; n >= t0; --n, first = false)
            for (int q = 0; q < ni; ++q) {
                A[q].rec_t0 = t0;
                ck(launch_adjoint_step<real>(A[q], n, first, st), "adjoint step");
                ck(launch_objective<real>(dv[q], sim->cur, d_cells[q], objs[q].n_cells, objs[q].comp_mask,
                                          objs[q].frequency, d_D[q], n, false, A[q].eb, st),
                   "adjoint source");
            }
    }
    // ---- back to the state after N steps
    restore(nseg);
    sim->t = N;
    set_dev_step<real>(sim, N);
    for (int q = 0; q < ni; ++q)
        if (dv[q].dft)
            ck(cudaMemcpy(dv[q].dft, dft_keep[q].data(), dft_keep[q].size() * sizeof(double2), cudaMemcpyHostToDevice),
               "dft");
    // ---- dF/d(eps) = -eps^{-2} sum_c dF/d(inverse eps at the voxel's E_c point)
    long long off = 0;
    for (int q = 0; q < ni; ++q) {
        const long long nd = (long long)hv[q].des_eps.size();
        if (!nd) continue;
        std::vector<double> g((size_t)nd * 3);
        ck(cudaMemcpy(g.data(), A[q].g, g.size() * sizeof(double), cudaMemcpyDeviceToHost), "gradient");
        for (long long d = 0; d < nd; ++d) {
            const double e = hv[q].des_eps[d];
            grad[off + d] = -(g[3 * d] + g[3 * d + 1] + g[3 * d + 2]) / (e * e);
        }
        off += nd;
    }
    for (void* p : temps) sim->dfree(p);
}

template <typename T>
bool same_bits(const std::vector<T>& a, const std::vector<T>& b) {
    return a.size() == b.size() && (a.empty() || memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

// Can instances a and b share tile launches?  Their tile lists depend on
// the grid, the CPML slabs and the H-source boxes; the tile kernels read the
// time step, the CPML profiles and the coefficient table from the lead's
// descriptor, so those must agree bit for bit.
template <typename real>
bool same_tiles(const HostInst<real>& ha, const InstDev<real>& a, const HostInst<real>& hb, const InstDev<real>& b) {
    if (a.nx != b.nx || a.ny != b.ny || a.nz != b.nz || a.px != b.px) return false;
    if (memcmp(&a.S, &b.S, sizeof(real)) != 0) return false;
    for (int ax = 0; ax < 3; ++ax)
        if (a.pl[ax] != b.pl[ax] || a.ph[ax] != b.ph[ax] || !same_bits(ha.prof[ax], hb.prof[ax])) return false;
    if (a.ncoef != b.ncoef || a.n_combos != b.n_combos || !same_bits(ha.coef, hb.coef)) return false;
    auto hboxes = [](const InstDev<real>& I) {
        std::vector<int> v;
        for (int s = 0; s < I.n_src; ++s)
            if (I.src[s].comp >= 3) {
                v.push_back(I.src[s].comp);
                for (int ax = 0; ax < 3; ++ax) v.push_back(I.src[s].lo[ax]), v.push_back(I.src[s].n[ax]);
            }
        return v;
    };
    return hboxes(a) == hboxes(b);
}

// Move the arrays of `members` (one group, lead first) into one allocation
// per array: fields and combo bytes of member r at r * vol elements from the
// lead's, psi at r * 2 * vol.
template <typename real>
void pack_group(sj_sim* sim, const std::vector<int>& members) {
    auto& dv = devv<real>(sim);
    const long long vol = dv[members[0]].vol;
    const size_t G = members.size();
    cudaStream_t st = sim->stream;
    auto pack = [&](auto get, size_t bytes) {  // get(q) -> reference to instance q's pointer
        char* arena = (char*)sim->dalloc(G * bytes, false);
        for (size_t r = 0; r < G; ++r)
            ck(cudaMemcpyAsync(arena + r * bytes, get(members[r]), bytes, cudaMemcpyDeviceToDevice, st), "pack");
        ck(cudaStreamSynchronize(st), "pack sync");
        for (size_t r = 0; r < G; ++r) {
            auto& ptr = get(members[r]);
            sim->dfree((void*)ptr);
            ptr = reinterpret_cast<std::remove_reference_t<decltype(ptr)>>(arena + r * bytes);
        }
    };
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 6; ++c) pack([&](int q) -> real*& { return dv[q].F[b][c]; }, vol * sizeof(real));
    pack([&](int q) -> const uint8_t*& { return dv[q].combo; }, (size_t)vol);
    for (int a = 0; a < 3; ++a) {
        if (!dv[members[0]].psiE[a]) continue;
        pack([&](int q) -> real*& { return dv[q].psiE[a]; }, 2 * vol * sizeof(real));
        for (int b = 0; b < 2; ++b) pack([&](int q) -> real*& { return dv[q].psiH[b][a]; }, 2 * vol * sizeof(real));
    }
}

// Sort the instances into LeanGroups (first fit, in instance order) and
// pack each group of two or more.  A group's psi offsets (2 r vol + 2 vol)
// stay below 2^32 elements.
template <typename real>
void group_instances(sj_sim* sim) {
    auto& hv = hostv<real>(sim);
    auto& dv = devv<real>(sim);
    std::vector<std::vector<int>> groups;
    for (int q = 0; q < sim->n_inst; ++q) {
        bool placed = false;
        for (auto& g : groups) {
            const int lead = g[0];
            const long long cap = ((1LL << 32) - 1) / (2 * dv[lead].vol);
            if ((long long)g.size() < std::min(cap, 65535LL) && same_tiles(hv[lead], dv[lead], hv[q], dv[q])) {
                g.push_back(q);
                placed = true;
                break;
            }
        }
        if (!placed) groups.push_back({q});
    }
    sim->lgroups.clear();
    sim->lmembers = groups;
    for (const auto& g : groups) {
        if (g.size() > 1) pack_group<real>(sim, g);
        sim->lgroups.push_back(LeanGroup{g[0], (int)g.size()});
    }
}

template <typename real>
void create_t(sj_sim* sim, int n, const sj_instance_desc* insts) {
    auto& hv = hostv<real>(sim);
    auto& dv = devv<real>(sim);
    hv.resize(n);
    dv.resize(n);
    for (int q = 0; q < n; ++q) {
        build_instance<real>(sim, insts[q], hv[q], dv[q]);
        dv[q].index = q;
        dv[q].guard_bound = sim->guard_bound;
        dv[q].guard_flag = sim->d_guard_flag;
        dv[q].guard = sim->d_guard;
    }
    sim->snaps.assign(n, Snapshots{});
    group_instances<real>(sim);
    upload_table<real>(sim);
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

int sj_abi_version(void) { return SJ_ABI_VERSION; }

int64_t sj_abi_struct_size(int32_t which) {
    switch (which) {
        case 0: return sizeof(sj_grid_desc);
        case 1: return sizeof(sj_pole);
        case 2: return sizeof(sj_csg_node);
        case 3: return sizeof(sj_region_desc);
        case 4: return sizeof(sj_scene_desc);
        case 5: return sizeof(sj_material_desc);
        case 6: return sizeof(sj_pml_desc);
        case 7: return sizeof(sj_source_desc);
        case 8: return sizeof(sj_probe_desc);
        case 9: return sizeof(sj_instance_desc);
        case 10: return sizeof(sj_design_desc);
        case 11: return sizeof(sj_objective_desc);
        case 12: return sizeof(sj_phase_result);
        default: return -1;
    }
}

const char* sj_last_error(const sj_sim* sim) {
    return sim ? sim->err.c_str() : g_create_error.c_str();
}

int sj_batch_create(int32_t n, const sj_instance_desc* insts, int32_t precision, sj_sim** out) {
    if (!out) return finish(nullptr, SJ_E_INVALID, "out is NULL");
    *out = nullptr;
    if (n < 1 || !insts) return finish(nullptr, SJ_E_INVALID, "need at least one instance");
    if (precision != SJ_F64 && precision != SJ_F32) return finish(nullptr, SJ_E_INVALID, "bad precision");
    std::unique_ptr<sj_sim> sim(new sj_sim());
    try {
        sim->precision = precision;
        sim->n_inst = n;
        // the fused single pass is the fastest schedule in both precisions
        sim->schedule = SJ_SCHED_FUSED;
        ck(cudaStreamCreateWithFlags(&sim->stream, cudaStreamNonBlocking), "stream create");
        sim->own_stream = true;
        sim->d_state = (DevState*)sim->dalloc(sizeof(DevState));
        sim->d_scratch = (double*)sim->dalloc(64);
        sim->d_guard_flag = (int*)sim->dalloc(sizeof(int));
        ck(cudaHostAlloc((void**)&sim->h_guard, sizeof(GuardRecord), cudaHostAllocMapped), "guard record");
        memset(sim->h_guard, 0, sizeof(GuardRecord));
        ck(cudaHostGetDevicePointer((void**)&sim->d_guard, sim->h_guard, 0), "guard record address");
        if (precision == SJ_F64)
            create_t<double>(sim.get(), n, insts);
        else
            create_t<float>(sim.get(), n, insts);
        ck(cudaStreamSynchronize(sim->stream), "create sync");
    } catch (const Fail& f) {
        return finish(nullptr, f.code, f.msg);
    } catch (const std::exception& ex) {
        return finish(nullptr, SJ_E_NOMEM, ex.what());
    }
    *out = sim.release();
    return SJ_OK;
}

int sj_create(const sj_instance_desc* inst, int32_t precision, sj_sim** out) {
    return sj_batch_create(1, inst, precision, out);
}

int sj_destroy(sj_sim* sim) {
    delete sim;
    return SJ_OK;
}

int sj_set_stream(sj_sim* sim, void* stream) {
    if (!sim) return SJ_E_INVALID;
    SJ_TRY(sim)
    ck(cudaStreamSynchronize(sim->stream), "sync");
    if (sim->own_stream) cudaStreamDestroy(sim->stream);
    if (stream) {
        sim->stream = (cudaStream_t)stream;
        sim->own_stream = false;
    } else {
        ck(cudaStreamCreateWithFlags(&sim->stream, cudaStreamNonBlocking), "stream create");
        sim->own_stream = true;
    }
    SJ_CATCH(sim)
}

int32_t sj_get_schedule(const sj_sim* sim) { return sim ? sim->schedule : -1; }

int sj_set_schedule(sj_sim* sim, int32_t schedule) {
    if (!sim) return SJ_E_INVALID;
    if (schedule != SJ_SCHED_FUSED && schedule != SJ_SCHED_SPLIT && schedule != SJ_SCHED_TMA)
        return finish(sim, SJ_E_INVALID, "unknown schedule");
    const bool des = sim->precision == SJ_F64 ? any_design<double>(sim) : any_design<float>(sim);
    if (des && schedule == SJ_SCHED_TMA)
        return finish(sim, SJ_E_INVALID, "instances with a design region step with the fused or split schedule");
    sim->schedule = schedule;
    return SJ_OK;
}

int sj_set_design(sj_sim* sim, int32_t inst, const sj_design_desc* design) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return SJ_E_INVALID;
    SJ_TRY(sim)
    if (sim->precision == SJ_F64)
        set_design_t<double>(sim, inst, design);
    else
        set_design_t<float>(sim, inst, design);
    SJ_CATCH(sim)
}

int sj_objective(sj_sim* sim, const sj_objective_desc* objectives, int64_t n_steps, double* obj) {
    if (!sim) return SJ_E_INVALID;
    SJ_TRY(sim)
    if (sim->precision == SJ_F64)
        adjoint_t<double>(sim, objectives, n_steps, n_steps, nullptr, 0, obj, false);
    else
        adjoint_t<float>(sim, objectives, n_steps, n_steps, nullptr, 0, obj, false);
    SJ_CATCH(sim)
}

int sj_adjoint_gradient(sj_sim* sim, const sj_objective_desc* objectives, int64_t n_steps, int32_t checkpoint_every,
                        double* d_obj_d_eps, size_t cap, double* obj) {
    if (!sim) return SJ_E_INVALID;
    SJ_TRY(sim)
    if (sim->precision == SJ_F64)
        adjoint_t<double>(sim, objectives, n_steps, checkpoint_every, d_obj_d_eps, cap, obj);
    else
        adjoint_t<float>(sim, objectives, n_steps, checkpoint_every, d_obj_d_eps, cap, obj);
    SJ_CATCH(sim)
}

int sj_set_tiling(sj_sim* sim, int32_t tile_y, int32_t ring, int32_t zseg) {
    if (!sim) return SJ_E_INVALID;
    if (sim->schedule == SJ_SCHED_FUSED) {
        if (zseg != 8 && zseg != 16 && zseg != 32)
            return finish(sim, SJ_E_INVALID, "fused schedule: zseg must be 8, 16 or 32");
        sim->l_zb = zseg;
        sim->drop_graphs();
        return SJ_OK;
    }
    const int sb = sim->precision == SJ_F64 ? fused_smem_bytes<double>(tile_y, ring)
                                            : fused_smem_bytes<float>(tile_y, ring);
    if (sb < 0) return finish(sim, SJ_E_INVALID, "unsupported tiling (tile_y, ring)");
    if (sb > FUSED_MAX_SMEM) return finish(sim, SJ_E_INVALID, "tiling needs more shared memory than one SM has");
    if (zseg < 1) return finish(sim, SJ_E_INVALID, "zseg must be >= 1");
    sim->f_ty = tile_y;
    sim->f_ring = ring;
    sim->f_zs = zseg;
    sim->fused_ready = false;
    sim->drop_graphs();
    return SJ_OK;
}

int sj_set_fused_columns(sj_sim* sim, int32_t columns) {
    if (!sim) return SJ_E_INVALID;
    if (columns != 0 && columns != 1) return finish(sim, SJ_E_INVALID, "columns must be 0 (automatic) or 1");
    sim->l_one_column = columns;
    sim->drop_graphs();
    return SJ_OK;
}

int sj_set_fused_launch(sj_sim* sim, int32_t mode) {
    if (!sim) return SJ_E_INVALID;
    if (mode != SJ_LAUNCH_GROUPED && mode != SJ_LAUNCH_QUEUE) return finish(sim, SJ_E_INVALID, "bad launch mode");
    SJ_TRY(sim)
    if (mode == SJ_LAUNCH_QUEUE) {
        const bool ok = sim->precision == SJ_F32 ? queue_eligible<float>(sim) : false;
        if (!ok)
            fail(SJ_E_INVALID, "the queued launch runs FP32 two-column tiles: every instance's nx must be a "
                               "multiple of 32 and one column per thread off");
    }
    ck(cudaStreamSynchronize(sim->stream), "sync");
    sim->l_launch = mode;
    sim->drop_graphs();
    SJ_CATCH(sim)
}

int32_t sj_get_fused_launch(const sj_sim* sim) { return sim ? sim->l_launch : -1; }

int sj_get_tiling(const sj_sim* sim, int32_t* tile_y, int32_t* ring, int32_t* zseg) {
    if (!sim || !tile_y || !ring || !zseg) return SJ_E_INVALID;
    if (sim->schedule == SJ_SCHED_FUSED) {
        *tile_y = 8;
        *ring = 0;
        *zseg = sim->l_zb;
        return SJ_OK;
    }
    *tile_y = sim->f_ty;
    *ring = sim->f_ring;
    *zseg = sim->f_zs;
    return SJ_OK;
}

int sj_autotune(sj_sim* sim, int32_t steps, int32_t* tile_y, int32_t* ring, int32_t* zseg,
                float* ms_per_step) {
    if (!sim || steps < 1) return SJ_E_INVALID;
    SJ_TRY(sim)
    sim->drop_graphs();
    if (sim->precision == SJ_F64)
        autotune<double>(sim, steps, tile_y, ring, zseg, ms_per_step);
    else
        autotune<float>(sim, steps, tile_y, ring, zseg, ms_per_step);
    check_status(sim);
    SJ_CATCH(sim)
}

int sj_synchronize(sj_sim* sim) {
    if (!sim) return SJ_E_INVALID;
    SJ_TRY(sim)
    check_status(sim);
    fail_if_diverged(sim);
    SJ_CATCH(sim)
}

int sj_set_wait_limit(sj_sim* sim, int64_t ns) {
    if (!sim) return SJ_E_INVALID;
    if (ns < 0 || ns > 10000000000ll) return finish(sim, SJ_E_INVALID, "wait limit must be in [0, 10 s]");
    SJ_TRY(sim)
    ck(cudaStreamSynchronize(sim->stream), "sync");
    sim->tma_wait_ns = (unsigned long long)ns;
    sim->fl.wait_ns = sim->tma_wait_ns;
    sim->drop_graphs();
    SJ_CATCH(sim)
}

int sj_set_test_stall(sj_sim* sim, int32_t on) {
    if (!sim) return SJ_E_INVALID;
    SJ_TRY(sim)
    ck(cudaStreamSynchronize(sim->stream), "sync");
    sim->test_stall = on ? 1 : 0;
    sim->fl.stall = sim->test_stall;
    sim->drop_graphs();
    SJ_CATCH(sim)
}

int sj_set_divergence_guard(sj_sim* sim, double bound) {
    if (!sim) return SJ_E_INVALID;
    if (!(bound >= 0)) return finish(sim, SJ_E_INVALID, "guard bound must be >= 0 (0 = off)");
    SJ_TRY(sim)
    if (sim->precision == SJ_F64)
        set_guard_t<double>(sim, bound);
    else
        set_guard_t<float>(sim, bound);
    SJ_CATCH(sim)
}

int sj_divergence(const sj_sim* sim, int64_t* step, int32_t* inst, int32_t* monitor, double* value) {
    if (!sim) return -1;
    if (!diverged(sim)) return 0;
    const volatile GuardRecord* g = sim->h_guard;
    if (step) *step = g->step;
    if (inst) *inst = g->inst;
    if (monitor) *monitor = g->monitor;
    if (value) *value = g->value;
    return 1;
}

int sj_step(sj_sim* sim, int64_t n) {
    if (!sim) return SJ_E_INVALID;
    if (n < 0) return finish(sim, SJ_E_INVALID, "n_steps < 0");
    SJ_TRY(sim)
    fail_if_diverged(sim);
    if (sim->precision == SJ_F64)
        do_steps<double>(sim, n);
    else
        do_steps<float>(sim, n);
    SJ_CATCH(sim)
}

int sj_step_graph(sj_sim* sim, int64_t n, int32_t chunk) {
    if (!sim) return SJ_E_INVALID;
    if (n < 0) return finish(sim, SJ_E_INVALID, "n_steps < 0");
    SJ_TRY(sim)
    fail_if_diverged(sim);
    if (sim->precision == SJ_F64)
        do_steps_graph<double>(sim, n, chunk);
    else
        do_steps_graph<float>(sim, n, chunk);
    SJ_CATCH(sim)
}

int64_t sj_steps_done(const sj_sim* sim) { return sim ? sim->t : -1; }

int sj_transfer_bytes(const sj_sim* sim, int64_t* h2d, int64_t* d2h) {
    if (!sim || !h2d || !d2h) return SJ_E_INVALID;
    *h2d = sim->h2d;
    *d2h = sim->d2h;
    return SJ_OK;
}
int32_t sj_n_instances(const sj_sim* sim) { return sim ? sim->n_inst : -1; }

#define INST_GET(field, bad)                                                                  \
    if (!sim || inst < 0 || inst >= sim->n_inst) return bad;                                  \
    return sim->precision == SJ_F64 ? sim->hi64[inst].field : sim->hi32[inst].field;

double sj_dt(const sj_sim* sim, int32_t inst) { INST_GET(dt, NAN) }
double sj_time(const sj_sim* sim, int32_t inst) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return NAN;
    return sim->t * sj_dt(sim, inst);
}
double sj_last_source_time(const sj_sim* sim, int32_t inst) { INST_GET(last_source_time, NAN) }
int64_t sj_voxels(const sj_sim* sim, int32_t inst) { INST_GET(voxels, -1) }
double sj_bytes_per_step(const sj_sim* sim, int32_t inst) { INST_GET(bytes_per_step, NAN) }
int32_t sj_launches_per_step(const sj_sim* sim) {
    if (!sim) return -1;
    if (sim->schedule == SJ_SCHED_FUSED) {
        // counts from the tile classification (the lists need not be on the device yet)
        std::vector<LeanTiles> lt(sim->n_inst);
        std::vector<unsigned> lists[LEAN_CLASSES];
        std::vector<int2> passes[LEAN_FIX_PASSES];
        LeanFix fx{};
        for (int q = 0; q < sim->n_inst; ++q) {
            const int r = sim->precision == SJ_F64 ? lean_classify(sim->h64[q], sim->l_zb, lists)
                                                   : lean_classify(sim->h32[q], sim->l_zb, lists);
            if (r != 0) return -1;
            for (int c = 0; c < LEAN_CLASSES; ++c) lt[q].count[c] = (long long)lists[c].size();
        }
        if (sim->precision == SJ_F64)
            lean_fix_blocks(sim->h64.data(), sim->n_inst, passes);
        else
            lean_fix_blocks(sim->h32.data(), sim->n_inst, passes);
        for (int p = 0; p < LEAN_FIX_PASSES; ++p) fx.count[p] = (long long)passes[p].size();
        const LeanGroup* lg = sim->lgroups.data();
        const int ng = (int)sim->lgroups.size();
        sj_sim* ms = const_cast<sj_sim*>(sim);
        if (sim->precision == SJ_F32 && sim->l_launch == SJ_LAUNCH_QUEUE && queue_eligible<float>(ms) &&
            ng <= LEAN_QUEUE_GROUPS) {
            // one queued launch for every group's plain, slab and multi tiles
            int total = 1;
            for (int p = 0; p < LEAN_FIX_PASSES; ++p) total += fx.count[p] > 0;
            for (int q = 0; q < sim->n_inst; ++q)
                if (lt[q].count[LEAN_PLAIN] + lt[q].count[LEAN_SLAB] + lt[q].count[LEAN_MULTI] > 0) return total + 1;
            return total;
        }
        return lean_launches(lt.data(), lg, ng, fx);
    }
    if (sim->schedule == SJ_SCHED_TMA) return 1;
    int maxp = 0;
    for (int q = 0; q < sim->n_inst; ++q)
        maxp = std::max(maxp, sim->precision == SJ_F64 ? sim->h64[q].n_probe : sim->h32[q].n_probe);
    return maxp > 0 ? 3 : 2;  // probe, H pass, E pass
}
int64_t sj_n_samples(const sj_sim* sim, int32_t inst) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return -1;
    const int ss = sim->precision == SJ_F64 ? sim->hi64[inst].save_span : sim->hi32[inst].save_span;
    return (sim->t + ss - 1) / ss;
}

int64_t sj_monitor_spectrum_length(const sj_sim* sim, int32_t inst) {
    const int64_t n = sj_n_samples(sim, inst);
    if (n < 1) return n < 0 ? -1 : 0;
    // as the reference computes it: (unsigned long)(log(N) / log(2))
    const unsigned long l2 = (unsigned long)(std::log((double)n) / std::log(2.0));
    return (int64_t)1 << l2;
}

int sj_monitor_spectrum(sj_sim* sim, int32_t inst, double* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return SJ_E_INVALID;
    SJ_TRY(sim)
    check_status(sim);
    const int nm = sim->precision == SJ_F64 ? sim->hi64[inst].n_mon : sim->hi32[inst].n_mon;
    const double* dm = sim->precision == SJ_F64 ? sim->hi64[inst].d_mon : sim->hi32[inst].d_mon;
    const long long n = sj_n_samples(sim, inst), np = sj_monitor_spectrum_length(sim, inst);
    if ((size_t)nm * np * 2 > cap) fail(SJ_E_RANGE, "out too small: n_monitors * length * 2 doubles");
    if (nm > 0 && np > 0) {
        double* d_out = (double*)sim->dalloc((size_t)nm * np * 2 * sizeof(double), false);
        cudaError_t e = launch_spectrum(dm, nm, n, np, d_out, sim->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sim->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy(out, d_out, (size_t)nm * np * 2 * sizeof(double), cudaMemcpyDeviceToHost);
        sim->dfree(d_out);
        ck(e, "monitor spectrum");
        sim->d2h += (long long)nm * np * 2 * sizeof(double);
    }
    SJ_CATCH(sim)
}

int sj_read_monitors(sj_sim* sim, int32_t inst, double* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return SJ_E_INVALID;
    SJ_TRY(sim)
    check_status(sim);
    const int nm = sim->precision == SJ_F64 ? sim->hi64[inst].n_mon : sim->hi32[inst].n_mon;
    double* dm = sim->precision == SJ_F64 ? sim->hi64[inst].d_mon : sim->hi32[inst].d_mon;
    const long long ns = sj_n_samples(sim, inst);
    if ((size_t)nm * ns > cap) fail(SJ_E_RANGE, "output buffer too small for monitors");
    if (nm == 0 || ns == 0) return SJ_OK;
    std::vector<double> tmp((size_t)nm * ns);
    ck(cudaMemcpy(tmp.data(), dm, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost), "mon read");
    sim->d2h += (long long)(tmp.size() * sizeof(double));
    for (long long s = 0; s < ns; ++s)
        for (int m = 0; m < nm; ++m) out[(size_t)m * ns + s] = tmp[(size_t)s * nm + m];
    SJ_CATCH(sim)
}

int sj_read_dft(sj_sim* sim, int32_t inst, double* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return SJ_E_INVALID;
    SJ_TRY(sim)
    check_status(sim);
    int nd, nf;
    double2* p;
    if (sim->precision == SJ_F64) {
        nd = sim->hi64[inst].n_dft, nf = sim->hi64[inst].n_freq, p = sim->h64[inst].dft;
    } else {
        nd = sim->hi32[inst].n_dft, nf = sim->hi32[inst].n_freq, p = sim->h32[inst].dft;
    }
    if ((size_t)nd * nf * 2 > cap) fail(SJ_E_RANGE, "output buffer too small for DFT");
    if (nd && nf) ck(cudaMemcpy(out, p, (size_t)nd * nf * sizeof(double2), cudaMemcpyDeviceToHost), "dft read");
    sim->d2h += (long long)nd * nf * sizeof(double2);
    SJ_CATCH(sim)
}

int sj_set_snapshots(sj_sim* sim, int32_t inst, int32_t comp, int32_t every, int32_t depth) {
    if (!sim || inst < 0 || inst >= sim->n_inst || comp < 0 || comp > 5) return SJ_E_INVALID;
    SJ_TRY(sim)
    if (every < 0) fail(SJ_E_INVALID, "every must be >= 0");
    if (every > 0 && (depth < 1 || depth > 64)) fail(SJ_E_INVALID, "depth must be in [1, 64]");
    ck(cudaStreamSynchronize(sim->stream), "sync");
    if (sim->copy_stream) ck(cudaStreamSynchronize(sim->copy_stream), "sync");
    sim->release(sim->snaps[inst]);
    if (every > 0) {
        if (!sim->copy_stream)
            ck(cudaStreamCreateWithFlags(&sim->copy_stream, cudaStreamNonBlocking), "copy stream");
        const size_t bytes = (size_t)sj_voxels(sim, inst) * (sim->precision == SJ_F64 ? 8 : 4);
        Snapshots& S = sim->snaps[inst];
        S.comp = comp, S.every = every, S.depth = depth;
        S.step.assign(depth, -1);
        for (int k = 0; k < depth; ++k) {
            void* h = nullptr;
            cudaEvent_t a = nullptr, b = nullptr;
            if (cudaMallocHost(&h, bytes) != cudaSuccess) {
                sim->release(S);
                fail(SJ_E_NOMEM, "pinned snapshot buffer of " + std::to_string(bytes) + " bytes");
            }
            S.host.push_back(h);
            S.dev.push_back(sim->dalloc(bytes, false));
            ck(cudaEventCreateWithFlags(&a, cudaEventDisableTiming), "event");
            S.staged.push_back(a);
            ck(cudaEventCreateWithFlags(&b, cudaEventDisableTiming), "event");
            S.done.push_back(b);
        }
    }
    SJ_CATCH(sim)
}

int sj_take_snapshot(sj_sim* sim, int32_t inst, int64_t* step, double* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst || !step) return SJ_E_INVALID;
    SJ_TRY(sim)
    Snapshots& S = sim->snaps[inst];
    *step = -1;
    if (S.count > 0) {
        const size_t nv = (size_t)sj_voxels(sim, inst);
        if (!out || nv > cap) fail(SJ_E_RANGE, "output buffer too small for the snapshot");
        const int slot = S.head;
        ck(cudaEventSynchronize(S.done[slot]), "snapshot wait");
        if (sim->precision == SJ_F64) {
            memcpy(out, S.host[slot], nv * sizeof(double));
        } else {
            const float* h = (const float*)S.host[slot];
            for (size_t k = 0; k < nv; ++k) out[k] = (double)h[k];
        }
        *step = S.step[slot];
        S.head = (S.head + 1) % S.depth;
        S.count -= 1;
    }
    SJ_CATCH(sim)
}

int32_t sj_snapshots_pending(const sj_sim* sim, int32_t inst) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return -1;
    return sim->snaps[inst].count;
}

int sj_read_field(sj_sim* sim, int32_t inst, int32_t comp, double* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst || comp < 0 || comp > 5) return SJ_E_INVALID;
    SJ_TRY(sim)
    if ((size_t)sj_voxels(sim, inst) > cap) fail(SJ_E_RANGE, "output buffer too small for field");
    if (sim->precision == SJ_F64)
        read_field_t<double>(sim, inst, comp, out);
    else
        read_field_t<float>(sim, inst, comp, out);
    SJ_CATCH(sim)
}

int sj_write_field(sj_sim* sim, int32_t inst, int32_t comp, const double* in, size_t n) {
    if (!sim || inst < 0 || inst >= sim->n_inst || comp < 0 || comp > 5) return SJ_E_INVALID;
    SJ_TRY(sim)
    if ((size_t)sj_voxels(sim, inst) != n) fail(SJ_E_RANGE, "field size mismatch");
    if (sim->precision == SJ_F64)
        write_field_t<double>(sim, inst, comp, in);
    else
        write_field_t<float>(sim, inst, comp, in);
    SJ_CATCH(sim)
}

int sj_read_class_map(sj_sim* sim, int32_t inst, uint8_t* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst) return SJ_E_INVALID;
    SJ_TRY(sim)
    const bool d64 = sim->precision == SJ_F64;
    const int nx = d64 ? sim->hi64[inst].nx : sim->hi32[inst].nx;
    const int ny = d64 ? sim->hi64[inst].ny : sim->hi32[inst].ny;
    const int nz = d64 ? sim->hi64[inst].nz : sim->hi32[inst].nz;
    const int px = d64 ? sim->hi64[inst].px : sim->hi32[inst].px;
    const std::vector<uint32_t>& keys = d64 ? sim->hi64[inst].keys : sim->hi32[inst].keys;
    const uint8_t* combo = d64 ? sim->h64[inst].combo : sim->h32[inst].combo;
    const size_t nv = (size_t)nx * ny * nz;
    if (3 * nv > cap) fail(SJ_E_RANGE, "output buffer too small for class map");
    std::vector<uint8_t> tmp(nv);
    ck(cudaStreamSynchronize(sim->stream), "sync");
    ck(cudaMemcpy2D(tmp.data(), nx, combo, px, nx, (size_t)ny * nz, cudaMemcpyDeviceToHost), "combo read");
    for (size_t q = 0; q < nv; ++q)
        for (int c = 0; c < 3; ++c) out[c * nv + q] = (uint8_t)((keys[tmp[q]] >> (8 * c)) & 255);
    SJ_CATCH(sim)
}

int sj_max_abs_e(sj_sim* sim, int32_t inst, double* out) {
    if (!sim || inst < 0 || inst >= sim->n_inst || !out) return SJ_E_INVALID;
    SJ_TRY(sim)
    if (sim->precision == SJ_F64)
        ck(launch_max_abs_e<double>(sim->h64[inst], sim->cur, sim->d_scratch, sim->stream), "max");
    else
        ck(launch_max_abs_e<float>(sim->h32[inst], sim->cur, sim->d_scratch, sim->stream), "max");
    ck(cudaMemcpyAsync(out, sim->d_scratch, sizeof(double), cudaMemcpyDeviceToHost, sim->stream), "max read");
    ck(cudaStreamSynchronize(sim->stream), "sync");
    SJ_CATCH(sim)
}

int sj_energy(sj_sim* sim, int32_t inst, double* out) {
    if (!sim || inst < 0 || inst >= sim->n_inst || !out) return SJ_E_INVALID;
    SJ_TRY(sim)
    const int np = energy_partials();
    double* part = (double*)sim->dalloc((size_t)(np + 1) * sizeof(double), false);
    cudaError_t e;
    if (sim->precision == SJ_F64) {
        const double dx = sim->hi64[inst].dx;
        e = launch_energy<double>(sim->h64[inst], sim->cur, 0.5 * dx * dx * dx, part, part + np, sim->stream);
    } else {
        const double dx = sim->hi32[inst].dx;
        e = launch_energy<float>(sim->h32[inst], sim->cur, 0.5 * dx * dx * dx, part, part + np, sim->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, part + np, sizeof(double), cudaMemcpyDeviceToHost, sim->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sim->stream);
    sim->dfree(part);
    ck(e, "energy");
    sim->d2h += (long long)sizeof(double);
    SJ_CATCH(sim)
}

int sj_flux(sj_sim* sim, int32_t inst, int32_t n_points, const int32_t* rows, double dA, double* out, size_t cap) {
    if (!sim || inst < 0 || inst >= sim->n_inst || n_points < 1 || !rows || !out) return SJ_E_INVALID;
    SJ_TRY(sim)
    const std::vector<int>& comp = sim->precision == SJ_F64 ? sim->hi64[inst].dft_comp : sim->hi32[inst].dft_comp;
    const int n_freq = sim->precision == SJ_F64 ? sim->hi64[inst].n_freq : sim->hi32[inst].n_freq;
    const double2* dft = sim->precision == SJ_F64 ? sim->h64[inst].dft : sim->h32[inst].dft;
    if (n_freq < 1 || comp.empty()) fail(SJ_E_INVALID, "the instance has no DFT probes or frequencies");
    if (cap < (size_t)n_freq) fail(SJ_E_RANGE, "output holds fewer than n_freqs values");
    // (E1, E2, H1, H2) must be the tangential components of one normal axis
    for (int p = 0; p < n_points; ++p) {
        int c[4];
        for (int m = 0; m < 4; ++m) {
            const int r = rows[4 * p + m];
            if (r < 0 || r >= (int)comp.size()) fail(SJ_E_RANGE, "DFT row out of range");
            c[m] = comp[r];
        }
        bool ok = false;
        for (int a = 0; a < 3; ++a) {
            const int t1 = (a + 1) % 3, t2 = (a + 2) % 3;
            ok |= c[0] == t1 && c[1] == t2 && c[2] == 3 + t1 && c[3] == 3 + t2;
        }
        if (!ok) fail(SJ_E_INVALID, "flux rows must be (E1, E2, H1, H2) tangential to one axis, in that order");
    }
    const size_t rb = (size_t)n_points * 4 * sizeof(int32_t);
    char* buf = (char*)sim->dalloc(rb + (size_t)n_freq * sizeof(double), false);
    cudaError_t e = cudaMemcpyAsync(buf, rows, rb, cudaMemcpyHostToDevice, sim->stream);
    double* d_out = reinterpret_cast<double*>(buf + rb);  // rb = 16 n_points: 8-byte aligned
    if (e == cudaSuccess)
        e = launch_flux(dft, n_freq, reinterpret_cast<const int*>(buf), n_points, dA, d_out, sim->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, (size_t)n_freq * sizeof(double), cudaMemcpyDeviceToHost, sim->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sim->stream);
    sim->dfree(buf);
    ck(e, "flux");
    sim->h2d += (long long)rb;
    sim->d2h += (long long)n_freq * (long long)sizeof(double);
    SJ_CATCH(sim)
}

int sj_rasterize(const sj_grid_desc* grid, const sj_scene_desc* scene, uint8_t* out) {
    if (!grid || !scene || !out) return finish(nullptr, SJ_E_INVALID, "NULL argument");
    try {
        if (grid->nx < 1 || grid->ny < 1 || grid->nz < 1 || !(grid->dx > 0))
            fail(SJ_E_INVALID, "bad grid");
        check_scene(scene);
        if (scene->smooth_n != 0)
            fail(SJ_E_INVALID, "a smoothed scene has fill counts, not region masks (sj_rasterize_counts)");
        sj_sim tmp;
        ck(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking), "stream");
        tmp.own_stream = true;
        sj_csg_node* d_nodes;
        int* d_start;
        upload_scene(&tmp, scene, &d_nodes, &d_start);
        const int nx = grid->nx, ny = grid->ny, nz = grid->nz;
        const long long nv = (long long)nx * ny * nz;
        uint8_t* d = (uint8_t*)tmp.dalloc(3 * nv);
        ck(launch_rasterize(d_nodes, d_start, scene->n_regions, nx, ny, nz, grid->dx, grid->origin, d, nv,
                            nx, tmp.stream),
           "rasterize");
        ck(cudaMemcpyAsync(out, d, 3 * nv, cudaMemcpyDeviceToHost, tmp.stream), "mask read");
        ck(cudaStreamSynchronize(tmp.stream), "sync");
    } catch (const Fail& f) {
        return finish(nullptr, f.code, f.msg);
    }
    return SJ_OK;
}

int sj_rasterize_counts(const sj_grid_desc* grid, const sj_scene_desc* scene, uint8_t* out) {
    if (!grid || !scene || !out) return finish(nullptr, SJ_E_INVALID, "NULL argument");
    try {
        if (grid->nx < 1 || grid->ny < 1 || grid->nz < 1 || !(grid->dx > 0))
            fail(SJ_E_INVALID, "bad grid");
        check_scene(scene);
        sj_sim tmp;
        ck(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking), "stream");
        tmp.own_stream = true;
        sj_csg_node* d_nodes;
        int* d_start;
        upload_scene(&tmp, scene, &d_nodes, &d_start);
        const int nx = grid->nx, ny = grid->ny, nz = grid->nz, R = scene->n_regions;
        const long long nv = (long long)nx * ny * nz;
        const std::vector<double> offs =
            scene->smooth_n > 0 ? smooth_points(scene->smooth_n, scene->smooth_rad) : std::vector<double>();
        double* d_offs = tmp.upload(offs);
        unsigned long long* d = (unsigned long long*)tmp.dalloc(3 * nv * sizeof(unsigned long long));
        ck(launch_rasterize_counts(d_nodes, d_start, R, nx, ny, nz, grid->dx, grid->origin, d_offs,
                                   (int)(offs.size() / 3), d, nv, nx, nullptr, 0, nullptr, tmp.stream),
           "rasterize counts");
        std::vector<unsigned long long> keys(3 * nv);
        ck(cudaMemcpyAsync(keys.data(), d, keys.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           tmp.stream),
           "count read");
        ck(cudaStreamSynchronize(tmp.stream), "sync");
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < R; ++r)
                for (long long q = 0; q < nv; ++q)
                    out[((long long)c * R + r) * nv + q] = (uint8_t)((keys[c * nv + q] >> (8 * r)) & 255);
    } catch (const Fail& f) {
        return finish(nullptr, f.code, f.msg);
    }
    return SJ_OK;
}

int sj_smooth_points(int32_t smooth_n, double smooth_rad, double* out, size_t cap) {
    if (!out) return finish(nullptr, SJ_E_INVALID, "NULL argument");
    if (smooth_n < 0 || smooth_n > SJ_MAX_SMOOTH_N) return finish(nullptr, SJ_E_INVALID, "smooth_n must be in [0, 31]");
    if (!(smooth_rad > 0) || !std::isfinite(smooth_rad))
        return finish(nullptr, SJ_E_INVALID, "smooth_rad must be finite and > 0");
    if ((size_t)24 * smooth_n > cap) return finish(nullptr, SJ_E_RANGE, "out holds fewer than 24 smooth_n doubles");
    const std::vector<double> p = smooth_points(smooth_n, smooth_rad);
    std::copy(p.begin(), p.end(), out);
    return SJ_OK;
}

int sj_rasterize_static(const sj_grid_desc* grid, const sj_scene_desc* scene, uint8_t* d_out_masks,
                        void* stream) {
    const char* msg = "";
    const int rc = rasterize_static(grid, scene, d_out_masks, static_cast<cudaStream_t>(stream), &msg);
    if (rc != SJ_OK) return finish(nullptr, rc, msg);
    return SJ_OK;
}

int sj_extract_phases(int32_t n_series, int32_t n_samples, const double* t_pts, const double* v,
                      double lowpass_inc, sj_phase_result* out) {
    if (n_series < 0 || (n_series > 0 && (!t_pts || !v || !out)))
        return finish(nullptr, SJ_E_INVALID, "NULL argument");
    if (n_samples < 8 || n_samples > 4096) return finish(nullptr, SJ_E_INVALID, "n_samples must be in [8, 4096]");
    if (!(lowpass_inc > 0)) return finish(nullptr, SJ_E_INVALID, "lowpass_inc must be > 0");
    if (!(t_pts[1] - t_pts[0] > 0)) return finish(nullptr, SJ_E_INVALID, "t_pts must increase");
    if (n_series == 0) return SJ_OK;
    // every region starts on a 16-double boundary (the workspace holds double2 arrays)
    auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
    const size_t nv = al((size_t)n_series * n_samples);
    const size_t nw = (size_t)n_series * (size_t)phase_workspace(n_samples);
    void* buf = nullptr;
    const size_t bytes = (nv + al(n_samples) + nw) * sizeof(double) + (size_t)n_series * sizeof(sj_phase_result);
    if (cudaMalloc(&buf, bytes) != cudaSuccess) return finish(nullptr, SJ_E_NOMEM, "cudaMalloc failed");
    double* d_v = static_cast<double*>(buf);
    double* d_t = d_v + nv;
    double* d_w = d_t + al(n_samples);
    sj_phase_result* d_out = reinterpret_cast<sj_phase_result*>(d_w + nw);
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_v, v, nv * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_t, t_pts, n_samples * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_phases(d_v, n_samples, 1, n_series, n_samples, d_t, lowpass_inc, d_w, d_out, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, (size_t)n_series * sizeof(sj_phase_result), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (s) cudaStreamDestroy(s);
    cudaFree(buf);
    if (e != cudaSuccess) return finish(nullptr, SJ_E_CUDA, std::string("phase extraction: ") + cudaGetErrorString(e));
    return SJ_OK;
}

int sj_extract_monitor_phases(sj_sim* sim, double lowpass_inc, sj_phase_result* out, size_t cap) {
    if (!sim || !out) return SJ_E_INVALID;
    if (!(lowpass_inc > 0)) return finish(sim, SJ_E_INVALID, "lowpass_inc must be > 0");
    SJ_TRY(sim)
    const int n = sim->n_inst;
    std::vector<int> nmon(n), span(n);
    std::vector<double> dt(n);
    std::vector<const double*> mon(n);
    for (int q = 0; q < n; ++q) {
        if (sim->precision == SJ_F64)
            nmon[q] = sim->hi64[q].n_mon, span[q] = sim->hi64[q].save_span, dt[q] = sim->hi64[q].dt,
            mon[q] = sim->h64[q].mon;
        else
            nmon[q] = sim->hi32[q].n_mon, span[q] = sim->hi32[q].save_span, dt[q] = sim->hi32[q].dt,
            mon[q] = sim->h32[q].mon;
    }
    size_t total = 0, wtotal = 0, ttotal = 0;
    std::vector<int> ns(n);
    for (int q = 0; q < n; ++q) {
        ns[q] = (int)((sim->t + span[q] - 1) / span[q]);
        if (nmon[q] == 0) continue;
        if (ns[q] < 8 || ns[q] > 4096) fail(SJ_E_RANGE, "each series needs 8 .. 4096 monitor samples");
        total += nmon[q];
        wtotal += (size_t)nmon[q] * (size_t)phase_workspace(ns[q]);
        ttotal += ns[q];
    }
    if (cap < total) fail(SJ_E_RANGE, "output holds fewer entries than the sim has monitors");
    if (total == 0) return SJ_OK;
    std::vector<double> ts;
    ts.reserve(ttotal);
    for (int q = 0; q < n; ++q)
        if (nmon[q])
            for (int k = 0; k < ns[q]; ++k) ts.push_back((double)k * (dt[q] * span[q]));
    const size_t tpad = (ttotal + 15) & ~(size_t)15;  // the workspace after it starts on a 16-double boundary
    char* buf = (char*)sim->dalloc((tpad + wtotal) * sizeof(double) + total * sizeof(sj_phase_result), false);
    double* d_t = reinterpret_cast<double*>(buf);
    double* d_w = d_t + tpad;
    sj_phase_result* d_out = reinterpret_cast<sj_phase_result*>(d_w + wtotal);
    cudaError_t e = cudaMemcpyAsync(d_t, ts.data(), ttotal * sizeof(double), cudaMemcpyHostToDevice, sim->stream);
    size_t so = 0, wo = 0, to = 0;
    for (int q = 0; q < n && e == cudaSuccess; ++q) {
        if (!nmon[q]) continue;
        // mon[sample][n_mon]: series stride 1, sample stride n_mon
        e = launch_phases(mon[q], 1, nmon[q], nmon[q], ns[q], d_t + to, lowpass_inc, d_w + wo, d_out + so,
                          sim->stream);
        so += nmon[q];
        wo += (size_t)nmon[q] * (size_t)phase_workspace(ns[q]);
        to += ns[q];
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, total * sizeof(sj_phase_result), cudaMemcpyDeviceToHost, sim->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sim->stream);
    sim->dfree(buf);
    ck(e, "phase extraction");
    sim->h2d += (long long)(ttotal * sizeof(double));
    sim->d2h += (long long)(total * sizeof(sj_phase_result));
    SJ_CATCH(sim)
}

int sj_source_dipole(const sj_source_desc* src, double t, double* re, double* im) {
    if (!src || !re || !im) return SJ_E_INVALID;
    const std::complex<double> v = dipole(*src, t);
    *re = v.real();
    *im = v.imag();
    return SJ_OK;
}

int sj_source_current(const sj_source_desc* src, double t, double dt, double* re, double* im) {
    if (!src || !re || !im || !(dt > 0)) return SJ_E_INVALID;
    const std::complex<double> v = current(*src, t, dt);
    *re = v.real();
    *im = v.imag();
    return SJ_OK;
}

double sj_source_last_time(const sj_source_desc* src) { return src ? last_time(*src) : NAN; }

}  // extern "C"
