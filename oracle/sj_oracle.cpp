/*
 * sj_oracle.cpp — TEST INFRASTRUCTURE ONLY.  The CPU oracle of the sim_juncs
 * GB300 stepper: a plain FP64 restatement, parallelised with OpenMP, that the
 * parity tests and the CPU baseline of bench.py run beside the CUDA library.
 * Nothing in the product (sim_juncs_gb300/) links, imports or calls it.
 *
 * What it restates, and from where:
 *   - the time loop of bound_geom::run (src/disp.cpp:690-749): monitors are
 *     sampled before step n when n % save_span == 0;
 *   - meep's fields::step() (meep v1.24, an external dependency absent here):
 *     the textbook Yee leapfrog with mu = 1, stretched-coordinate CPML
 *     auxiliaries on every face (meep::pml(thickness), src/disp.cpp:527;
 *     quadratic profile, R = 1e-15, meep's defaults), and meep's Lorentzian /
 *     Drude polarisation update (lorentzian_susceptibility, added per root and
 *     pole at src/disp.cpp:529-548);
 *   - cgs_material_function::in_bound (src/disp.cpp:264-283), over
 *     composite_object::in and the primitives' in() (src/cgs.cpp:34-120,
 *     403-449), evaluated in the reference's operation order, with the
 *     stochastic smoothing samples of generate_smooth_pts (src/disp.cpp:56-112)
 *     when the scene's smooth_n > 0;
 *   - gaussian_src_time_phase (src/disp.cpp:378-400) and the current
 *     (d(t) - d(t - dt)) / dt injected through add_volume_source
 *     (src/disp.cpp:614).
 * Parity against meep itself is unpinned: meep is not available to run.
 * The discretisation conventions are written out at the top of include/sj.h.
 *
 * Build: see oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).
 */
#include "../include/sj.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <omp.h>

namespace {

const double kOff[6][3] = {{0.5, 0, 0}, {0, 0.5, 0}, {0, 0, 0.5},
                           {0, 0.5, 0.5}, {0.5, 0, 0.5}, {0.5, 0.5, 0}};

std::string g_err;

// ---------------------------------------------------------------- sources
std::complex<double> dipole(const sj_source_desc& s, double t) {
    if (s.kind == SJ_SRC_GAUSSIAN) {
        // gaussian_src_time_phase constructor + dipole (src/disp.cpp:378-400)
        const double omega = 2 * M_PI * s.frequency;
        const double width = s.width;
        const double phi = s.phase + M_PI;
        const double peak = 0.5 * (s.start_time + s.end_time);
        double cutoff = (s.end_time - s.start_time) * 0.5;
        const std::complex<double> amp = 1.0 / std::complex<double>(0, -omega);
        while (exp(-cutoff * cutoff / (2 * width * width)) < 1e-100) cutoff *= 0.9;
        cutoff = float(cutoff);
        const double tt = t - peak;
        if (float(fabs(tt)) > cutoff) return 0.0;
        return exp(-tt * tt / (2 * width * width)) * std::polar(1.0, -omega * tt - phi) * amp;
    }
    const float rt = float(t);
    if (rt < s.start_time || rt > s.end_time) return 0.0;
    const std::complex<double> iw(0, -2 * M_PI * s.frequency);
    if (s.width == 0.0) return std::exp(iw * t) / iw;
    const double ts = (t - s.start_time) / s.width - 3.0;
    const double te = (s.end_time - t) / s.width - 3.0;
    return std::exp(iw * t) / iw * (1.0 + tanh(ts)) * (1.0 + tanh(te)) * 0.25;
}

// ---------------------------------------------------------------- CSG
void matvec(const double* m, double x, double y, double z, double& a, double& b, double& c) {
    // matrix::operator* (src/geometry.hpp:88-99): ret = 0; ret += m*v, left to right
    a = 0; a += m[0] * x; a += m[1] * y; a += m[2] * z;
    b = 0; b += m[3] * x; b += m[4] * y; b += m[5] * z;
    c = 0; c += m[6] * x; c += m[7] * y; c += m[8] * z;
}

int leaf_in(const sj_csg_node& nd, double x, double y, double z) {
    double rx, ry, rz;
    matvec(nd.m, x, y, z, rx, ry, rz);
    if (nd.op == SJ_CSG_PLANE) {
        // plane::in (src/cgs.cpp:92-99)
        const double d = rx * nd.p[0] + ry * nd.p[1] + rz * nd.p[2];
        return d > nd.p[3] ? 0 : 1;
    }
    double qx, qy, qz;
    matvec(nd.t, rx - nd.c[0], ry - nd.c[1], rz - nd.c[2], qx, qy, qz);
    if (nd.op == SJ_CSG_BOX) {  // box::in (src/cgs.cpp:52-70)
        if (fabs(qx) > nd.p[0]) return nd.invert;
        if (fabs(qy) > nd.p[1]) return nd.invert;
        if (fabs(qz) > nd.p[2]) return nd.invert;
        return 1 - nd.invert;
    }
    if (nd.op == SJ_CSG_SPHERE) {  // sphere::in (src/cgs.cpp:34-39)
        double s2 = 0;
        s2 += qx * qx;
        s2 += qy * qy;
        s2 += qz * qz;
        return sqrt(s2) > nd.p[0] ? nd.invert : 1 - nd.invert;
    }
    // cylinder::in (src/cgs.cpp:110-120)
    const double h = nd.p[0], r1 = nd.p[1], r2 = nd.p[2];
    if (qz < 0 || qz > h) return nd.invert;
    const double cr = qx * qx + qy * qy;
    if (cr * h > (r2 - r1) * qz + r1 * h) return nd.invert;
    return 1 - nd.invert;
}

int program_in(const sj_csg_node* nodes, int n, double x, double y, double z) {
    std::vector<int> stk;
    stk.reserve(16);
    for (int q = 0; q < n; ++q) {
        const sj_csg_node& nd = nodes[q];
        if (nd.op <= SJ_CSG_PLANE) {
            stk.push_back(leaf_in(nd, x, y, z));
        } else if (nd.op == SJ_CSG_UNION || nd.op == SJ_CSG_INTERSECT) {
            const int b = stk.back();
            stk.pop_back();
            const int a = stk.back();
            stk.pop_back();
            stk.push_back(nd.invert ^ (nd.op == SJ_CSG_UNION ? (a | b) : (a & b)));
        } else if (nd.op == SJ_CSG_PASS) {
            stk.back() = nd.invert ^ stk.back();
        } else if (nd.op == SJ_CSG_CONST) {
            stk.push_back(nd.invert & 1);
        } else {
            stk.push_back(0);
        }
    }
    return stk.empty() ? 0 : stk.back();
}

// generate_smooth_pts (src/disp.cpp:56-112) as the cgs_material_function
// constructors call it, seed DEF_SEED (src/disp.hpp:34: the double
// 0xd9a28bf3, converted to uint64_t); the seed_seq words are seed & 0xffff
// and (seed & 0xffff0000) >> 32, which is 0.  Returns the 8 n reflected
// offsets, 3 doubles each.
std::vector<double> smooth_offsets(int n, double rad) {
    const unsigned long long seed = 0xd9a28bf3ull;
    std::seed_seq seq{(unsigned)(seed & 0xffffull), (unsigned)((seed & 0xffff0000ull) >> 32)};
    std::mt19937 eng(seq);
    std::normal_distribution<double> gauss(0.0, rad);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    std::vector<double> pts;
    for (int q = 0; q < n; ++q) {
        const double ti = uni(eng);                       // theta_inv
        const double cth = 1 - 2 * ti;
        const double sth = 2 * sqrt(ti * (1 - ti));
        const double ph = 2 * M_PI * uni(eng);
        const double rr = gauss(eng);
        const double v[3] = {rr * sth * cos(ph), rr * sth * cos(ph), rr * cth};  // y as written there
        for (int a = 0; a < 8; ++a) {                     // signs: x outermost, z innermost
            pts.push_back((a & 4) ? v[0] : -v[0]);
            pts.push_back((a & 2) ? v[1] : -v[1]);
            pts.push_back((a & 1) ? v[2] : -v[2]);
        }
    }
    return pts;
}

// in_bound's this_ret of each region at (x, y, z), 8 bits per region
unsigned long long point_counts(const sj_scene_desc* sc, const std::vector<double>& offs, double x, double y,
                                double z) {
    unsigned long long key = 0;
    const size_t n = offs.size() / 3;
    for (int r = 0; r < sc->n_regions; ++r) {
        const sj_region_desc& rg = sc->regions[r];
        unsigned cnt = (unsigned)program_in(rg.nodes, rg.n_nodes, x, y, z);
        for (size_t q = 0; q < n; ++q)
            cnt += (unsigned)program_in(rg.nodes, rg.n_nodes, x + offs[3 * q], y + offs[3 * q + 1], z + offs[3 * q + 2]);
        key |= (unsigned long long)cnt << (8 * r);
    }
    return key;
}

std::vector<double> scene_offsets(const sj_scene_desc* sc) {
    if (sc->smooth_n < 0 || sc->smooth_n > SJ_MAX_SMOOTH_N) throw std::string("bad smooth_n");
    if (sc->smooth_n == 0) return {};
    if (!(sc->smooth_rad > 0)) throw std::string("bad smooth_rad");
    return smooth_offsets(sc->smooth_n, sc->smooth_rad);
}

// ---------------------------------------------------------------- oracle state
struct Src {
    sj_source_desc d;
    int lo[3], n[3];
    std::vector<double> w[3];
};

struct Probe {
    int comp, mon, dft;
    long long idx[8];
    double w[8];
};

}  // namespace

struct sjo_sim {
    int nx, ny, nz;
    long long N;
    double dx, dt, S;
    int save_span;
    long long t = 0;
    std::vector<double> F[6];
    // materials: class index per E component and class tables
    std::vector<uint8_t> cls[3];
    std::vector<double> inv_eps;      // [class]
    int np = 0;
    std::vector<double> A, B, C;      // per pole
    std::vector<double> csig;         // [class][pole] = C_p * sigma
    std::vector<std::vector<double>> P, Pm;  // [pole*3+comp][N]
    // CPML
    std::vector<double> bi[3], ci[3], bh[3], ch[3];
    std::vector<char> oni[3], onh[3];
    std::vector<double> psiE[3][2], psiH[3][2];  // [axis][slot][N]
    std::vector<Src> src;
    std::vector<Probe> probes;
    std::vector<double> freqs;
    int n_mon = 0, n_dft = 0;
    std::vector<std::vector<double>> mon;        // [monitor][samples]
    std::vector<std::complex<double>> dft;       // [dft][freq]
    // design region: per-voxel inverse eps at the voxel's E points
    int des_lo[3] = {0, 0, 0}, des_n[3] = {0, 0, 0};
    std::vector<double> des_inv;                 // [n2][n1][n0]
    double* rec_acc = nullptr;                   // when set: acc of the E update at design points [d][3]

    long long des_index(int i, int j, int k) const {
        const int u = i - des_lo[0], v = j - des_lo[1], w = k - des_lo[2];
        if (des_inv.empty() || u < 0 || v < 0 || w < 0 || u >= des_n[0] || v >= des_n[1] || w >= des_n[2]) return -1;
        return ((long long)w * des_n[1] + v) * des_n[0] + u;
    }

    long long at(int i, int j, int k) const { return ((long long)k * ny + j) * nx + i; }
};

namespace {

void build(sjo_sim* s, const sj_instance_desc& d) {
    const sj_grid_desc& g = d.grid;
    if (g.nx < 1 || g.ny < 1 || g.nz < 1 || !(g.dx > 0)) throw std::string("bad grid");
    s->nx = g.nx, s->ny = g.ny, s->nz = g.nz;
    s->N = (long long)g.nx * g.ny * g.nz;
    s->dx = g.dx;
    s->dt = g.dt > 0 ? g.dt : 0.5 * g.dx;
    s->S = s->dt / s->dx;
    s->save_span = d.save_span > 0 ? d.save_span : 1;
    for (int c = 0; c < 6; ++c) s->F[c].assign(s->N, 0.0);

    // ---- materials
    const sj_material_desc& m = d.material;
    std::vector<double> eps;
    std::vector<sj_pole> poles;
    std::vector<double> sigma;
    int ncls;
    for (int c = 0; c < 3; ++c) s->cls[c].assign(s->N, 0);
    if (m.class_map) {
        ncls = m.n_classes;
        eps.assign(m.eps_inf, m.eps_inf + ncls);
        poles.assign(m.poles, m.poles + m.n_poles);
        sigma.assign(m.sigma, m.sigma + (size_t)ncls * m.n_poles);
        for (int c = 0; c < 3; ++c)
            for (long long q = 0; q < s->N; ++q) s->cls[c][q] = m.class_map[c * s->N + q];
    } else {
        const sj_scene_desc* sc = m.scene;
        if (!sc) throw std::string("no material");
        const int R = sc->n_regions;
        ncls = 1 << R;
        std::vector<std::pair<int, double>> owner;
        for (int r = 0; r < R; ++r)
            for (int q = 0; q < sc->regions[r].n_poles; ++q) {
                poles.push_back(sc->regions[r].poles[q]);
                owner.push_back({r, sc->regions[r].sigma[q]});
            }
        const std::vector<double> offs = scene_offsets(sc);
        if (!offs.empty()) {
            // smoothed: class = the point's tuple of counts (sorted distinct tuples)
            if (sc->combine != SJ_EPS_SUM) throw std::string("smoothing needs SJ_EPS_SUM");
            std::vector<unsigned long long> keys(3 * s->N);
#pragma omp parallel for schedule(dynamic)
            for (int k = 0; k < s->nz; ++k)
                for (int j = 0; j < s->ny; ++j)
                    for (int i = 0; i < s->nx; ++i)
                        for (int c = 0; c < 3; ++c) {
                            const double x = g.origin[0] + ((double)i + (c == 0 ? 0.5 : 0.0)) * g.dx;
                            const double y = g.origin[1] + ((double)j + (c == 1 ? 0.5 : 0.0)) * g.dx;
                            const double z = g.origin[2] + ((double)k + (c == 2 ? 0.5 : 0.0)) * g.dx;
                            keys[c * s->N + s->at(i, j, k)] = point_counts(sc, offs, x, y, z);
                        }
            std::vector<unsigned long long> uniq(keys);
            std::sort(uniq.begin(), uniq.end());
            uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
            if (uniq.size() > 256) throw std::string("more than 256 smoothed point classes");
            ncls = (int)uniq.size();
            for (int c = 0; c < 3; ++c)
                for (long long q = 0; q < s->N; ++q)
                    s->cls[c][q] = (uint8_t)(std::lower_bound(uniq.begin(), uniq.end(), keys[c * s->N + q]) - uniq.begin());
            const double n1 = (double)(offs.size() / 3 + 1);   // smooth_n + 1 after the x8
            eps.assign(ncls, 0.0);
            sigma.assign((size_t)ncls * poles.size(), 0.0);
            for (int mm = 0; mm < ncls; ++mm) {
                double ret = 0;
                for (int r = 0; r < R; ++r)
                    ret += sc->ambient_eps + (sc->regions[r].eps - sc->ambient_eps) * (double)((uniq[mm] >> (8 * r)) & 255) / n1;
                eps[mm] = R == 0 ? sc->ambient_eps : ret;
                for (size_t p = 0; p < poles.size(); ++p)
                    sigma[(size_t)mm * poles.size() + p] =
                        0.0 + (owner[p].second - 0.0) * (double)((uniq[mm] >> (8 * owner[p].first)) & 255) / n1;
            }
        } else {
        eps.assign(ncls, 0.0);
        sigma.assign((size_t)ncls * poles.size(), 0.0);
        for (int mm = 0; mm < ncls; ++mm) {
            int first = -1;
            for (int r = R - 1; r >= 0; --r)
                if ((mm >> r) & 1) first = r;
            if (sc->combine == SJ_EPS_FIRST) {
                // the first root containing the point decides
                eps[mm] = first >= 0 ? sc->regions[first].eps : sc->ambient_eps;
            } else if (R == 0) {
                eps[mm] = sc->ambient_eps;
            } else {
                // in_bound (src/disp.cpp:264-283), smooth_n = 0
                double ret = 0;
                for (int r = 0; r < R; ++r)
                    ret += sc->ambient_eps + (sc->regions[r].eps - sc->ambient_eps) * (double)((mm >> r) & 1) / 1.0;
                eps[mm] = ret;
            }
            for (size_t p = 0; p < poles.size(); ++p) {
                double in = (double)((mm >> owner[p].first) & 1);
                if (sc->combine == SJ_EPS_FIRST && owner[p].first != first) in = 0.0;
                sigma[(size_t)mm * poles.size() + p] = 0.0 + (owner[p].second - 0.0) * in / 1.0;
            }
        }
#pragma omp parallel for schedule(static)
        for (int k = 0; k < s->nz; ++k)
            for (int j = 0; j < s->ny; ++j)
                for (int i = 0; i < s->nx; ++i)
                    for (int c = 0; c < 3; ++c) {
                        const double x = g.origin[0] + ((double)i + (c == 0 ? 0.5 : 0.0)) * g.dx;
                        const double y = g.origin[1] + ((double)j + (c == 1 ? 0.5 : 0.0)) * g.dx;
                        const double z = g.origin[2] + ((double)k + (c == 2 ? 0.5 : 0.0)) * g.dx;
                        unsigned mask = 0;
                        for (int r = 0; r < R; ++r) {
                            const sj_region_desc& rg = sc->regions[r];
                            if (program_in(rg.nodes, rg.n_nodes, x, y, z)) mask |= 1u << r;
                        }
                        s->cls[c][s->at(i, j, k)] = (uint8_t)mask;
                    }
        }
    }
    s->inv_eps.resize(ncls);
    for (int c = 0; c < ncls; ++c) s->inv_eps[c] = 1.0 / eps[c];
    s->np = (int)poles.size();
    s->A.resize(s->np), s->B.resize(s->np), s->C.resize(s->np);
    for (int p = 0; p < s->np; ++p) {
        // lorentzian_susceptibility::update_P in meep's frequency units (2 pi)
        const double w = 2 * M_PI * poles[p].omega_0, gm = 2 * M_PI * poles[p].gamma, dt = s->dt;
        const double den = 1 + gm * dt / 2;
        s->A[p] = (2 - w * w * dt * dt * (poles[p].drude ? 0.0 : 1.0)) / den;
        s->B[p] = -(1 - gm * dt / 2) / den;
        s->C[p] = w * w * dt * dt / den;
    }
    s->csig.assign((size_t)ncls * s->np, 0.0);
    for (int c = 0; c < ncls; ++c)
        for (int p = 0; p < s->np; ++p) s->csig[(size_t)c * s->np + p] = s->C[p] * sigma[(size_t)c * s->np + p];
    s->P.assign(3 * s->np, std::vector<double>(s->N, 0.0));
    s->Pm.assign(3 * s->np, std::vector<double>(s->N, 0.0));

    // ---- CPML
    const double R = d.pml.r_asymptotic > 0 ? d.pml.r_asymptotic : 1e-15;
    const double pw = d.pml.power > 0 ? d.pml.power : 2.0;
    for (int a = 0; a < 3; ++a) {
        const int n = a == 0 ? s->nx : (a == 1 ? s->ny : s->nz);
        const double o = g.origin[a], L = n * s->dx;
        const double dlo = d.pml.thickness[a][0], dhi = d.pml.thickness[a][1];
        s->bi[a].assign(n, 1.0), s->ci[a].assign(n, 0.0), s->bh[a].assign(n, 1.0), s->ch[a].assign(n, 0.0);
        s->oni[a].assign(n, 0), s->onh[a].assign(n, 0);
        for (int i = 0; i < n; ++i)
            for (int h = 0; h < 2; ++h) {
                const double q = o + (i + 0.5 * h) * s->dx;
                double sg = 0;
                if (dlo > 0 && q < o + dlo) sg += -(pw + 1) * log(R) / (2 * dlo) * pow((o + dlo - q) / dlo, pw);
                if (dhi > 0 && q > o + L - dhi) sg += -(pw + 1) * log(R) / (2 * dhi) * pow((q - (o + L - dhi)) / dhi, pw);
                const double b = exp(-(sg + d.pml.alpha) * s->dt);
                const double c = sg > 0 ? sg / (sg + d.pml.alpha) * (b - 1) : 0.0;
                (h ? s->bh : s->bi)[a][i] = b;
                (h ? s->ch : s->ci)[a][i] = c;
                if (sg > 0) (h ? s->onh : s->oni)[a][i] = 1;
            }
        for (int q = 0; q < 2; ++q) {
            s->psiE[a][q].assign(s->N, 0.0);
            s->psiH[a][q].assign(s->N, 0.0);
        }
    }

    // ---- sources
    s->src.clear();
    for (int q = 0; q < d.n_sources; ++q) {
        Src sv;
        sv.d = d.sources[q];
        const int comp = sv.d.component;
        for (int a = 0; a < 3; ++a) {
            const int n = a == 0 ? s->nx : (a == 1 ? s->ny : s->nz);
            const double lo = std::min(sv.d.lo[a], sv.d.hi[a]), hi = std::max(sv.d.lo[a], sv.d.hi[a]);
            std::vector<double> w(n, 0.0);
            if (hi - lo <= 1e-9 * s->dx) {
                const double u = (lo - g.origin[a]) / s->dx - kOff[comp][a];
                const double i0 = floor(u), f = u - i0;
                const long long a0 = (long long)i0;
                if (a0 >= 0 && a0 < n) w[a0] += (1 - f) / s->dx;
                if (a0 + 1 >= 0 && a0 + 1 < n) w[a0 + 1] += f / s->dx;
            } else {
                for (int i = 0; i < n; ++i) {
                    const double q2 = g.origin[a] + (i + kOff[comp][a]) * s->dx;
                    const double ov = std::min(hi, q2 + 0.5 * s->dx) - std::max(lo, q2 - 0.5 * s->dx);
                    if (ov > 0) w[i] = ov / s->dx;
                }
            }
            sv.w[a] = w;
            sv.lo[a] = 0;
            sv.n[a] = n;
        }
        s->src.push_back(sv);
    }

    // ---- probes
    s->probes.clear();
    s->n_mon = s->n_dft = 0;
    for (int p = 0; p < d.n_probes; ++p) {
        const sj_probe_desc& pd = d.probes[p];
        Probe pr;
        pr.comp = pd.component;
        pr.mon = (pd.flags & SJ_PROBE_MONITOR) ? s->n_mon++ : -1;
        pr.dft = (pd.flags & SJ_PROBE_DFT) ? s->n_dft++ : -1;
        long long i0[3];
        double f[3];
        for (int a = 0; a < 3; ++a) {
            const double u = (pd.pos[a] - g.origin[a]) / s->dx - kOff[pd.component][a];
            const double fl = floor(u);
            i0[a] = (long long)fl;
            f[a] = u - fl;
        }
        for (int m8 = 0; m8 < 8; ++m8) {
            const int di = m8 & 1, dj = (m8 >> 1) & 1, dk = (m8 >> 2) & 1;
            const long long ii = i0[0] + di, jj = i0[1] + dj, kk = i0[2] + dk;
            const double w = (di ? f[0] : 1 - f[0]) * (dj ? f[1] : 1 - f[1]) * (dk ? f[2] : 1 - f[2]);
            pr.idx[m8] = -1;
            pr.w[m8] = 0;
            if (ii >= 0 && ii < s->nx && jj >= 0 && jj < s->ny && kk >= 0 && kk < s->nz) {
                pr.idx[m8] = (kk * s->ny + jj) * s->nx + ii;
                pr.w[m8] = w;
            }
        }
        s->probes.push_back(pr);
    }
    s->freqs.assign(d.freqs, d.freqs + d.n_freqs);
    s->mon.assign(s->n_mon, std::vector<double>());
    s->dft.assign((size_t)s->n_dft * s->freqs.size(), 0.0);
}

double src_sum(const sjo_sim* s, int comp, int i, int j, int k, const std::vector<double>& tabs, double acc) {
    for (size_t q = 0; q < s->src.size(); ++q) {
        const Src& sv = s->src[q];
        if (sv.d.component != comp) continue;
        if (sv.w[0][i] != 0 && sv.w[1][j] != 0 && sv.w[2][k] != 0)
            acc -= tabs[q] * sv.w[0][i] * sv.w[1][j] * sv.w[2][k];
    }
    return acc;
}

// One step n -> n+1 (formulas at the top of include/sj.h).
void step_once(sjo_sim* s) {
    const long long n = s->t;
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const double S = s->S, dt = s->dt;
    // probes before the step
    for (const Probe& pr : s->probes) {
        double v = 0;
        for (int m8 = 0; m8 < 8; ++m8)
            if (pr.idx[m8] >= 0) v += pr.w[m8] * s->F[pr.comp][pr.idx[m8]];
        if (pr.mon >= 0 && n % s->save_span == 0) s->mon[pr.mon].push_back(v);
        if (pr.dft >= 0) {
            const double tt = pr.comp < 3 ? (double)n * dt : ((double)n - 0.5) * dt;
            for (size_t f = 0; f < s->freqs.size(); ++f) {
                const double ph = 2 * M_PI * s->freqs[f] * tt;
                s->dft[(size_t)pr.dft * s->freqs.size() + f] += std::complex<double>(v * cos(ph) * dt, v * sin(ph) * dt);
            }
        }
    }
    // per-source dt * J at this step
    std::vector<double> tabE(s->src.size()), tabH(s->src.size());
    for (size_t q = 0; q < s->src.size(); ++q) {
        const sj_source_desc& sd = s->src[q].d;
        const double half = sd.component < 3 ? 0.5 : 0.0;
        const double tt = ((double)n + half) * dt;
        const std::complex<double> a(sd.amplitude[0], sd.amplitude[1]);
        const std::complex<double> cur = (dipole(sd, tt) - dipole(sd, tt - dt)) / dt;
        tabE[q] = tabH[q] = dt * std::real(a * cur);
    }
    std::vector<double>* F = s->F;
    auto E = [&](int c, int i, int j, int k) -> double {
        return (i < nx && j < ny && k < nz) ? F[c][s->at(i, j, k)] : 0.0;
    };
    auto Hm = [&](int c, int i, int j, int k) -> double {
        return (i >= 0 && j >= 0 && k >= 0) ? F[3 + c][s->at(i, j, k)] : 0.0;
    };
    // H^{n+1/2}
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long long o = s->at(i, j, k);
                const int idx[3] = {i, j, k};
                for (int ca = 0; ca < 3; ++ca) {
                    const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
                    int p1[3] = {i, j, k}, p2[3] = {i, j, k};
                    p1[a1] += 1;
                    p2[a2] += 1;
                    const double d1 = E(a2, p1[0], p1[1], p1[2]) - E(a2, i, j, k);
                    const double d2 = E(a1, p2[0], p2[1], p2[2]) - E(a1, i, j, k);
                    double cur = d1 - d2;
                    const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
                    if (s->onh[a1][idx[a1]]) {
                        double& psi = s->psiH[a1][s1][o];
                        psi = s->bh[a1][idx[a1]] * psi + s->ch[a1][idx[a1]] * d1;
                        cur += psi;
                    }
                    if (s->onh[a2][idx[a2]]) {
                        double& psi = s->psiH[a2][s2][o];
                        psi = s->bh[a2][idx[a2]] * psi + s->ch[a2][idx[a2]] * d2;
                        cur -= psi;
                    }
                    double acc = -(S * cur);
                    acc = src_sum(s, 3 + ca, i, j, k, tabH, acc);
                    F[3 + ca][o] = F[3 + ca][o] + acc;
                }
            }
    // E^{n+1}
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long long o = s->at(i, j, k);
                const int idx[3] = {i, j, k};
                for (int ca = 0; ca < 3; ++ca) {
                    const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
                    int p1[3] = {i, j, k}, p2[3] = {i, j, k};
                    p1[a1] -= 1;
                    p2[a2] -= 1;
                    const double d1 = Hm(a2, i, j, k) - Hm(a2, p1[0], p1[1], p1[2]);
                    const double d2 = Hm(a1, i, j, k) - Hm(a1, p2[0], p2[1], p2[2]);
                    double cur = d1 - d2;
                    const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
                    if (s->oni[a1][idx[a1]]) {
                        double& psi = s->psiE[a1][s1][o];
                        psi = s->bi[a1][idx[a1]] * psi + s->ci[a1][idx[a1]] * d1;
                        cur += psi;
                    }
                    if (s->oni[a2][idx[a2]]) {
                        double& psi = s->psiE[a2][s2][o];
                        psi = s->bi[a2][idx[a2]] * psi + s->ci[a2][idx[a2]] * d2;
                        cur -= psi;
                    }
                    double acc = S * cur;
                    acc = src_sum(s, ca, i, j, k, tabE, acc);
                    const int cl = s->cls[ca][o];
                    const double eo = F[ca][o];
                    for (int p = 0; p < s->np; ++p) {
                        const double cs = s->csig[(size_t)cl * s->np + p];
                        double& pp = s->P[3 * p + ca][o];
                        double& pm = s->Pm[3 * p + ca][o];
                        if (cs == 0.0 && pp == 0.0 && pm == 0.0) continue;
                        const double pn = pp, pq = pm;
                        const double pnew = s->A[p] * pn + s->B[p] * pq + cs * eo;
                        acc -= (pnew - pn);
                        pm = pn;
                        pp = pnew;
                    }
                    const long long dd = s->des_index(i, j, k);
                    if (dd >= 0 && s->rec_acc) s->rec_acc[dd * 3 + ca] = acc;
                    F[ca][o] = eo + (dd >= 0 ? s->des_inv[dd] : s->inv_eps[cl]) * acc;
                }
            }
    s->t += 1;
}

// Zero fields, auxiliaries, polarisations, monitors and DFTs; t = 0.
void reset_state(sjo_sim* s) {
    for (int c = 0; c < 6; ++c) std::fill(s->F[c].begin(), s->F[c].end(), 0.0);
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 2; ++q) {
            std::fill(s->psiE[a][q].begin(), s->psiE[a][q].end(), 0.0);
            std::fill(s->psiH[a][q].begin(), s->psiH[a][q].end(), 0.0);
        }
    for (auto& v : s->P) std::fill(v.begin(), v.end(), 0.0);
    for (auto& v : s->Pm) std::fill(v.begin(), v.end(), 0.0);
    for (auto& m : s->mon) m.clear();
    std::fill(s->dft.begin(), s->dft.end(), std::complex<double>(0.0, 0.0));
    s->t = 0;
}

// Objective DFT: D[cell][c] += dt E_c^n(cell) e^{i 2 pi f n dt} for the E
// components in the mask, sampled before step n.
void objective_sample(const sjo_sim* s, const sj_objective_desc& ob, long long n,
                      std::vector<std::complex<double>>& D) {
    const double th = 2 * M_PI * ob.frequency * (double)n * s->dt;
    const std::complex<double> w(cos(th) * s->dt, sin(th) * s->dt);
    for (int q = 0; q < ob.n_cells; ++q) {
        const int* c3 = ob.cells + 3 * q;
        const long long o = s->at(c3[0], c3[1], c3[2]);
        for (int c = 0; c < 3; ++c)
            if ((ob.comp_mask >> c) & 1) D[3 * q + c] += s->F[c][o] * w;
    }
}

// Forward run of n_steps from rest; returns F and, when acc is given, the
// E-update acc at the design points per step ([n][d][3]).
double objective_forward(sjo_sim* s, const sj_objective_desc& ob, long long n_steps, double* acc,
                         std::vector<std::complex<double>>& D) {
    reset_state(s);
    D.assign((size_t)3 * ob.n_cells, std::complex<double>(0.0, 0.0));
    const long long nd = (long long)s->des_inv.size();
    for (long long n = 0; n < n_steps; ++n) {
        objective_sample(s, ob, n, D);
        s->rec_acc = acc ? acc + (size_t)n * nd * 3 : nullptr;
        step_once(s);
    }
    s->rec_acc = nullptr;
    double F = 0;
    for (const auto& d : D) F += std::norm(d);
    return F;
}

// The discrete adjoint: for n = N-1 .. 0, the transpose of the E update
// (polarisation ADE, E-side psi, curl of H) and then of the H update
// (H-side psi, curl of E), plus dF/dE^n from the objective DFT.  Returns
// dF/d(inverse eps) at the design points ([d][3]).  Gather form: each
// cell collects the contributions of its neighbours from per-cell arrays.
void adjoint_sweep(sjo_sim* s, const sj_objective_desc& ob, long long n_steps, const double* acc,
                   const std::vector<std::complex<double>>& D, std::vector<double>& g) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const long long N = s->N;
    const double S = s->S, dt = s->dt;
    const long long nd = (long long)s->des_inv.size();
    std::vector<double> eb[3], hb[3], d1[3], d2[3], psEb[3][2], psHb[3][2];
    for (int c = 0; c < 3; ++c) {
        eb[c].assign(N, 0.0), hb[c].assign(N, 0.0), d1[c].assign(N, 0.0), d2[c].assign(N, 0.0);
        for (int q = 0; q < 2; ++q) psEb[c][q].assign(N, 0.0), psHb[c][q].assign(N, 0.0);
    }
    std::vector<std::vector<double>> pb(3 * s->np, std::vector<double>(N, 0.0)), pmb = pb;
    g.assign((size_t)nd * 3, 0.0);
    const int nn[3] = {nx, ny, nz};
    for (long long n = n_steps - 1; n >= 0; --n) {
        const double* accn = acc + (size_t)n * nd * 3;
        // ---- transpose of the E update: eb holds dF/dE^{n+1}
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const long long o = s->at(i, j, k);
                    const int idx[3] = {i, j, k};
                    const long long dd = s->des_index(i, j, k);
                    for (int ca = 0; ca < 3; ++ca) {
                        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
                        const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
                        const int cl = s->cls[ca][o];
                        const double inv = dd >= 0 ? s->des_inv[dd] : s->inv_eps[cl];
                        const double ebo = eb[ca][o];
                        if (dd >= 0) g[dd * 3 + ca] += ebo * accn[dd * 3 + ca];
                        const double ab = inv * ebo;
                        double ein = ebo;
                        for (int p = 0; p < s->np; ++p) {
                            const double cs = s->csig[(size_t)cl * s->np + p];
                            if (cs == 0.0) continue;  // P is never excited there and does not reach E
                            const double pnb = pb[3 * p + ca][o] - ab;
                            const double pnbar = pmb[3 * p + ca][o] + ab + s->A[p] * pnb;
                            pmb[3 * p + ca][o] = s->B[p] * pnb;
                            pb[3 * p + ca][o] = pnbar;
                            ein += cs * pnb;
                        }
                        eb[ca][o] = ein;
                        const double cb = S * ab;
                        double t1 = cb, t2 = -cb;
                        if (s->oni[a1][idx[a1]]) {
                            const double t = psEb[a1][s1][o] + cb;
                            t1 = cb + s->ci[a1][idx[a1]] * t;
                            psEb[a1][s1][o] = s->bi[a1][idx[a1]] * t;
                        }
                        if (s->oni[a2][idx[a2]]) {
                            const double t = psEb[a2][s2][o] - cb;
                            t2 = -cb + s->ci[a2][idx[a2]] * t;
                            psEb[a2][s2][o] = s->bi[a2][idx[a2]] * t;
                        }
                        d1[ca][o] = t1;  // adjoint of d1 = H_a2(o) - H_a2(o - e_a1)
                        d2[ca][o] = t2;  // adjoint of d2 = H_a1(o) - H_a1(o - e_a2)
                    }
                }
        // gather into hb (dF/dH^{n+1/2} = from the future + from this E update)
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const long long o = s->at(i, j, k);
                    const int idx[3] = {i, j, k};
                    for (int ca = 0; ca < 3; ++ca) {
                        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
                        // d1 of E_ca reads H_a2 at o and o - e_a1
                        double v = d1[ca][o];
                        if (idx[a1] + 1 < nn[a1]) {
                            int q[3] = {i, j, k};
                            q[a1] += 1;
                            v -= d1[ca][s->at(q[0], q[1], q[2])];
                        }
                        hb[a2][o] += v;
                        // d2 of E_ca reads H_a1 at o and o - e_a2
                        double w = d2[ca][o];
                        if (idx[a2] + 1 < nn[a2]) {
                            int q[3] = {i, j, k};
                            q[a2] += 1;
                            w -= d2[ca][s->at(q[0], q[1], q[2])];
                        }
                        hb[a1][o] += w;
                    }
                }
        // ---- transpose of the H update: hb holds dF/dH^{n+1/2}; it carries
        // over unchanged to H^{n-1/2}
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const long long o = s->at(i, j, k);
                    const int idx[3] = {i, j, k};
                    for (int ca = 0; ca < 3; ++ca) {
                        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
                        const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
                        const double cb = -S * hb[ca][o];
                        double t1 = cb, t2 = -cb;
                        if (s->onh[a1][idx[a1]]) {
                            const double t = psHb[a1][s1][o] + cb;
                            t1 = cb + s->ch[a1][idx[a1]] * t;
                            psHb[a1][s1][o] = s->bh[a1][idx[a1]] * t;
                        }
                        if (s->onh[a2][idx[a2]]) {
                            const double t = psHb[a2][s2][o] - cb;
                            t2 = -cb + s->ch[a2][idx[a2]] * t;
                            psHb[a2][s2][o] = s->bh[a2][idx[a2]] * t;
                        }
                        d1[ca][o] = t1;  // adjoint of d1 = E_a2(o + e_a1) - E_a2(o)
                        d2[ca][o] = t2;  // adjoint of d2 = E_a1(o + e_a2) - E_a1(o)
                    }
                }
        // gather into eb
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const long long o = s->at(i, j, k);
                    const int idx[3] = {i, j, k};
                    for (int ca = 0; ca < 3; ++ca) {
                        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
                        // H_ca's d1 reads E_a2 at o + e_a1 and o
                        double v = -d1[ca][o];
                        if (idx[a1] > 0) {
                            int q[3] = {i, j, k};
                            q[a1] -= 1;
                            v += d1[ca][s->at(q[0], q[1], q[2])];
                        }
                        eb[a2][o] += v;
                        // H_ca's d2 reads E_a1 at o + e_a2 and o
                        double w = -d2[ca][o];
                        if (idx[a2] > 0) {
                            int q[3] = {i, j, k};
                            q[a2] -= 1;
                            w += d2[ca][s->at(q[0], q[1], q[2])];
                        }
                        eb[a1][o] += w;
                    }
                }
        // ---- dF/dE^n of the objective DFT
        const double th = 2 * M_PI * ob.frequency * (double)n * dt;
        const double cth = cos(th), sth = sin(th);
        for (int q = 0; q < ob.n_cells; ++q) {
            const int* c3 = ob.cells + 3 * q;
            const long long o = s->at(c3[0], c3[1], c3[2]);
            for (int c = 0; c < 3; ++c)
                if ((ob.comp_mask >> c) & 1) {
                    const std::complex<double>& d = D[3 * q + c];
                    eb[c][o] += 2 * dt * (d.real() * cth + d.imag() * sth);
                }
        }
    }
}

}  // namespace

extern "C" {

const char* sjo_last_error(void) { return g_err.c_str(); }
// OpenMP threads the stepping loops use
int sjo_threads(void) { return omp_get_max_threads(); }

int sjo_create(const sj_instance_desc* d, sjo_sim** out) {
    *out = nullptr;
    sjo_sim* s = new sjo_sim();
    try {
        build(s, *d);
    } catch (const std::string& e) {
        g_err = e;
        delete s;
        return SJ_E_INVALID;
    }
    *out = s;
    return SJ_OK;
}

int sjo_destroy(sjo_sim* s) {
    delete s;
    return SJ_OK;
}

int sjo_step(sjo_sim* s, int64_t n) {
    for (int64_t q = 0; q < n; ++q) step_once(s);
    return SJ_OK;
}

int64_t sjo_steps_done(const sjo_sim* s) { return s->t; }
double sjo_dt(const sjo_sim* s) { return s->dt; }
int64_t sjo_n_samples(const sjo_sim* s) { return (s->t + s->save_span - 1) / s->save_span; }

int sjo_read_monitors(sjo_sim* s, double* out, size_t cap) {
    const long long ns = sjo_n_samples(s);
    if ((size_t)s->n_mon * ns > cap) return SJ_E_RANGE;
    for (int m = 0; m < s->n_mon; ++m)
        for (long long q = 0; q < ns; ++q) out[m * ns + q] = s->mon[m][q];
    return SJ_OK;
}

int sjo_read_dft(sjo_sim* s, double* out, size_t cap) {
    if (s->dft.size() * 2 > cap) return SJ_E_RANGE;
    for (size_t q = 0; q < s->dft.size(); ++q) {
        out[2 * q] = s->dft[q].real();
        out[2 * q + 1] = s->dft[q].imag();
    }
    return SJ_OK;
}

int sjo_read_field(sjo_sim* s, int comp, double* out, size_t cap) {
    if ((size_t)s->N > cap || comp < 0 || comp > 5) return SJ_E_RANGE;
    memcpy(out, s->F[comp].data(), s->N * sizeof(double));
    return SJ_OK;
}

int sjo_write_field(sjo_sim* s, int comp, const double* in, size_t n) {
    if ((size_t)s->N != n || comp < 0 || comp > 5) return SJ_E_RANGE;
    memcpy(s->F[comp].data(), in, n * sizeof(double));
    return SJ_OK;
}

int sjo_read_class_map(sjo_sim* s, uint8_t* out, size_t cap) {
    if ((size_t)s->N * 3 > cap) return SJ_E_RANGE;
    for (int c = 0; c < 3; ++c) memcpy(out + c * s->N, s->cls[c].data(), s->N);
    return SJ_OK;
}

// CPU rasteriser: out[3][nz][ny][nx] region bitmasks at the E points.
int sjo_rasterize(const sj_grid_desc* g, const sj_scene_desc* sc, uint8_t* out) {
    const long long N = (long long)g->nx * g->ny * g->nz;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i)
                for (int c = 0; c < 3; ++c) {
                    const double x = g->origin[0] + ((double)i + (c == 0 ? 0.5 : 0.0)) * g->dx;
                    const double y = g->origin[1] + ((double)j + (c == 1 ? 0.5 : 0.0)) * g->dx;
                    const double z = g->origin[2] + ((double)k + (c == 2 ? 0.5 : 0.0)) * g->dx;
                    unsigned mask = 0;
                    for (int r = 0; r < sc->n_regions; ++r)
                        if (program_in(sc->regions[r].nodes, sc->regions[r].n_nodes, x, y, z)) mask |= 1u << r;
                    out[c * N + ((long long)k * g->ny + j) * g->nx + i] = (uint8_t)mask;
                }
    return SJ_OK;
}

// in_bound's per-region counts at the E points: out[3][R][nz][ny][nx]
int sjo_rasterize_counts(const sj_grid_desc* g, const sj_scene_desc* sc, uint8_t* out) {
    std::vector<double> offs;
    try {
        offs = scene_offsets(sc);
    } catch (const std::string& e) {
        g_err = e;
        return SJ_E_INVALID;
    }
    const long long N = (long long)g->nx * g->ny * g->nz;
    const int R = sc->n_regions;
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i)
                for (int c = 0; c < 3; ++c) {
                    const double x = g->origin[0] + ((double)i + (c == 0 ? 0.5 : 0.0)) * g->dx;
                    const double y = g->origin[1] + ((double)j + (c == 1 ? 0.5 : 0.0)) * g->dx;
                    const double z = g->origin[2] + ((double)k + (c == 2 ? 0.5 : 0.0)) * g->dx;
                    const unsigned long long key = point_counts(sc, offs, x, y, z);
                    const long long q = ((long long)k * g->ny + j) * g->nx + i;
                    for (int r = 0; r < R; ++r) out[((long long)c * R + r) * N + q] = (uint8_t)((key >> (8 * r)) & 255);
                }
    return SJ_OK;
}

// the smoothing offsets: out[8 n][3]
int sjo_smooth_points(int32_t n, double rad, double* out) {
    const std::vector<double> p = smooth_offsets(n, rad);
    std::copy(p.begin(), p.end(), out);
    return SJ_OK;
}

// cgs_material_function::in_bound (src/disp.cpp:264-283) at arbitrary points,
// the scene's smoothing included: out[n]
int sjo_in_bound(const sj_scene_desc* sc, const double* pts, int64_t n, double* out) {
    std::vector<double> offs;
    try {
        offs = scene_offsets(sc);
    } catch (const std::string& e) {
        g_err = e;
        return SJ_E_INVALID;
    }
    const double n1 = (double)(offs.size() / 3 + 1);
    for (int64_t q = 0; q < n; ++q) {
        const unsigned long long key = point_counts(sc, offs, pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
        if (sc->n_regions == 0) {
            out[q] = sc->ambient_eps;
            continue;
        }
        double ret = 0;
        for (int r = 0; r < sc->n_regions; ++r)
            ret += sc->ambient_eps + (sc->regions[r].eps - sc->ambient_eps) * (double)((key >> (8 * r)) & 255) / n1;
        out[q] = ret;
    }
    return SJ_OK;
}

// CSG inclusion at arbitrary points: out[n] = in_root(point) for one region
int sjo_csg_in(const sj_csg_node* nodes, int n_nodes, const double* pts, int64_t n_pts, uint8_t* out) {
    for (int64_t q = 0; q < n_pts; ++q) out[q] = (uint8_t)program_in(nodes, n_nodes, pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
    return SJ_OK;
}

static int fail(const char* msg) {
    g_err = msg;
    return SJ_E_INVALID;
}

int sjo_set_design(sjo_sim* s, const sj_design_desc* d) {
    if (!d) {
        s->des_inv.clear();
        return SJ_OK;
    }
    long long nd = 1;
    for (int a = 0; a < 3; ++a) {
        const int n = a == 0 ? s->nx : (a == 1 ? s->ny : s->nz);
        if (d->n[a] < 1 || d->lo[a] < 0 || d->lo[a] + d->n[a] > n) return fail("design box outside the grid");
        s->des_lo[a] = d->lo[a], s->des_n[a] = d->n[a];
        nd *= d->n[a];
    }
    s->des_inv.resize(nd);
    for (long long q = 0; q < nd; ++q) {
        if (!(d->eps[q] > 0)) return fail("design eps must be > 0");
        s->des_inv[q] = 1.0 / d->eps[q];
    }
    return SJ_OK;
}

// F after n_steps from rest (no gradient)
int sjo_objective(sjo_sim* s, const sj_objective_desc* ob, int64_t n_steps, double* F) {
    std::vector<std::complex<double>> D;
    *F = objective_forward(s, *ob, n_steps, nullptr, D);
    return SJ_OK;
}

// F and dF/d(eps) at the design voxels ([d], eps = 1 / inverse eps)
int sjo_adjoint(sjo_sim* s, const sj_objective_desc* ob, int64_t n_steps, double* grad, double* F) {
    const long long nd = (long long)s->des_inv.size();
    if (nd == 0) return fail("no design region");
    std::vector<double> acc((size_t)n_steps * nd * 3);
    std::vector<std::complex<double>> D;
    *F = objective_forward(s, *ob, n_steps, acc.data(), D);
    std::vector<double> g;
    adjoint_sweep(s, *ob, n_steps, acc.data(), D, g);
    for (long long q = 0; q < nd; ++q) {
        const double inv = s->des_inv[q];
        grad[q] = -inv * inv * (g[3 * q] + g[3 * q + 1] + g[3 * q + 2]);
    }
    return SJ_OK;
}

int sjo_source_dipole(const sj_source_desc* src, double t, double* re, double* im) {
    const std::complex<double> v = dipole(*src, t);
    *re = v.real();
    *im = v.imag();
    return SJ_OK;
}

}  // extern "C"
