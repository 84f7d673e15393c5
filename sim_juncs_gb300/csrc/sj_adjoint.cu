// Discrete adjoint of the split schedule's step, and the objective DFT.
//
// The step is linear in the fields with coefficients that do not depend on
// them (S, eps_inf^{-1}, the CPML b and c, the ADE's A, B and C sigma), so
// its adjoint is the reverse sequence of the transposed sub-updates, with the
// same coefficients: for step n, first the transpose of the E update
// (eps_inf^{-1}, the polarisation ADE, the E-side psi, the backward
// differences of H), then the transpose of the H update (the H-side psi and
// the forward differences of E).  A difference's adjoint is scattered to the
// two cells it reads: a kernel writes the per-cell adjoints of both
// differences (t1, t2 for the E update, t3, t4 for the H update) and the
// next gathers them, one thread per cell, so no two threads write one value.
// Per step: k_adj_e (the E update's transpose), then k_adj_e_gather_h (the
// gather into dF/dH and, at the same cell, the H update's transpose).  The
// gather of the H update's differences into dF/dE^n needs every cell's t3,
// t4 of step n, so it runs at the start of step n-1's k_adj_e, which reads
// the same cell's eb next (k_adj_e<GATHER>): a step is two launches.  The
// objective's dF/dE^n source, added to eb between the steps, then precedes
// that gather instead of following it (the same sum in another order), and
// the last step's gather, whose dF/dE^0 nothing reads, is never run.  The
// gradient with respect to a design voxel's inverse eps is
// sum_n dF/dE^{n+1} * acc^n, acc^n being the E update's bracket at step n,
// recorded while the segment is re-run forward.
// One launch per instance; the descriptor travels as a kernel parameter.
#include "sj_physics.cuh"

namespace sj {

namespace {

constexpr int AX = 32, AY = 8;

template <typename real>
__device__ __forceinline__ real prof_at(const InstDev<real>& I, int a, int q, int which) {
    // which: 0 = b (integer points), 1 = c (integer), 2 = b (half), 3 = c (half)
    return I.prof[a][which * dim_of(I, a) + q];
}

template <typename real>
__device__ __forceinline__ long long stride_of(const InstDev<real>& I, int a) {
    return a == 0 ? 1LL : (a == 1 ? (long long)I.px : I.plane);
}

template <typename real>
__device__ __forceinline__ long long design_index(const InstDev<real>& I, int i, int j, int k) {
    if (!I.dinv) return -1;
    const int u = i - I.des_lo[0], v = j - I.des_lo[1], w = k - I.des_lo[2];
    if ((unsigned)u >= (unsigned)I.des_n[0] || (unsigned)v >= (unsigned)I.des_n[1] ||
        (unsigned)w >= (unsigned)I.des_n[2])
        return -1;
    return ((long long)w * I.des_n[1] + v) * I.des_n[0] + u;
}

// Transpose of the E update at one voxel (three components).  eb holds
// dF/dE^{n+1} on entry and the E update's share of dF/dE^n on exit; with
// GATHER, eb first completes dF/dE^{n+1} with what the H update's
// differences of step n+1 read from E here (t3, t4 of this cell and of its
// -1 neighbours).  Every load of the voxel goes out first (eb, t3 and t4, the E-side
// psi adjoints of its slab axes, the polarisation adjoints of the poles its
// material has: pmask), then the three components are formed in turn.
// Offsets within the instance are 32-bit (sj_adjoint_gradient admits grids
// of fewer than 2^31 voxels), and each slab axis' profile is read once.
#ifndef SJ_ADJ_E_MINB
#define SJ_ADJ_E_MINB 3
#endif
template <typename real, bool GATHER>
__global__ void __launch_bounds__(AX * AY, SJ_ADJ_E_MINB) k_adj_e(const __grid_constant__ AdjDev<real> A, long long n) {
    const InstDev<real>& I = A.I;
    const int i = blockIdx.x * AX + threadIdx.x, j = blockIdx.y * AY + threadIdx.y, k = blockIdx.z;
    if (i >= I.nx || j >= I.ny) return;
    const unsigned vol = (unsigned)I.vol;
    const unsigned st[3] = {1u, (unsigned)I.px, (unsigned)I.plane};
    const unsigned o = (unsigned)k * st[2] + (unsigned)j * st[1] + (unsigned)i;
    const int idx[3] = {i, j, k};
    const int cb = I.combo[o];
    const real* cf = I.coef + cb * I.ncoef;
    const unsigned mask = I.pmask[cb];
    const unsigned di = mask ? ((unsigned)(k - I.dlo[2]) * (unsigned)I.dn[1] + (unsigned)(j - I.dlo[1])) *
                                       (unsigned)I.dn[0] + (unsigned)(i - I.dlo[0])
                             : 0u;
    const size_t dvol = (size_t)I.dvol;
    const long long d = design_index(I, i, j, k);
    const long long nd = (long long)I.des_n[0] * I.des_n[1] * I.des_n[2];
    const bool sl[3] = {in_slab(I, 0, i), in_slab(I, 1, j), in_slab(I, 2, k)};
    // the CPML profile (integer points) of each slab axis at the voxel
    real pb_[3], pc_[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        pb_[a] = sl[a] ? prof_at(I, a, idx[a], 0) : real(0);
        pc_[a] = sl[a] ? prof_at(I, a, idx[a], 1) : real(0);
    }
    real ebo[3], q1[3], q2[3];
    real g3[3], g4[3], m3[3], m4[3];  // GATHER: t3, t4 here and at the -1 neighbours
    int pa[3], pz[3];
    real pa0[3], pa1[3], pz0[3], pz1[3];
    unsigned rest[3];
#pragma unroll
    for (int ca = 0; ca < 3; ++ca) {
        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
        const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
        ebo[ca] = A.eb[ca][o];
        q1[ca] = sl[a1] ? A.psEb[a1][(unsigned)s1 * vol + o] : real(0);
        q2[ca] = sl[a2] ? A.psEb[a2][(unsigned)s2 * vol + o] : real(0);
        if (GATHER) {
            g3[ca] = A.t3[ca][o], g4[ca] = A.t4[ca][o];
            m3[ca] = idx[a1] > 0 ? A.t3[ca][o - st[a1]] : real(0);
            m4[ca] = idx[a2] > 0 ? A.t4[ca][o - st[a2]] : real(0);
        }
        const unsigned m = (mask >> (8 * ca)) & 255u, m2 = m & (m - 1);
        pa[ca] = m ? __ffs(m) - 1 : -1;
        pz[ca] = m2 ? __ffs(m2) - 1 : -1;
        rest[ca] = m2 & (m2 - 1);
        // a pole's dF/dP^{n+1} at level 0 of its rows, dF/dP^n three rows on
        const real* P0 = A.pb + (size_t)(max(pa[ca], 0) * 6 + ca) * dvol + di;
        const real* P1 = A.pb + (size_t)(max(pz[ca], 0) * 6 + ca) * dvol + di;
        pa0[ca] = m ? P0[0] : real(0), pa1[ca] = m ? P0[3 * dvol] : real(0);
        pz0[ca] = m2 ? P1[0] : real(0), pz1[ca] = m2 ? P1[3 * dvol] : real(0);
    }
    if (GATHER) {
        // dF/dE^{n+1} += what the H update's differences of step n+1 read here
#pragma unroll
        for (int ca = 0; ca < 3; ++ca) {
            const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
            real v = -g3[ca];
            if (idx[a1] > 0) v += m3[ca];
            ebo[a2] += v;
            real w = -g4[ca];
            if (idx[a2] > 0) w += m4[ca];
            ebo[a1] += w;
        }
    }
#pragma unroll
    for (int ca = 0; ca < 3; ++ca) {
        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
        const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
        const real inv = d >= 0 ? I.dinv[d] : cf[ca];
        if (d >= 0) A.g[d * 3 + ca] += (double)ebo[ca] * (double)A.rec[((n - A.rec_t0) * nd + d) * 3 + ca];
        const real ab = inv * ebo[ca];  // adjoint of the bracket acc
        real ein = ebo[ca];
        // one pole's ADE transpose: (dF/dP^{n+1}, dF/dP^n) -> (dF/dP^n, dF/dP^{n-1})
        auto pole = [&](int p, real q0v, real q1v) {
            real* p0 = A.pb + (size_t)(p * 6 + ca) * dvol + di;
            real* p1 = p0 + 3 * dvol;
            const real pnb = q0v - ab;                    // dF/dP^{n+1}
            const real pn = q1v + ab + I.A[p] * pnb;      // dF/dP^n
            *p1 = I.B[p] * pnb;                           // dF/dP^{n-1}
            *p0 = pn;
            ein += cf[3 + 3 * p + ca] * pnb;
        };
        if (pa[ca] >= 0) pole(pa[ca], pa0[ca], pa1[ca]);
        if (pz[ca] >= 0) pole(pz[ca], pz0[ca], pz1[ca]);
        for (unsigned m = rest[ca]; m; m &= m - 1) {
            const int p = __ffs(m) - 1;
            const real* x = A.pb + (size_t)(p * 6 + ca) * dvol + di;
            pole(p, x[0], x[3 * dvol]);
        }
        A.eb[ca][o] = ein;
        const real cv = I.S * ab;  // adjoint of the curl
        real t1 = cv, t2 = -cv;
        if (sl[a1]) {
            const real t = q1[ca] + cv;
            t1 = cv + pc_[a1] * t;
            A.psEb[a1][(unsigned)s1 * vol + o] = pb_[a1] * t;
        }
        if (sl[a2]) {
            const real t = q2[ca] - cv;
            t2 = -cv + pc_[a2] * t;
            A.psEb[a2][(unsigned)s2 * vol + o] = pb_[a2] * t;
        }
        A.t1[ca][o] = t1;  // adjoint of H_a2(o) - H_a2(o - e_a1)
        A.t2[ca][o] = t2;  // adjoint of H_a1(o) - H_a1(o - e_a2)
    }
}

// dF/dH^{n+1/2} += what the E update's differences read from H at this cell
// (t1, t2 of this cell and its +1 neighbours); then, at the same cell, the
// transpose of the H update: hb carries over unchanged to H^{n-1/2}, its
// share through the curl of E goes to t3, t4.
template <typename real>
__global__ void __launch_bounds__(AX * AY) k_adj_e_gather_h(const __grid_constant__ AdjDev<real> A) {
    const InstDev<real>& I = A.I;
    const int i = blockIdx.x * AX + threadIdx.x, j = blockIdx.y * AY + threadIdx.y, k = blockIdx.z;
    if (i >= I.nx || j >= I.ny) return;
    const long long o = (long long)k * I.plane + (long long)j * I.px + i;
    const int idx[3] = {i, j, k};
    real hb[3] = {A.hb[0][o], A.hb[1][o], A.hb[2][o]};
    for (int ca = 0; ca < 3; ++ca) {
        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
        real v = A.t1[ca][o];
        if (idx[a1] + 1 < dim_of(I, a1)) v -= A.t1[ca][o + stride_of(I, a1)];
        hb[a2] += v;
        real w = A.t2[ca][o];
        if (idx[a2] + 1 < dim_of(I, a2)) w -= A.t2[ca][o + stride_of(I, a2)];
        hb[a1] += w;
    }
    for (int ca = 0; ca < 3; ++ca) {
        A.hb[ca][o] = hb[ca];
        const int a1 = (ca + 1) % 3, a2 = (ca + 2) % 3;
        const int s1 = ca > a1 ? ca - 1 : ca, s2 = ca > a2 ? ca - 1 : ca;
        const real cv = -I.S * hb[ca];
        real t1 = cv, t2 = -cv;
        if (in_slab(I, a1, idx[a1])) {
            real* ps = A.psHb[a1] + (long long)s1 * I.vol + o;
            const real t = *ps + cv;
            t1 = cv + prof_at(I, a1, idx[a1], 3) * t;
            *ps = prof_at(I, a1, idx[a1], 2) * t;
        }
        if (in_slab(I, a2, idx[a2])) {
            real* ps = A.psHb[a2] + (long long)s2 * I.vol + o;
            const real t = *ps - cv;
            t2 = -cv + prof_at(I, a2, idx[a2], 3) * t;
            *ps = prof_at(I, a2, idx[a2], 2) * t;
        }
        A.t3[ca][o] = t1;  // adjoint of E_a2(o + e_a1) - E_a2(o)
        A.t4[ca][o] = t2;  // adjoint of E_a1(o + e_a2) - E_a1(o)
    }
}

// One thread per (objective cell, E component in the mask).
template <typename real>
__global__ void k_objective(const __grid_constant__ InstDev<real> I, int cur, const int* __restrict__ cells,
                            int n_cells, int mask, double freq, double2* D, long long n, int sample,
                            real* ebx, real* eby, real* ebz) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = t / 3, c = t % 3;
    if (q >= n_cells || !((mask >> c) & 1)) return;
    const long long o = (long long)cells[3 * q + 2] * I.plane + (long long)cells[3 * q + 1] * I.px + cells[3 * q];
    double sn, cs;
    sincospi(2.0 * freq * ((double)n * I.dt), &sn, &cs);
    if (sample) {
        const double e = (double)I.F[cur][c][o] * I.dt;
        double2 v = D[t];
        v.x += e * cs;
        v.y += e * sn;
        D[t] = v;
    } else {
        real* eb = c == 0 ? ebx : (c == 1 ? eby : ebz);
        const double2 v = D[t];
        eb[o] += (real)(2.0 * I.dt * (v.x * cs + v.y * sn));
    }
}

}  // namespace

template <typename real>
cudaError_t launch_adjoint_step(const AdjDev<real>& a, long long n, bool first, cudaStream_t s) {
    const dim3 block(AX, AY), grid((a.I.nx + AX - 1) / AX, (a.I.ny + AY - 1) / AY, a.I.nz);
    if (first)
        k_adj_e<real, false><<<grid, block, 0, s>>>(a, n);
    else
        k_adj_e<real, true><<<grid, block, 0, s>>>(a, n);
    k_adj_e_gather_h<real><<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}


template <typename real>
cudaError_t launch_objective(const InstDev<real>& I, int cur, const int* d_cells, int n_cells, int comp_mask,
                             double freq, double2* d_D, long long n, bool sample, real* const* eb, cudaStream_t s) {
    const int threads = 3 * n_cells;
    if (threads == 0) return cudaSuccess;
    k_objective<real><<<(threads + 127) / 128, 128, 0, s>>>(I, cur, d_cells, n_cells, comp_mask, freq, d_D, n,
                                                            sample ? 1 : 0, eb ? eb[0] : nullptr,
                                                            eb ? eb[1] : nullptr, eb ? eb[2] : nullptr);
    return cudaGetLastError();
}

template cudaError_t launch_adjoint_step<float>(const AdjDev<float>&, long long, bool, cudaStream_t);
template cudaError_t launch_adjoint_step<double>(const AdjDev<double>&, long long, bool, cudaStream_t);
template cudaError_t launch_objective<float>(const InstDev<float>&, int, const int*, int, int, double, double2*,
                                             long long, bool, float* const*, cudaStream_t);
template cudaError_t launch_objective<double>(const InstDev<double>&, int, const int*, int, int, double, double2*,
                                              long long, bool, double* const*, cudaStream_t);
}  // namespace sj
