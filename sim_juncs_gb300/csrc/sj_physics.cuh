// Per-voxel update arithmetic shared by every stepping schedule.
//
// The formulas restate the leapfrog Yee update, the stretched-coordinate
// CPML auxiliaries and meep's Lorentz/Drude auxiliary-differential equation
// (the lorentzian_susceptibility objects built at src/disp.cpp:538-547),
// in the exact operation order the CPU oracle uses.
#pragma once
#include "sj_internal.h"

namespace sj {

// Store monitor sample v of monitor column ms taken before step n, and apply
// the divergence guard (bound_geom::run flags samples above 1000,
// src/disp.cpp:727-729): the first sample of the sim with |v| above the bound,
// or not finite, is recorded in the host-mapped record, flag last.
template <typename real>
__device__ __forceinline__ void monitor_store(const InstDev<real>& I, long long n, int ms, double v,
                                              DevState* st) {
    const long long s = n / I.save_span;
    if (s < I.mon_cap)
        I.mon[s * I.n_mon + ms] = v;
    else
        st->status = SJ_E_RANGE;
    const double b = I.guard_bound;
    if (b > 0.0 && (!(fabs(v) <= b) || isinf(v)) && I.guard_flag) {
        if (atomicCAS(I.guard_flag, 0, 1) == 0) {
            GuardRecord* g = I.guard;
            g->inst = I.index;
            g->monitor = ms;
            g->step = n;
            g->value = v;
            __threadfence_system();
            *reinterpret_cast<volatile int*>(&g->flag) = 1;
            __threadfence_system();
        }
    }
}

template <typename real>
__device__ __forceinline__ int dim_of(const InstDev<real>& I, int a) {
    return a == 0 ? I.nx : (a == 1 ? I.ny : I.nz);
}

// Is coordinate q of axis a inside that axis' CPML face slabs?
template <typename real>
__device__ __forceinline__ bool in_slab(const InstDev<real>& I, int a, int q) {
    return q < I.pl[a] || q >= dim_of(I, a) - I.ph[a];
}

// curl term of component axis CA (0..2) including the CPML auxiliaries.
// d1 = difference along A1 = CA+1, d2 = along A2 = CA+2 (mod 3).
// HALF selects the half-integer profile (H components) or the integer one (E).
// o is the voxel's offset (psi arrays share the field layout); psi_in and
// psi_out may alias (in-place schedules); store = false recomputes a cell
// another block owns without writing its auxiliaries.
template <typename real, int CA, bool HALF>
__device__ __forceinline__ real curl_psi(const InstDev<real>& I, int i, int j, int k, long long o,
                                         real d1, real d2, real* const* psi_in, real* const* psi_out,
                                         bool store = true) {
    constexpr int A1 = (CA + 1) % 3, A2 = (CA + 2) % 3;
    constexpr int P1 = (CA > A1) ? CA - 1 : CA;  // slot of CA in axis A1's pair
    constexpr int P2 = (CA > A2) ? CA - 1 : CA;
    constexpr int BOFF = HALF ? 2 : 0;
    real cur = d1 - d2;
    {
        const int q = A1 == 0 ? i : (A1 == 1 ? j : k);
        if (in_slab(I, A1, q)) {
            const int n = dim_of(I, A1);
            const real b = I.prof[A1][BOFF * n + q];
            const real c = I.prof[A1][(BOFF + 1) * n + q];
            const long long x = (long long)P1 * I.vol + o;
            const real psi = b * psi_in[A1][x] + c * d1;
            if (store) psi_out[A1][x] = psi;
            cur += psi;
        }
    }
    {
        const int q = A2 == 0 ? i : (A2 == 1 ? j : k);
        if (in_slab(I, A2, q)) {
            const int n = dim_of(I, A2);
            const real b = I.prof[A2][BOFF * n + q];
            const real c = I.prof[A2][(BOFF + 1) * n + q];
            const long long x = (long long)P2 * I.vol + o;
            const real psi = b * psi_in[A2][x] + c * d2;
            if (store) psi_out[A2][x] = psi;
            cur -= psi;
        }
    }
    return cur;
}

// Subtract every source of component `comp` that covers (i,j,k) at step n.
template <typename real>
__device__ __forceinline__ real apply_sources(const InstDev<real>& I, int comp, int i, int j, int k,
                                              long long n, real acc) {
    for (int s = 0; s < I.n_src; ++s) {
        const SrcDev<real>& src = I.src[s];
        if (src.comp != comp) continue;
        const int di = i - src.lo[0], dj = j - src.lo[1], dk = k - src.lo[2];
        if ((unsigned)di < (unsigned)src.n[0] && (unsigned)dj < (unsigned)src.n[1] &&
            (unsigned)dk < (unsigned)src.n[2]) {
            acc -= (real)src.tab[n] * src.w[0][di] * src.w[1][dj] * src.w[2][dk];
        }
    }
    return acc;
}

// E-component finish: sources, polarisation ADE, eps_inf^{-1} scaling.
template <typename real, int CA>
__device__ __forceinline__ real e_finish(const InstDev<real>& I, int i, int j, int k, long long n,
                                         int cb, real e_old, real cur, bool store = true,
                                         bool sources = true) {
    real acc = I.S * cur;
    if (sources && I.n_src) acc = apply_sources(I, CA, i, j, k, n, acc);
    const real* cf = I.coef + (long long)cb * I.ncoef;
    if (I.cflag[cb] & 1) {
        const long long di =
            ((long long)(k - I.dlo[2]) * I.dn[1] + (j - I.dlo[1])) * I.dn[0] + (i - I.dlo[0]);
        for (int p = 0; p < I.n_poles; ++p) {
            if (cf[3 + 3 * p + CA] == real(0)) continue;  // P stays 0: acc - (+0) = acc
            real* pp = I.P + ((long long)(p * 2 + 0) * 3 + CA) * I.dvol + di;
            real* pm = I.P + ((long long)(p * 2 + 1) * 3 + CA) * I.dvol + di;
            const real pn = *pp, pq = *pm;
            const real pnew = I.A[p] * pn + I.B[p] * pq + cf[3 + 3 * p + CA] * e_old;
            acc -= (pnew - pn);
            if (store) {
                *pm = pn;
                *pp = pnew;
            }
        }
    }
    real inv = cf[CA];
    if (I.dinv) {  // design region: per-voxel inverse eps; acc recorded while a segment is re-run
        const int u = i - I.des_lo[0], v = j - I.des_lo[1], w = k - I.des_lo[2];
        if ((unsigned)u < (unsigned)I.des_n[0] && (unsigned)v < (unsigned)I.des_n[1] &&
            (unsigned)w < (unsigned)I.des_n[2]) {
            const long long d = ((long long)w * I.des_n[1] + v) * I.des_n[0] + u;
            inv = I.dinv[d];
            if (store && I.rec_acc && n >= I.rec_t0 && n < I.rec_t0 + I.rec_len) {
                const long long nd = (long long)I.des_n[0] * I.des_n[1] * I.des_n[2];
                I.rec_acc[((n - I.rec_t0) * nd + d) * 3 + CA] = acc;
            }
        }
    }
    return e_old + inv * acc;
}

// e_finish with the combo's coefficient row (cf) and dispersion flag supplied
// by the caller (e.g. from a shared-memory copy of the combo table).
template <typename real, int CA>
__device__ __forceinline__ real e_finish_row(const InstDev<real>& I, int i, int j, int k, long long n,
                                             const real* cf, bool disp, real e_old, real cur, bool store,
                                             bool sources) {
    real acc = I.S * cur;
    if (sources && I.n_src) acc = apply_sources(I, CA, i, j, k, n, acc);
    if (disp) {
        const long long di =
            ((long long)(k - I.dlo[2]) * I.dn[1] + (j - I.dlo[1])) * I.dn[0] + (i - I.dlo[0]);
        for (int p = 0; p < I.n_poles; ++p) {
            if (cf[3 + 3 * p + CA] == real(0)) continue;  // P stays 0: acc - (+0) = acc
            real* pp = I.P + ((long long)(p * 2 + 0) * 3 + CA) * I.dvol + di;
            real* pm = I.P + ((long long)(p * 2 + 1) * 3 + CA) * I.dvol + di;
            const real pn = *pp, pq = *pm;
            const real pnew = I.A[p] * pn + I.B[p] * pq + cf[3 + 3 * p + CA] * e_old;
            acc -= (pnew - pn);
            if (store) {
                *pm = pn;
                *pp = pnew;
            }
        }
    }
    return e_old + cf[CA] * acc;
}

}  // namespace sj
