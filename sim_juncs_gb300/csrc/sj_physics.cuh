// Per-voxel update arithmetic shared by every stepping schedule.
//
// The formulas restate the leapfrog Yee update, the stretched-coordinate
// CPML auxiliaries and meep's Lorentz/Drude auxiliary-differential equation
// (the lorentzian_susceptibility objects built at src/disp.cpp:538-547),
// in the exact operation order the CPU oracle uses.
#pragma once
#include "sj_internal.h"

namespace sj {

template <typename real>
__device__ __forceinline__ int dim_of(const InstDev<real>& I, int a) {
    return a == 0 ? I.nx : (a == 1 ? I.ny : I.nz);
}

// Offset of voxel (i,j,k) inside the CPML slab storage of axis a, or -1.
// Slab layouts: x -> [nz][ny][pl+ph], y -> [nz][pl+ph][px], z -> [pl+ph][ny][px].
template <typename real>
__device__ __forceinline__ long long slab_idx(const InstDev<real>& I, int a, int i, int j, int k) {
    const int q = a == 0 ? i : (a == 1 ? j : k);
    const int n = dim_of(I, a);
    const int pl = I.pl[a], ph = I.ph[a];
    int qq;
    if (q < pl)
        qq = q;
    else if (q >= n - ph)
        qq = q - (n - ph) + pl;
    else
        return -1;
    const int w = pl + ph;
    if (a == 0) return ((long long)k * I.ny + j) * w + qq;
    if (a == 1) return ((long long)k * w + qq) * I.px + i;
    return ((long long)qq * I.ny + j) * I.px + i;
}

// curl term of component axis CA (0..2) including the CPML auxiliaries.
// d1 = difference along A1 = CA+1, d2 = along A2 = CA+2 (mod 3).
// HALF selects the half-integer profile (H components) or the integer one (E).
// psi_in/psi_out may alias (in-place schedules); store = false recomputes a
// cell another block owns without writing its auxiliaries.
template <typename real, int CA, bool HALF>
__device__ __forceinline__ real curl_psi(const InstDev<real>& I, int i, int j, int k, real d1,
                                         real d2, real* const* psi_in, real* const* psi_out,
                                         bool store = true) {
    constexpr int A1 = (CA + 1) % 3, A2 = (CA + 2) % 3;
    constexpr int P1 = (CA > A1) ? CA - 1 : CA;  // slot of CA in axis A1's pair
    constexpr int P2 = (CA > A2) ? CA - 1 : CA;
    constexpr int BOFF = HALF ? 2 : 0;
    real cur = d1 - d2;
    {
        const long long s = slab_idx(I, A1, i, j, k);
        if (s >= 0) {
            const int n = dim_of(I, A1);
            const int q = A1 == 0 ? i : (A1 == 1 ? j : k);
            const real b = I.prof[A1][BOFF * n + q];
            const real c = I.prof[A1][(BOFF + 1) * n + q];
            const long long o = (long long)P1 * I.slabvol[A1] + s;
            const real psi = b * psi_in[A1][o] + c * d1;
            if (store) psi_out[A1][o] = psi;
            cur += psi;
        }
    }
    {
        const long long s = slab_idx(I, A2, i, j, k);
        if (s >= 0) {
            const int n = dim_of(I, A2);
            const int q = A2 == 0 ? i : (A2 == 1 ? j : k);
            const real b = I.prof[A2][BOFF * n + q];
            const real c = I.prof[A2][(BOFF + 1) * n + q];
            const long long o = (long long)P2 * I.slabvol[A2] + s;
            const real psi = b * psi_in[A2][o] + c * d2;
            if (store) psi_out[A2][o] = psi;
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
