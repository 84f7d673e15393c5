// Fused single-pass leapfrog stepper (the "fused" schedule, default for FP32).
//
// One step reads E^n, H^{n-1/2} (ping-pong buffer `cur`) and writes
// H^{n+1/2}, E^{n+1} (buffer cur^1): each field component crosses HBM once in
// and once out per step.
//
// A thread owns one (i, j) column and marches along z over a segment of ZB
// planes; a block is a 32 x 8 tile of columns.  For each plane k the thread
// updates H at its own cell and recomputes H at (i-1, j) and (i, j-1) — the
// two neighbours the E update needs, owned by other threads — instead of
// exchanging them, so the kernels need no shared memory and no barrier; the
// neighbour values come from L1/L2.  E and H of plane k+1 that become plane
// k's values next iteration are carried in registers, as is the own H of
// plane k-1.  A segment starting at z0 > 0 first recomputes H of plane z0-1
// (owned by the previous segment).  The ping-pong buffers (fields and H-side
// CPML psi) make the recomputation race-free: nothing a block reads is
// written during the step.
//
// Three kernels share the tiles of a step, by what a tile's footprint (own
// cells and the recomputed x-1/y-1/z-1 neighbours) touches.  k_lean_plain
// takes tiles clear of CPML slabs, sources and dispersive voxels: a short
// loop that keeps few registers and runs at high occupancy.  k_lean_slab
// takes tiles in the slabs of exactly one axis (most of the CPML volume),
// compiled per axis so the other axes' terms vanish.  k_lean_general takes
// the rest (slab edges and corners, sources, polarisations) and the probe
// blocks.  The three run concurrently on forked streams, and the last block
// of the step, whichever kernel it belongs to, advances the step counter.
// All evaluate one update
// formula, so a voxel's result does not depend on which kernel (or which
// tiling) updated it:
//   H^{n+1/2} = fma(-S, curl E, H^{n-1/2}) [- dt J_H]
//   E^{n+1}   = fma(S ε∞⁻¹, curl H, E^n) [then fma(-ε∞⁻¹, dt J + Σ_p ΔP_p, ·)]
// with curl including the CPML ψ terms.  This file is compiled with
// contraction off (-fmad=false): every fused multiply-add is the explicit
// one written here.
#include <algorithm>
#include <vector>

#include "sj_physics.cuh"

namespace sj {

constexpr int LX = 32, LY = 8;      // tile of columns per block
constexpr int LMAXF = 256;

// resident blocks per SM each kernel is compiled for (register budget)
#ifndef SJ_LEAN_PLAIN_MINB
#define SJ_LEAN_PLAIN_MINB 4
#endif
#ifndef SJ_LEAN_SLAB_MINB
#define SJ_LEAN_SLAB_MINB 4
#endif
#ifndef SJ_LEAN_GEN_MINB
#define SJ_LEAN_GEN_MINB 3
#endif
template <typename real>
constexpr int plain_minb() { return sizeof(real) == 4 ? SJ_LEAN_PLAIN_MINB : 3; }
template <typename real>
constexpr int slab_minb() { return sizeof(real) == 4 ? SJ_LEAN_SLAB_MINB : 2; }
template <typename real>
constexpr int general_minb() { return sizeof(real) == 4 ? SJ_LEAN_GEN_MINB : 2; }

// Reads of buffer `cur` (fields, H-side psi), profiles and material tables
// go through the non-coherent path: nothing writes them during the step, and
// the compiler may then move them ahead of the stores of the previous plane.
template <typename real>
__device__ __forceinline__ real ldg(const real* p, long long o) {
    return __ldg(p + o);
}
template <typename real>
__device__ __forceinline__ real ldz(const real* p, long long o, bool ok) {
    return ok ? __ldg(p + o) : real(0);
}

// Does the tile's footprint touch a source (own cells and the x-1 / y-1 /
// z-1 neighbours whose H it recomputes), or do its own cells touch the
// bounding box of the dispersive voxels?  Block-uniform.
template <typename real>
__device__ __forceinline__ bool tile_has_extras(const InstDev<real>& I, int i0, int j0, int z0, int z1) {
    const int xa = max(i0 - 1, 0), xb = min(i0 + LX, I.nx) - 1;
    const int ya = max(j0 - 1, 0), yb = min(j0 + LY, I.ny) - 1;
    const int za = max(z0 - 1, 0), zb = z1 - 1;
    for (int q = 0; q < I.n_src; ++q) {
        const SrcDev<real>& sv = I.src[q];
        if (sv.lo[0] <= xb && sv.lo[0] + sv.n[0] > xa && sv.lo[1] <= yb && sv.lo[1] + sv.n[1] > ya &&
            sv.lo[2] <= zb && sv.lo[2] + sv.n[2] > za)
            return true;
    }
    if (I.n_poles > 0 && I.dvol > 0 && I.dlo[0] <= xb && I.dlo[0] + I.dn[0] > i0 && I.dlo[1] <= yb &&
        I.dlo[1] + I.dn[1] > j0 && I.dlo[2] <= zb && I.dlo[2] + I.dn[2] > z0)
        return true;
    return false;
}

// ------------------------------------------------------------- plain tiles
template <typename real, int ZB>
__device__ __forceinline__ void plain_block(const InstDev<real>& I, int tx, int ty, int tz, int cur) {
    const int i = tx * LX + threadIdx.x, j = ty * LY + threadIdx.y;
    const int z0 = tz * ZB, z1 = min(I.nz, z0 + ZB);
    if (i >= I.nx || j >= I.ny) return;
    const long long px = I.px, plane = I.plane;
    const real* eX = I.F[cur][0];
    const real* eY = I.F[cur][1];
    const real* eZ = I.F[cur][2];
    const real* hX = I.F[cur][3];
    const real* hY = I.F[cur][4];
    const real* hZ = I.F[cur][5];
    real* oEX = I.F[cur ^ 1][0];
    real* oEY = I.F[cur ^ 1][1];
    real* oEZ = I.F[cur ^ 1][2];
    real* oHX = I.F[cur ^ 1][3];
    real* oHY = I.F[cur ^ 1][4];
    real* oHZ = I.F[cur ^ 1][5];
    const real S = I.S;
    const bool xm = i > 0, ym = j > 0, xp = i + 1 < I.nx, yp = j + 1 < I.ny;

    int k = z0 > 0 ? z0 - 1 : 0;
    long long o = (long long)k * plane + (long long)j * px + i;
    real ex_c = ldg(eX, o), ey_c = ldg(eY, o);
    real exm_c = ldz(eX, o - 1, xm), eym_c = ldz(eY, o - px, ym);
    real hxp = 0, hyp = 0;
    for (; k < z1; ++k, o += plane) {
        const bool kp = k + 1 < I.nz;
        const real ex_n = ldz(eX, o + plane, kp), ey_n = ldz(eY, o + plane, kp);
        const real exm_n = ldz(eX, o + plane - 1, kp && xm), eym_n = ldz(eY, o + plane - px, kp && ym);
        const real ez = ldg(eZ, o);
        const real ez_xp = ldz(eZ, o + 1, xp), ez_yp = ldz(eZ, o + px, yp);
        const real ey_xp = ldz(eY, o + 1, xp), ex_yp = ldz(eX, o + px, yp);
        const real hx = fma(-S, (ez_yp - ez) - (ey_n - ey_c), ldg(hX, o));
        const real hy = fma(-S, (ex_n - ex_c) - (ez_xp - ez), ldg(hY, o));
        const real hz = fma(-S, (ey_xp - ey_c) - (ex_yp - ex_c), ldg(hZ, o));
        if (k >= z0) {
            const real ez_xm = ldz(eZ, o - 1, xm), ez_ym = ldz(eZ, o - px, ym);
            const real ex_xmyp = ldz(eX, o - 1 + px, xm && yp), ey_xpym = ldz(eY, o + 1 - px, xp && ym);
            const real ex_ym = ldz(eX, o - px, ym), ey_xm = ldz(eY, o - 1, xm);
            const real hy_xm = xm ? fma(-S, (exm_n - exm_c) - (ez - ez_xm), ldg(hY, o - 1)) : real(0);
            const real hz_xm = xm ? fma(-S, (ey_c - ey_xm) - (ex_xmyp - exm_c), ldg(hZ, o - 1)) : real(0);
            const real hx_ym = ym ? fma(-S, (ez - ez_ym) - (eym_n - eym_c), ldg(hX, o - px)) : real(0);
            const real hz_ym = ym ? fma(-S, (ey_xpym - eym_c) - (ex_c - ex_ym), ldg(hZ, o - px)) : real(0);
            oHX[o] = hx;
            oHY[o] = hy;
            oHZ[o] = hz;
            const real* cf = I.coef + (int)__ldg(I.combo + o) * I.ncoef;
            oEX[o] = fma(S * ldg(cf, 0), (hz - hz_ym) - (hy - hyp), ex_c);
            oEY[o] = fma(S * ldg(cf, 1), (hx - hxp) - (hz - hz_xm), ey_c);
            oEZ[o] = fma(S * ldg(cf, 2), (hy - hy_xm) - (hx - hx_ym), ez);
        }
        hxp = hx;
        hyp = hy;
        ex_c = ex_n;
        ey_c = ey_n;
        exm_c = exm_n;
        eym_c = eym_n;
    }
}

// ------------------------------------------------------- slab / general tiles
// dt J of every source of component `comp` covering (i, j, k) at step n
template <typename real>
__device__ __forceinline__ real source_sum(const InstDev<real>& I, int comp, int i, int j, int k, long long n,
                                           bool& hit) {
    real acc = 0;
    for (int s = 0; s < I.n_src; ++s) {
        const SrcDev<real>& src = I.src[s];
        if (src.comp != comp) continue;
        const int di = i - src.lo[0], dj = j - src.lo[1], dk = k - src.lo[2];
        if ((unsigned)di < (unsigned)src.n[0] && (unsigned)dj < (unsigned)src.n[1] &&
            (unsigned)dk < (unsigned)src.n[2]) {
            acc += (real)src.tab[n] * src.w[0][di] * src.w[1][dj] * src.w[2][dk];
            hit = true;
        }
    }
    return acc;
}

// One CPML term of a curl: psi = fma(b, psi_old, c d), added (ADD) or
// subtracted from cv where the cell is in the slab (on).  psi_old is read
// only for slab cells (non-coherently for the ping-pong H side, NC); AX
// (compile time) removes axes a tile cannot touch.
template <bool AX, bool ADD, bool NC, typename real>
__device__ __forceinline__ void pml_term(real& cv, bool on, real b, real c, real d, const real* pin, real* pout,
                                         long long x, bool store) {
    if (!AX) return;
    const real po = on ? (NC ? __ldg(pin + x) : pin[x]) : real(0);
    const real ps = fma(b, po, c * d);
    if (on) {
        if (store) pout[x] = ps;
        cv = ADD ? cv + ps : cv - ps;
    }
}

// H^{n+1/2} = fma(-S, curl, H^{n-1/2}) [- dt J]
template <bool EXTRAS, typename real>
__device__ __forceinline__ real h_new(const InstDev<real>& I, int comp, real cv, real hold, bool src, int ci, int cj,
                                      int k, long long n) {
    real h = fma(-I.S, cv, hold);
    if (EXTRAS && src) {
        bool hit = false;
        const real J = source_sum(I, comp, ci, cj, k, n, hit);
        if (hit) h = h - J;
    }
    return h;
}

// E^{n+1} of the own cell: Yee term, then sources and the polarisation ADE
// as one correction scaled by eps_inf^{-1}.
template <bool EXTRAS, int CA, typename real>
__device__ __forceinline__ real e_new(const InstDev<real>& I, int i, int j, int k, long long n, const real* cf,
                                      bool disp, real e_old, real cv, bool store, bool src) {
    real e = fma(I.S * ldg(cf, CA), cv, e_old);
    if (!EXTRAS) return e;
    bool hit = false;
    real corr = src ? source_sum(I, CA, i, j, k, n, hit) : real(0);
    if (disp) {
        const long long di =
            ((long long)(k - I.dlo[2]) * I.dn[1] + (j - I.dlo[1])) * I.dn[0] + (i - I.dlo[0]);
        for (int p = 0; p < I.n_poles; ++p) {
            real* pp = I.P + ((long long)(p * 2 + 0) * 3 + CA) * I.dvol + di;
            real* pm = I.P + ((long long)(p * 2 + 1) * 3 + CA) * I.dvol + di;
            const real pn = *pp, pq = *pm;
            const real pnew = I.A[p] * pn + I.B[p] * pq + ldg(cf, 3 + 3 * p + CA) * e_old;
            corr += pnew - pn;
            if (store) {
                *pm = pn;
                *pp = pnew;
            }
        }
        hit = true;
    }
    if (hit) e = fma(-ldg(cf, CA), corr, e);
    return e;
}

// Slab axes a tile's footprint touches (bit a = axis a): the same footprint
// test as the host's plain box.
template <typename real>
__device__ __forceinline__ int tile_slab_mask(const InstDev<real>& I, int i0, int j0, int z0, int z1) {
    int m = 0;
    if (!(max(i0 - 1, 0) >= I.pl[0] && min(i0 + LX, I.nx) - 1 < I.nx - I.ph[0])) m |= 1;
    if (!(max(j0 - 1, 0) >= I.pl[1] && min(j0 + LY, I.ny) - 1 < I.ny - I.ph[1])) m |= 2;
    if (!(max(z0 - 1, 0) >= I.pl[2] && z1 - 1 < I.nz - I.ph[2])) m |= 4;
    return m;
}

// Tile update with CPML on the axes in MASK (runtime per-cell flags inside)
// and, with EXTRAS, sources and polarisations.  The x and y profile values of
// the column are loaded once; z values once per plane.
template <typename real, int ZB, int MASK, bool EXTRAS>
__device__ __forceinline__ void tile_block(const InstDev<real>& I, int tx, int ty, int tz, long long n, int cur,
                                           bool dry) {
    constexpr bool SX = (MASK & 1) != 0, SY = (MASK & 2) != 0, SZ = (MASK & 4) != 0;
    const int i = tx * LX + threadIdx.x, j = ty * LY + threadIdx.y;
    const int z0 = tz * ZB, z1 = min(I.nz, z0 + ZB);
    if (i >= I.nx || j >= I.ny) return;

    const int nx = I.nx, ny = I.ny, nz = I.nz;
    const long long px = I.px, plane = I.plane, vol = I.vol;
    const real* eX = I.F[cur][0];
    const real* eY = I.F[cur][1];
    const real* eZ = I.F[cur][2];
    const real* hX = I.F[cur][3];
    const real* hY = I.F[cur][4];
    const real* hZ = I.F[cur][5];
    real* oEX = I.F[cur ^ 1][0];
    real* oEY = I.F[cur ^ 1][1];
    real* oEZ = I.F[cur ^ 1][2];
    real* oHX = I.F[cur ^ 1][3];
    real* oHY = I.F[cur ^ 1][4];
    real* oHZ = I.F[cur ^ 1][5];
    // psi of axis a: slot p at psi[a] + p * vol (H side ping-pong, E side in place)
    const real* hiX = SX ? I.psiH[cur][0] : nullptr;
    const real* hiY = SY ? I.psiH[cur][1] : nullptr;
    const real* hiZ = SZ ? I.psiH[cur][2] : nullptr;
    real* hoX = SX ? I.psiH[cur ^ 1][0] : nullptr;
    real* hoY = SY ? I.psiH[cur ^ 1][1] : nullptr;
    real* hoZ = SZ ? I.psiH[cur ^ 1][2] : nullptr;
    real* peX = SX ? I.psiE[0] : nullptr;
    real* peY = SY ? I.psiE[1] : nullptr;
    real* peZ = SZ ? I.psiE[2] : nullptr;

    const bool xm = i > 0, ym = j > 0, xp = i + 1 < nx, yp = j + 1 < ny;
    // CPML slab membership of the own cell and of the two recomputed neighbours
    const bool xo = SX && in_slab(I, 0, i), xo_m = SX && xm && in_slab(I, 0, i - 1);
    const bool yo = SY && in_slab(I, 1, j), yo_m = SY && ym && in_slab(I, 1, j - 1);
    // profiles (b, c) at integer (i) and half-integer (h) points of the column
    real bxi = 1, cxi = 0, bxh = 1, cxh = 0, bxhm = 1, cxhm = 0;
    real byi = 1, cyi = 0, byh = 1, cyh = 0, byhm = 1, cyhm = 0;
    if (SX) {
        const real* pr = I.prof[0];
        if (xo) bxi = ldg(pr, i), cxi = ldg(pr, nx + i), bxh = ldg(pr, 2 * nx + i), cxh = ldg(pr, 3 * nx + i);
        if (xo_m) bxhm = ldg(pr, 2 * nx + i - 1), cxhm = ldg(pr, 3 * nx + i - 1);
    }
    if (SY) {
        const real* pr = I.prof[1];
        if (yo) byi = ldg(pr, j), cyi = ldg(pr, ny + j), byh = ldg(pr, 2 * ny + j), cyh = ldg(pr, 3 * ny + j);
        if (yo_m) byhm = ldg(pr, 2 * ny + j - 1), cyhm = ldg(pr, 3 * ny + j - 1);
    }
    // sources touching this column's footprint (own, x-1 and y-1 cells)
    unsigned smask = 0;
    if (EXTRAS)
        for (int q = 0; q < I.n_src; ++q) {
            const SrcDev<real>& sv = I.src[q];
            if (sv.lo[0] <= i && sv.lo[0] + sv.n[0] > i - 1 && sv.lo[1] <= j && sv.lo[1] + sv.n[1] > j - 1)
                smask |= 1u << q;
        }

    int k = z0 > 0 ? z0 - 1 : 0;
    long long o = (long long)k * plane + (long long)j * px + i;
    // E^n of plane k carried between iterations: own Ex, Ey; Ex at (i-1); Ey at (j-1)
    real ex_c = ldg(eX, o), ey_c = ldg(eY, o);
    real exm_c = ldz(eX, o - 1, xm), eym_c = ldz(eY, o - px, ym);
    real hxp = 0, hyp = 0;  // H^{n+1/2} of plane k-1 at the own cell
    for (; k < z1; ++k, o += plane) {
        const bool kp = k + 1 < nz;
        const bool store = k >= z0;
        const bool zo = SZ && (k < I.pl[2] || k >= nz - I.ph[2]);
        real bzi = 1, czi = 0, bzh = 1, czh = 0;
        if (zo) {
            const real* pr = I.prof[2];
            bzi = ldg(pr, k), czi = ldg(pr, nz + k), bzh = ldg(pr, 2 * nz + k), czh = ldg(pr, 3 * nz + k);
        }
        bool src = false;
        if (EXTRAS)
            for (unsigned m = smask; m; m &= m - 1) {
                const SrcDev<real>& sv = I.src[__ffs(m) - 1];
                if (k >= sv.lo[2] && k < sv.lo[2] + sv.n[2]) src = true;
            }
        const real ex_n = ldz(eX, o + plane, kp), ey_n = ldz(eY, o + plane, kp);
        const real exm_n = ldz(eX, o + plane - 1, kp && xm), eym_n = ldz(eY, o + plane - px, kp && ym);
        const real ez = ldg(eZ, o);
        const real ez_xp = ldz(eZ, o + 1, xp), ez_yp = ldz(eZ, o + px, yp);
        const real ey_xp = ldz(eY, o + 1, xp), ex_yp = ldz(eX, o + px, yp);
        const bool sp = store && !dry;

        // H^{n+1/2} at the own cell (stored) ...
        real hx, hy, hz;
        {
            const real d1 = ez_yp - ez, d2 = ey_n - ey_c;
            real cv = d1 - d2;
            pml_term<SY, true, true>(cv, yo, byh, cyh, d1, hiY, hoY, o, sp);
            pml_term<SZ, false, true>(cv, zo, bzh, czh, d2, hiZ, hoZ, o, sp);
            hx = h_new<EXTRAS>(I, 3, cv, ldg(hX, o), src, i, j, k, n);
        }
        {
            const real d1 = ex_n - ex_c, d2 = ez_xp - ez;
            real cv = d1 - d2;
            pml_term<SZ, true, true>(cv, zo, bzh, czh, d1, hiZ + vol, hoZ + vol, o, sp);
            pml_term<SX, false, true>(cv, xo, bxh, cxh, d2, hiX, hoX, o, sp);
            hy = h_new<EXTRAS>(I, 4, cv, ldg(hY, o), src, i, j, k, n);
        }
        {
            const real d1 = ey_xp - ey_c, d2 = ex_yp - ex_c;
            real cv = d1 - d2;
            pml_term<SX, true, true>(cv, xo, bxh, cxh, d1, hiX + vol, hoX + vol, o, sp);
            pml_term<SY, false, true>(cv, yo, byh, cyh, d2, hiY + vol, hoY + vol, o, sp);
            hz = h_new<EXTRAS>(I, 5, cv, ldg(hZ, o), src, i, j, k, n);
        }
        if (store) {
            const real ez_xm = ldz(eZ, o - 1, xm), ez_ym = ldz(eZ, o - px, ym);
            const real ex_xmyp = ldz(eX, o - 1 + px, xm && yp), ey_xpym = ldz(eY, o + 1 - px, xp && ym);
            const real ex_ym = ldz(eX, o - px, ym), ey_xm = ldz(eY, o - 1, xm);
            // ... and, recomputed (psi read only), at (i-1, j) [Hy, Hz] and (i, j-1) [Hx, Hz]
            real hy_xm = 0, hz_xm = 0, hx_ym = 0, hz_ym = 0;
            if (xm) {
                const long long om = o - 1;
                {
                    const real d1 = exm_n - exm_c, d2 = ez - ez_xm;
                    real cv = d1 - d2;
                    pml_term<SZ, true, true>(cv, zo, bzh, czh, d1, hiZ + vol, hoZ + vol, om, false);
                    pml_term<SX, false, true>(cv, xo_m, bxhm, cxhm, d2, hiX, hoX, om, false);
                    hy_xm = h_new<EXTRAS>(I, 4, cv, ldg(hY, om), src, i - 1, j, k, n);
                }
                {
                    const real d1 = ey_c - ey_xm, d2 = ex_xmyp - exm_c;
                    real cv = d1 - d2;
                    pml_term<SX, true, true>(cv, xo_m, bxhm, cxhm, d1, hiX + vol, hoX + vol, om, false);
                    pml_term<SY, false, true>(cv, yo, byh, cyh, d2, hiY + vol, hoY + vol, om, false);
                    hz_xm = h_new<EXTRAS>(I, 5, cv, ldg(hZ, om), src, i - 1, j, k, n);
                }
            }
            if (ym) {
                const long long om = o - px;
                {
                    const real d1 = ez - ez_ym, d2 = eym_n - eym_c;
                    real cv = d1 - d2;
                    pml_term<SY, true, true>(cv, yo_m, byhm, cyhm, d1, hiY, hoY, om, false);
                    pml_term<SZ, false, true>(cv, zo, bzh, czh, d2, hiZ, hoZ, om, false);
                    hx_ym = h_new<EXTRAS>(I, 3, cv, ldg(hX, om), src, i, j - 1, k, n);
                }
                {
                    const real d1 = ey_xpym - eym_c, d2 = ex_c - ex_ym;
                    real cv = d1 - d2;
                    pml_term<SX, true, true>(cv, xo, bxh, cxh, d1, hiX + vol, hoX + vol, om, false);
                    pml_term<SY, false, true>(cv, yo_m, byhm, cyhm, d2, hiY + vol, hoY + vol, om, false);
                    hz_ym = h_new<EXTRAS>(I, 5, cv, ldg(hZ, om), src, i, j - 1, k, n);
                }
            }
            oHX[o] = hx;
            oHY[o] = hy;
            oHZ[o] = hz;
            // E^{n+1} at the own cell
            const int cb = __ldg(I.combo + o);
            const real* cf = I.coef + cb * I.ncoef;
            const bool disp = EXTRAS && (__ldg(I.cflag + cb) & 1) != 0;
            const bool si = !dry;
            {
                const real d1 = hz - hz_ym, d2 = hy - hyp;
                real cv = d1 - d2;
                pml_term<SY, true, false>(cv, yo, byi, cyi, d1, peY, peY, o, si);
                pml_term<SZ, false, false>(cv, zo, bzi, czi, d2, peZ, peZ, o, si);
                oEX[o] = e_new<EXTRAS, 0>(I, i, j, k, n, cf, disp, ex_c, cv, si, src);
            }
            {
                const real d1 = hx - hxp, d2 = hz - hz_xm;
                real cv = d1 - d2;
                pml_term<SZ, true, false>(cv, zo, bzi, czi, d1, peZ + vol, peZ + vol, o, si);
                pml_term<SX, false, false>(cv, xo, bxi, cxi, d2, peX, peX, o, si);
                oEY[o] = e_new<EXTRAS, 1>(I, i, j, k, n, cf, disp, ey_c, cv, si, src);
            }
            {
                const real d1 = hy - hy_xm, d2 = hx - hx_ym;
                real cv = d1 - d2;
                pml_term<SX, true, false>(cv, xo, bxi, cxi, d1, peX + vol, peX + vol, o, si);
                pml_term<SY, false, false>(cv, yo, byi, cyi, d2, peY + vol, peY + vol, o, si);
                oEZ[o] = e_new<EXTRAS, 2>(I, i, j, k, n, cf, disp, ez, cv, si, src);
            }
        }
        hxp = hx;
        hyp = hy;
        ex_c = ex_n;
        ey_c = ey_n;
        exm_c = exm_n;
        eym_c = eym_n;
    }
}

// Monitors (every save_span steps, before the step) and running DFT sums, read
// from buffer `cur`, which no stepping block writes during the launch.
template <typename real>
__device__ __forceinline__ void lean_probe_block(const InstDev<real>& I, long long chunk, long long n, int buf, DevState* st) {
    __shared__ double2 ph[2][LMAXF];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y;
    const double dt = I.dt;
    for (int f = tid; f < I.n_freq; f += nthr) {
        double s, c;
        const double fr = I.freqs[f];
        sincospi(2.0 * fr * ((double)n * dt), &s, &c);
        ph[0][f] = make_double2(c * dt, s * dt);
        sincospi(2.0 * fr * (((double)n - 0.5) * dt), &s, &c);
        ph[1][f] = make_double2(c * dt, s * dt);
    }
    __syncthreads();
    const long long p = chunk * nthr + tid;
    if (p >= I.n_probe) return;
    const int comp = I.probe_comp[p];
    const real* F = I.F[buf][comp];
    double v = 0.0;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const long long idx = I.probe_idx[8 * p + m];
        if (idx >= 0) v += I.probe_w[8 * p + m] * (double)F[idx];
    }
    const int ms = I.probe_mon[p];
    if (ms >= 0 && (n % I.save_span) == 0) {
        const long long s = n / I.save_span;
        if (s < I.mon_cap)
            I.mon[s * I.n_mon + ms] = v;
        else
            st->status = SJ_E_RANGE;
    }
    const int ds = I.probe_dft[p];
    if (ds >= 0) {
        double2* row = I.dft + (long long)ds * I.n_freq;
        const double2* pf = ph[comp >= 3 ? 1 : 0];
        for (int f = 0; f < I.n_freq; ++f) {
            double2 a = row[f];
            a.x += v * pf[f].x;
            a.y += v * pf[f].y;
            row[f] = a;
        }
    }
}

__device__ __forceinline__ int lean_find(const long long* pre, int n, long long b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// The instance descriptors travel in the launch's parameter space
// (__grid_constant__): every block reads them through the constant cache with
// block-uniform indices, so field pointers, extents and coefficients live in
// uniform registers instead of taking per-thread registers, which a
// descriptor table in global memory would.

// Every block of every launch of a step counts itself; the last one (of
// step_blocks) advances the step and flips the buffers.  The launches of a
// step may run concurrently: each block reads `cur` before it counts, so no
// block can see the flip of its own step.
template <typename real, int K>
__device__ __forceinline__ void finish_block(const LeanTable<real, K>& tab, DevState* st) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&st->done, 1u);
        if (prev == tab.step_blocks - 1) {
            if (!tab.dry) {
                st->step += 1;
                st->cur ^= 1;
            }
            st->done = 0;
            __threadfence();
        }
    }
}

// Plain tiles: block -> tile of the instance's plain box; tiles whose
// footprint holds a source or dispersive voxel are left to k_lean_general.
template <typename real, int ZB, int K>
__global__ void __launch_bounds__(LX * LY, plain_minb<real>())
k_lean_plain(const __grid_constant__ LeanTable<real, K> tab, DevState* st) {
    const int cur = st->cur;
    const long long b = blockIdx.x;
    const int ii = K == 1 ? 0 : lean_find(tab.plain_pre, tab.n_inst, b);
    const InstDev<real>& I = tab.inst[ii];
    const int* bx = tab.box[ii];
    const int bnx = bx[1] - bx[0], bny = bx[3] - bx[2];
    const long long local = b - tab.plain_pre[ii];
    const int tx = bx[0] + (int)(local % bnx);
    const int ty = bx[2] + (int)((local / bnx) % bny);
    const int tz = bx[4] + (int)(local / ((long long)bnx * bny));
    const int z0 = tz * ZB;
    // plain_block returns early for columns outside the grid; every thread
    // still reaches the barrier in finish_block
    if (!tile_has_extras(I, tx * LX, ty * LY, z0, min(I.nz, z0 + ZB))) plain_block<real, ZB>(I, tx, ty, tz, cur);
    finish_block(tab, st);
}

// Tile of block b among all tiles of an instance (x fastest, then y, z).
template <typename real>
__device__ __forceinline__ void tile_of(const InstDev<real>& I, long long local, int& tx, int& ty, int& tz) {
    const int ntx = (I.nx + LX - 1) / LX, nty = (I.ny + LY - 1) / LY;
    tx = (int)(local % ntx);
    ty = (int)((local / ntx) % nty);
    tz = (int)(local / ((long long)ntx * nty));
}

// Single-slab tiles: the footprint touches the slabs of exactly one axis and
// holds no source or dispersive voxel.  Every tile gets a block; the others
// only count themselves.
template <typename real, int ZB, int K>
__global__ void __launch_bounds__(LX * LY, slab_minb<real>())
k_lean_slab(const __grid_constant__ LeanTable<real, K> tab, DevState* st) {
    const int cur = st->cur;
    const long long b = blockIdx.x;
    const int ii = K == 1 ? 0 : lean_find(tab.item_pre, tab.n_inst, b);
    const InstDev<real>& I = tab.inst[ii];
    int tx, ty, tz;
    tile_of(I, b - tab.item_pre[ii], tx, ty, tz);
    const int z0 = tz * ZB, z1 = min(I.nz, z0 + ZB);
    const int m = tile_slab_mask(I, tx * LX, ty * LY, z0, z1);
    if ((m == 1 || m == 2 || m == 4) && !tile_has_extras(I, tx * LX, ty * LY, z0, z1)) {
        if (m == 1)
            tile_block<real, ZB, 1, false>(I, tx, ty, tz, 0, cur, tab.dry != 0);
        else if (m == 2)
            tile_block<real, ZB, 2, false>(I, tx, ty, tz, 0, cur, tab.dry != 0);
        else
            tile_block<real, ZB, 4, false>(I, tx, ty, tz, 0, cur, tab.dry != 0);
    }
    finish_block(tab, st);
}

// General tiles (several slab axes, or a source or dispersive voxel in the
// footprint), then the probe blocks.
template <typename real, int ZB, int K>
__global__ void __launch_bounds__(LX * LY, general_minb<real>())
k_lean_general(const __grid_constant__ LeanTable<real, K> tab, DevState* st) {
    const long long n = st->step;
    const int cur = st->cur;
    const long long b = blockIdx.x;
    if (b < tab.n_items) {
        const int ii = K == 1 ? 0 : lean_find(tab.item_pre, tab.n_inst, b);
        const InstDev<real>& I = tab.inst[ii];
        int tx, ty, tz;
        tile_of(I, b - tab.item_pre[ii], tx, ty, tz);
        const int z0 = tz * ZB, z1 = min(I.nz, z0 + ZB);
        const int m = tile_slab_mask(I, tx * LX, ty * LY, z0, z1);
        const bool ext = tile_has_extras(I, tx * LX, ty * LY, z0, z1);
        // tile_block returns early for columns outside the grid; every
        // thread still reaches the barrier below
        if (ext || (m != 0 && m != 1 && m != 2 && m != 4))
            tile_block<real, ZB, 7, true>(I, tx, ty, tz, n, cur, tab.dry != 0);
    } else if (!tab.dry) {
        const long long pb = b - tab.n_items;
        const int ii = K == 1 ? 0 : lean_find(tab.probe_pre, tab.n_inst, pb);
        lean_probe_block<real>(tab.inst[ii], pb - tab.probe_pre[ii], n, cur, st);
    }
    finish_block(tab, st);
}

long long lean_items(int nx, int ny, int nz, int zb) {
    return (long long)((nx + LX - 1) / LX) * ((ny + LY - 1) / LY) * ((nz + zb - 1) / zb);
}

namespace {

// Tiles [t0, t1) along one axis whose footprint [max(lo-1, 0), min(lo+w, n)-1]
// (lo = t*w) stays clear of both CPML slabs [0, pl) and [n-ph, n).
void clear_range(int n, int w, int pl, int ph, int* t0, int* t1) {
    const int nt = (n + w - 1) / w;
    int a = nt, b = 0;
    for (int t = 0; t < nt; ++t) {
        const int lo = std::max(t * w - 1, 0), hi = std::min(t * w + w, n) - 1;
        if (lo >= pl && hi < n - ph) {
            a = std::min(a, t);
            b = t + 1;
        }
    }
    if (a >= b) a = b = 0;
    *t0 = a;
    *t1 = b;
}

template <typename real, int K>
void fill_table(LeanTable<real, K>& t, const InstDev<real>* h, int n, int zb, int dry) {
    t.n_inst = n;
    t.dry = dry;
    t.step_blocks = 0;
    t.item_pre[0] = 0;
    t.plain_pre[0] = 0;
    t.probe_pre[0] = 0;
    for (int q = 0; q < n; ++q) {
        const InstDev<real>& I = h[q];
        t.inst[q] = I;
        int* bx = t.box[q];
        clear_range(I.nx, LX, I.pl[0], I.ph[0], bx + 0, bx + 1);
        clear_range(I.ny, LY, I.pl[1], I.ph[1], bx + 2, bx + 3);
        clear_range(I.nz, zb, I.pl[2], I.ph[2], bx + 4, bx + 5);
        const long long plain = (long long)(bx[1] - bx[0]) * (bx[3] - bx[2]) * (bx[5] - bx[4]);
        if (plain == 0) bx[0] = bx[1] = bx[2] = bx[3] = bx[4] = bx[5] = 0;
        t.item_pre[q + 1] = t.item_pre[q] + lean_items(I.nx, I.ny, I.nz, zb);
        t.plain_pre[q + 1] = t.plain_pre[q] + plain;
        t.probe_pre[q + 1] = t.probe_pre[q] + (I.n_probe + LX * LY - 1) / (LX * LY);
    }
    t.n_items = t.item_pre[n];
    t.any_slab = 0;
    for (int q = 0; q < n; ++q)
        for (int a = 0; a < 3; ++a) t.any_slab |= (h[q].pl[a] + h[q].ph[a]) > 0;
}

template <typename real, int K>
long long table_blocks(const LeanTable<real, K>& t) {
    const long long pb = t.dry ? 0 : t.plain_pre[t.n_inst];
    return pb + (t.any_slab ? t.n_items : 0) + t.n_items + t.probe_pre[t.n_inst];
}

// General tiles on the main stream, single-slab and plain tiles on the two
// side streams: the three kernels of a step overlap, filling each other's
// tails.
template <typename real, int K>
cudaError_t launch_table(const LeanTable<real, K>& t, int zb, DevState* st, const LeanStreams& ls) {
    const unsigned pblocks = t.dry ? 0u : (unsigned)t.plain_pre[t.n_inst];
    const unsigned sblocks = t.any_slab ? (unsigned)t.n_items : 0u;
    const unsigned gblocks = (unsigned)(t.n_items + t.probe_pre[t.n_inst]);
    const dim3 block(LX, LY);
    cudaStream_t ss = ls.side[0] ? ls.side[0] : ls.main;
    cudaStream_t sp = ls.side[1] ? ls.side[1] : ls.main;
#define SJ_ZB(Z)                                                                        \
    case Z:                                                                             \
        k_lean_general<real, Z, K><<<gblocks, block, 0, ls.main>>>(t, st);              \
        if (sblocks) k_lean_slab<real, Z, K><<<sblocks, block, 0, ss>>>(t, st);         \
        if (pblocks) k_lean_plain<real, Z, K><<<pblocks, block, 0, sp>>>(t, st);        \
        break;
    switch (zb) {  // z-segment length
        SJ_ZB(8)
        SJ_ZB(16)
        SJ_ZB(32)
        SJ_ZB(64)
        default: return cudaErrorInvalidValue;
    }
#undef SJ_ZB
    return cudaGetLastError();
}

}  // namespace

template <typename real>
int lean_launches(const InstDev<real>* h_insts, int n_inst, int zb) {
    int total = 0;
    for (int q0 = 0; q0 < n_inst; q0 += LEAN_TAB) {
        const int m = std::min(LEAN_TAB, n_inst - q0);
        static thread_local LeanTable<real, LEAN_TAB> t;
        fill_table(t, h_insts + q0, m, zb, 0);
        total += (t.plain_pre[m] > 0) + (t.any_slab != 0) + 1;
    }
    return total;
}
template int lean_launches<float>(const InstDev<float>*, int, int);
template int lean_launches<double>(const InstDev<double>*, int, int);

template <typename real>
cudaError_t launch_lean_step(const InstDev<real>* h_insts, int n_inst, int zb, int dry, DevState* st,
                             const LeanStreams& ls) {
    cudaError_t e = cudaSuccess;
    const bool fork = ls.side[0] && ls.side[1];
    if (fork) {
        e = cudaEventRecord(ls.fork, ls.main);
        for (int q = 0; q < 2 && e == cudaSuccess; ++q) e = cudaStreamWaitEvent(ls.side[q], ls.fork, 0);
        if (e != cudaSuccess) return e;
    }
    if (n_inst == 1) {
        LeanTable<real, 1> t;
        fill_table(t, h_insts, 1, zb, dry);
        t.step_blocks = (unsigned)table_blocks(t);
        e = launch_table(t, zb, st, ls);
    } else {
        // 29 KB parameter blocks: kept off the stack, one set per host thread
        static thread_local std::vector<LeanTable<real, LEAN_TAB>> tabs;
        const int nc = (n_inst + LEAN_TAB - 1) / LEAN_TAB;
        if ((int)tabs.size() < nc) tabs.resize(nc);
        long long total = 0;
        for (int c = 0; c < nc; ++c) {
            const int q0 = c * LEAN_TAB, m = std::min(LEAN_TAB, n_inst - q0);
            fill_table(tabs[c], h_insts + q0, m, zb, dry);
            total += table_blocks(tabs[c]);
        }
        for (int c = 0; c < nc && e == cudaSuccess; ++c) {
            tabs[c].step_blocks = (unsigned)total;
            e = launch_table(tabs[c], zb, st, ls);
        }
    }
    if (fork) {
        for (int q = 0; q < 2 && e == cudaSuccess; ++q) {
            e = cudaEventRecord(ls.join[q], ls.side[q]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ls.main, ls.join[q], 0);
        }
    }
    return e;
}

template cudaError_t launch_lean_step<double>(const InstDev<double>*, int, int, int, DevState*, const LeanStreams&);
template cudaError_t launch_lean_step<float>(const InstDev<float>*, int, int, int, DevState*, const LeanStreams&);
}  // namespace sj
