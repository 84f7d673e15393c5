// Fused single-pass leapfrog stepper (the "fused" schedule, default for FP32).
//
// One step reads E^n, H^{n-1/2} (ping-pong buffer `cur`) and writes
// H^{n+1/2}, E^{n+1} (buffer cur^1): each field component crosses HBM once in
// and once out per step.
//
// A block takes a tile of 32 x 8 (i, j) columns and marches along z over a
// segment of ZB planes; a segment starting at z0 > 0 first updates H of
// plane z0-1 (owned by the previous segment) without storing it.  The E
// update at (i, j, k) needs H of the cells at x-1 and y-1, which other
// threads (or other tiles) own; how a kernel gets them depends on the tile
// class.  The ping-pong buffers (fields and H-side CPML psi) keep every
// variant race-free: nothing a block reads is written during the step.
//
// The host sorts the tiles into one list per class, by what a tile's
// footprint (own cells and the x-1/y-1/z-1 neighbours) touches:
//   plain   (k_lean_plain2 / k_lean_plain): no CPML slab and no H source.
//           Where rows are whole (nx % 32 == 0): the two-column shared-halo
//           body below with no CPML axis; otherwise one column per thread
//           recomputing the x-1 and y-1 H from L1/L2.
//   slab    (k_lean_slab2 / k_lean_slab): the CPML slabs of one axis; multi
//           (k_lean_multi2 / k_lean_multi): of two or three.  Shared halo:
//           warps for the row below the tile and the column left of it
//           update H only; x-1 H comes by shuffle, y-1 H through a
//           double-buffered shared plane (one barrier per plane).  Two
//           columns per thread in FP32 where rows are whole (5 warps per
//           tile: 4 of row pairs, 1 of halo), else one (10 warps: 8 rows,
//           2 halo).
//           Compiled per axis set, so the other axes' terms vanish.
//   general (k_lean_general): an H source in the footprint; also runs the
//           probe blocks, and its blocks (the only ones that read the step
//           counter) count themselves: the last advances the step.
// Instances with the same grid, CPML and coefficient table form a group
// (LeanGroup) whose arrays sit at fixed strides: one launch per class covers
// the group's tiles (blockIdx.y = member).  The launches of a step go to
// streams forked from the caller's, one per class and group set, so they
// overlap; after they join, small correction kernels add the E sources and
// the polarisation ADE on their cells only.  All evaluate one update
// formula, so a voxel's result does not depend on which kernel (or which
// tiling) updated it:
//   H^{n+1/2} = fma(-S, curl E, H^{n-1/2}) [- dt J_H]
//   E^{n+1}   = fma(S ε∞⁻¹, curl H, E^n)
//               [then fma(-ε∞⁻¹, dt J_s, ·) per E source s, in order]
//               [then fma(-ε∞⁻¹, Σ_p (P_p^{n+1} - P_p^n), ·)]
// with curl including the CPML ψ terms.  This file is compiled with
// contraction off (-fmad=false): every fused multiply-add is the explicit
// one written here.
#include <algorithm>
#include <vector>

#include "sj_physics.cuh"

namespace sj {

constexpr int LX = 32, LY = 8;      // tile of columns per block
constexpr int FIX_THREADS = 256;    // cells per block of the correction kernels
constexpr int LMAXF = 256;

// resident blocks per SM each kernel is compiled for (register budget)
#ifndef SJ_LEAN_PLAIN_MINB
#define SJ_LEAN_PLAIN_MINB 5
#endif
#ifndef SJ_LEAN_PAIR_PLAIN_MINB
#define SJ_LEAN_PAIR_PLAIN_MINB 8
#endif
#ifndef SJ_LEAN_SLAB_MINB
#define SJ_LEAN_SLAB_MINB 4
#endif
#ifndef SJ_LEAN_MULTI_MINB
#define SJ_LEAN_MULTI_MINB 3
#endif
#ifndef SJ_LEAN_GEN_MINB
#define SJ_LEAN_GEN_MINB 2
#endif
template <typename real>
constexpr int plain_minb() { return sizeof(real) == 4 ? SJ_LEAN_PLAIN_MINB : 3; }
// the two-column plain kernel's 160-thread blocks
template <typename real>
constexpr int pair_plain_minb() { return sizeof(real) == 4 ? SJ_LEAN_PAIR_PLAIN_MINB : 2; }

template <typename real>
constexpr int slab_minb() { return sizeof(real) == 4 ? SJ_LEAN_SLAB_MINB : 2; }
template <typename real>
constexpr int multi_minb() { return sizeof(real) == 4 ? SJ_LEAN_MULTI_MINB : 2; }
template <typename real>
constexpr int general_minb() { return sizeof(real) == 4 ? SJ_LEAN_GEN_MINB : 1; }

// Reads of buffer `cur` (fields, H-side psi), profiles and material tables
// go through the non-coherent path: nothing writes them during the step, and
// the compiler may then move them ahead of the stores of the previous plane.
// L2 prefetch distance (planes): each warp (one 32-column row of a tile)
// asks the TMA unit to bring the row of plane k + LEAN_PF of every array the
// step reads into L2, one row per lane, so the loads of that plane find it
// there.
#ifndef SJ_LEAN_PF
#define SJ_LEAN_PF 1
#endif
constexpr int LEAN_PF = SJ_LEAN_PF;

// `bytes` at p into L2 when on: one predicated instruction, no branch (rows
// are 16-byte aligned: they start on 128-byte boundaries of padded rows)
__device__ __forceinline__ void prefetch_if(const void* p, unsigned bytes, bool on) {
    asm volatile(
        "{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q cp.async.bulk.prefetch.L2.global [%0], %1;\n\t}" ::"l"(p),
        "r"(bytes), "r"((unsigned)on));
}

// Element offsets within an instance are 32-bit (the host rejects grids
// whose two-slot psi arrays would not fit): one wide multiply-add per
// address.
template <typename real>
__device__ __forceinline__ real ldg(const real* p, unsigned o) {
    return __ldg(p + o);
}
template <typename real>
__device__ __forceinline__ real ldz(const real* p, unsigned o, bool ok) {
    return ok ? __ldg(p + o) : real(0);
}

__host__ __device__ inline int imax(int a, int b) { return a > b ? a : b; }
__host__ __device__ inline int imin(int a, int b) { return a < b ? a : b; }

// Does the tile's footprint (own cells and the x-1 / y-1 / z-1 neighbours
// whose H it recomputes) touch an H source?  E sources and polarisations
// are applied after the tile kernels (k_lean_esrc, k_lean_disp), so only H
// sources, which the E update of the same pass reads, need the general
// kernel.  Block-uniform.
template <typename real>
__host__ __device__ inline bool tile_has_hsource(const InstDev<real>& I, int i0, int j0, int z0, int z1) {
    const int xa = imax(i0 - 1, 0), xb = imin(i0 + LX, I.nx) - 1;
    const int ya = imax(j0 - 1, 0), yb = imin(j0 + LY, I.ny) - 1;
    const int za = imax(z0 - 1, 0), zb = z1 - 1;
    for (int q = 0; q < I.n_src; ++q) {
        const SrcDev<real>& sv = I.src[q];
        if (sv.comp >= 3 && sv.lo[0] <= xb && sv.lo[0] + sv.n[0] > xa && sv.lo[1] <= yb &&
            sv.lo[1] + sv.n[1] > ya && sv.lo[2] <= zb && sv.lo[2] + sv.n[2] > za)
            return true;
    }
    return false;
}

// Does the tile own a cell of the design region (adjoint)?  Those cells
// scale by their own eps^-1, which only the general kernel applies.
template <typename real>
__host__ __device__ inline bool tile_has_design(const InstDev<real>& I, int i0, int j0, int z0, int z1) {
    if (!I.dinv) return false;
    return i0 < I.des_lo[0] + I.des_n[0] && i0 + LX > I.des_lo[0] && j0 < I.des_lo[1] + I.des_n[1] &&
           j0 + LY > I.des_lo[1] && z0 < I.des_lo[2] + I.des_n[2] && z1 > I.des_lo[2];
}

// Does the tile's footprint or its z+1 plane reach a face of the grid?
template <typename real>
__host__ __device__ inline bool tile_edge(const InstDev<real>& I, int tx, int ty, int tz, int zb) {
    const int i0 = tx * LX, j0 = ty * LY, z1 = imin(I.nz, (tz + 1) * zb);
    return !(i0 > 0 && i0 + LX < I.nx && j0 > 0 && j0 + LY < I.ny && z1 < I.nz);
}

// The rows a column march prefetches into L2, LEAN_PF planes ahead, spread
// one row per lane (a single predicated instruction per warp and plane):
// lanes 0-5 the six field components, 6 the combo bytes, then four rows per
// CPML axis the tile's row uses (the two psi slots of H and of E), axes in
// x, y, z order and packed: x when the tile touches an x slab, y when the
// row is in a y slab, z (only on planes in a z slab) in any tile with SZ.
// At most 19 rows, so a 16-lane half-warp covers every single- and
// two-axis tile.  A lane's row is one word: the array's address (16-byte
// aligned) with bit 0 set for a z psi row and bit 1 for a byte array; 0 =
// no row.  The word waits in a shared-memory slot of the thread and is
// reloaded on every plane, so it holds no register across the march.  The
// element offset a row is prefetched at is a field offset; psi rows add qf
// (a group member's psi sits twice as far from the lead's as its fields).
template <typename real, bool SX, bool SY, bool SZ>
__device__ __forceinline__ unsigned long long lane_row(const InstDev<real>& I, int l, bool xt, bool yt,
                                                       unsigned qf = 0) {
    if (l < 6) return (unsigned long long)I.F[0][l];
    if (l == 6) return (unsigned long long)I.combo | 2ull;
    int m = l - 7;  // index among the psi rows in use
    for (int a = 0; a < 3; ++a) {
        if (!(a == 0 ? SX && xt : (a == 1 ? SY && yt : SZ))) continue;
        if (m < 4) {
            const real* b = m < 2 ? I.psiH[0][a] : I.psiE[a];
            return (unsigned long long)(b + qf + ((m & 1) ? I.vol : 0)) | (a == 2 ? 1ull : 0ull);
        }
        m -= 4;
    }
    return 0;
}
constexpr int LEAN_PF_SLOTS = LX * (LY + 2);  // threads of the largest tile block
// park the thread's row word; returns its slot
__device__ __forceinline__ volatile unsigned long long* lane_row_park(unsigned long long w) {
    __shared__ unsigned long long slots[LEAN_PF_SLOTS];
    volatile unsigned long long* s = slots + threadIdx.y * blockDim.x + threadIdx.x;
    *s = w;
    return s;
}
// the parked row at element offset r when the plane qualifies (zq: plane
// kq inside a z slab)
template <typename real>
__device__ __forceinline__ void prefetch_lane_row(volatile unsigned long long* slot, unsigned r, bool on, bool zq) {
    const unsigned long long w = *slot;
    const unsigned esz = (w & 2) ? 1u : (unsigned)sizeof(real);
    prefetch_if((const char*)(w & ~3ull) + (size_t)r * esz, 32 * esz, on && w != 0 && (zq || !(w & 1)));
}

// ------------------------------------------------------------- plain tiles
// EDGE = false: the tile's footprint and its z+1 plane stay inside the grid,
// so no load needs a bounds predicate.
template <typename real, int ZB, bool EDGE>
__device__ __forceinline__ void plain_block(const InstDev<real>& I, int tx, int ty, int tz, unsigned qf) {
    const int i = tx * LX + threadIdx.x, j = ty * LY + threadIdx.y;
    const int z0 = tz * ZB, z1 = min(I.nz, z0 + ZB);
    if (EDGE && (i >= I.nx || j >= I.ny)) return;
    const unsigned px = (unsigned)I.px, plane = (unsigned)I.plane;
    const real* eX = I.F[0][0];
    const real* eY = I.F[0][1];
    const real* eZ = I.F[0][2];
    const real* hX = I.F[0][3];
    const real* hY = I.F[0][4];
    const real* hZ = I.F[0][5];
    real* oEX = I.F[1][0];
    real* oEY = I.F[1][1];
    real* oEZ = I.F[1][2];
    real* oHX = I.F[1][3];
    real* oHY = I.F[1][4];
    real* oHZ = I.F[1][5];
    const real S = I.S;
    const bool xm = !EDGE || i > 0, ym = !EDGE || j > 0, xp = !EDGE || i + 1 < I.nx, yp = !EDGE || j + 1 < I.ny;

    int k = z0 > 0 ? z0 - 1 : 0;
    unsigned o = (unsigned)k * plane + (unsigned)j * px + (unsigned)i + qf;  // group member blockIdx.y
    real ex_c = ldg(eX, o), ey_c = ldg(eY, o);
    real exm_c = ldz(eX, o - 1, xm), eym_c = ldz(eY, o - px, ym);
    real hxp = 0, hyp = 0;
    const unsigned orow = o - threadIdx.x;  // row start of this warp at plane k
    const int k0 = k;
    volatile unsigned long long* lr = lane_row_park(lane_row<real, false, false, false>(I, threadIdx.x, false, false));
    for (; k < z1; ++k, o += plane) {
        const bool kp = !EDGE || k + 1 < I.nz;
        if (LEAN_PF > 0)
            prefetch_lane_row<real>(lr, orow + (unsigned)(k + 1 + LEAN_PF - k0) * plane,
                              k + 1 + LEAN_PF < I.nz && k + LEAN_PF < z1, false);
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

// Vector pairs for the two-column tile bodies.
template <typename real>
struct Pair;
template <>
struct Pair<float> {
    using T = float2;
};
template <>
struct Pair<double> {
    using T = double2;
};
template <typename real>
__device__ __forceinline__ typename Pair<real>::T ld2(const real* p, unsigned o) {
    return __ldg(reinterpret_cast<const typename Pair<real>::T*>(p + o));
}
template <typename real>
__device__ __forceinline__ void st2(real* p, unsigned o, real a, real b) {
    typename Pair<real>::T v;
    v.x = a;
    v.y = b;
    *reinterpret_cast<typename Pair<real>::T*>(p + o) = v;
}

constexpr unsigned FULL = 0xffffffffu;

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
// the CPML term with the old psi value po already loaded
template <bool AX, bool ADD, typename real>
__device__ __forceinline__ void pml_term_v(real& cv, bool on, real b, real c, real d, real po, real* pout,
                                           unsigned x, bool store) {
    if (!AX) return;
    // FP64 steps are bound by the FP64 pipe: a warp none of whose active
    // lanes lies in the slab skips the term (z slabs and, for one row per
    // warp, y slabs are warp-uniform); the bits are the same either way
    if (sizeof(real) == 8 && !__any_sync(__activemask(), on)) return;
    // branch-free: predicated store, the term folded in by select; outside
    // the slab cv + (-0) and cv - (+0) leave cv, sign of zero included
    const real ps = fma(b, po, c * d);
    if (on && store) pout[x] = ps;
    cv = ADD ? cv + (on ? ps : real(-0.0)) : cv - (on ? ps : real(0));
}
// old psi of a cell in the slab (predicated load), 0 elsewhere
template <bool AX, bool NC, typename real>
__device__ __forceinline__ real psi_old(bool on, const real* pin, unsigned x) {
    return (AX && on) ? (NC ? __ldg(pin + x) : pin[x]) : real(0);
}
template <bool AX, bool ADD, bool NC, typename real>
__device__ __forceinline__ void pml_term(real& cv, bool on, real b, real c, real d, const real* pin, real* pout,
                                         unsigned x, bool store) {
    pml_term_v<AX, ADD>(cv, on, b, c, d, psi_old<AX, NC>(on, pin, x), pout, x, store);
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

// E^{n+1} of the own cell, Yee and CPML terms (sources and polarisations are
// applied by k_lean_esrc and k_lean_disp after the tile kernels).
// (S eps_inf^-1 comes from the combo's coefficient row)
template <int CA, typename real>
__device__ __forceinline__ real e_new(const InstDev<real>& I, const real* cf, real e_old, real cv) {
    return fma(ldg(cf, I.ncoef - 3 + CA), cv, e_old);
}
// the same with the combo's S eps_inf^-1 already loaded
template <typename real>
__device__ __forceinline__ real e_new_v(real sinv, real e_old, real cv) {
    return fma(sinv, cv, e_old);
}

// Design region (adjoint): the cell's index in the design box, or -1
template <typename real>
__device__ __forceinline__ long long design_index(const InstDev<real>& I, int i, int j, int k) {
    if (!I.dinv) return -1;
    const int u = i - I.des_lo[0], v = j - I.des_lo[1], w = k - I.des_lo[2];
    if ((unsigned)u >= (unsigned)I.des_n[0] || (unsigned)v >= (unsigned)I.des_n[1] ||
        (unsigned)w >= (unsigned)I.des_n[2])
        return -1;
    return ((long long)w * I.des_n[1] + v) * I.des_n[0] + u;
}
// where the E-update bracket of design cell d, component c, at step n is
// recorded while a segment is re-run (null: not recording)
template <typename real>
__device__ __forceinline__ real* design_rec(const InstDev<real>& I, long long d, long long n, int c) {
    if (d < 0 || !I.rec_acc || n < I.rec_t0 || n >= I.rec_t0 + I.rec_len) return nullptr;
    const long long nd = (long long)I.des_n[0] * I.des_n[1] * I.des_n[2];
    return I.rec_acc + ((n - I.rec_t0) * nd + d) * 3 + c;
}
// E^{n+1} in a general tile: a design cell scales by S times its own eps^-1
// and, while recording, keeps the bracket S curl H (the corrections subtract
// the source and polarisation terms from it: the bracket of
// E^{n+1} = E^n + eps^-1 (S curl H - dt J - dP))
template <int CA, bool EXTRAS, typename real>
__device__ __forceinline__ real e_new_g(const InstDev<real>& I, const real* cf, real e_old, real cv, int i, int j,
                                        int k, long long n, bool dry) {
    if (EXTRAS) {
        const long long d = design_index(I, i, j, k);
        if (d >= 0) {
            if (!dry)
                if (real* r = design_rec(I, d, n, CA)) *r = I.S * cv;
            return fma(I.S * I.dinv[d], cv, e_old);
        }
    }
    return e_new<CA>(I, cf, e_old, cv);
}

// Slab axes a tile's footprint touches (bit a = axis a): the same footprint
// test as the host's plain box.
template <typename real>
__host__ __device__ inline int tile_slab_mask(const InstDev<real>& I, int i0, int j0, int z0, int z1) {
    int m = 0;
    if (!(imax(i0 - 1, 0) >= I.pl[0] && imin(i0 + LX, I.nx) - 1 < I.nx - I.ph[0])) m |= 1;
    if (!(imax(j0 - 1, 0) >= I.pl[1] && imin(j0 + LY, I.ny) - 1 < I.ny - I.ph[1])) m |= 2;
    if (!(imax(z0 - 1, 0) >= I.pl[2] && z1 - 1 < I.nz - I.ph[2])) m |= 4;
    return m;
}

// Tile update with CPML on the axes in MASK (runtime per-cell flags inside)
// and, with EXTRAS, H sources.  The x and y profile values of
// the column are loaded once; z values once per plane.
template <typename real, int ZB, int MASK, bool EXTRAS, bool EDGE>
__device__ __forceinline__ void tile_block(const InstDev<real>& I, int tx, int ty, int tz, long long n, bool dry) {
    constexpr bool SX = (MASK & 1) != 0, SY = (MASK & 2) != 0, SZ = (MASK & 4) != 0;
    const int i = tx * LX + threadIdx.x, j = ty * LY + threadIdx.y;
    const int z0 = tz * ZB, z1 = min(I.nz, z0 + ZB);
    if (EDGE && (i >= I.nx || j >= I.ny)) return;

    const int nx = I.nx, ny = I.ny, nz = I.nz;
    const unsigned px = (unsigned)I.px, plane = (unsigned)I.plane, vol = (unsigned)I.vol;
    const real* eX = I.F[0][0];
    const real* eY = I.F[0][1];
    const real* eZ = I.F[0][2];
    const real* hX = I.F[0][3];
    const real* hY = I.F[0][4];
    const real* hZ = I.F[0][5];
    real* oEX = I.F[1][0];
    real* oEY = I.F[1][1];
    real* oEZ = I.F[1][2];
    real* oHX = I.F[1][3];
    real* oHY = I.F[1][4];
    real* oHZ = I.F[1][5];
    // psi of axis a: slot p at psi[a] + p * vol (H side ping-pong, E side in place)
    const real* hiX = SX ? I.psiH[0][0] : nullptr;
    const real* hiY = SY ? I.psiH[0][1] : nullptr;
    const real* hiZ = SZ ? I.psiH[0][2] : nullptr;
    real* hoX = SX ? I.psiH[1][0] : nullptr;
    real* hoY = SY ? I.psiH[1][1] : nullptr;
    real* hoZ = SZ ? I.psiH[1][2] : nullptr;
    real* peX = SX ? I.psiE[0] : nullptr;
    real* peY = SY ? I.psiE[1] : nullptr;
    real* peZ = SZ ? I.psiE[2] : nullptr;

    const bool xm = !EDGE || i > 0, ym = !EDGE || j > 0, xp = !EDGE || i + 1 < nx, yp = !EDGE || j + 1 < ny;
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
    // H sources touching this column's footprint (own, x-1 and y-1 cells)
    unsigned smask = 0;
    if (EXTRAS)
        for (int q = 0; q < I.n_src; ++q) {
            const SrcDev<real>& sv = I.src[q];
            if (sv.comp >= 3 && sv.lo[0] <= i && sv.lo[0] + sv.n[0] > i - 1 && sv.lo[1] <= j &&
                sv.lo[1] + sv.n[1] > j - 1)
                smask |= 1u << q;
        }

    int k = z0 > 0 ? z0 - 1 : 0;
    unsigned o = (unsigned)k * plane + (unsigned)j * px + (unsigned)i;
    // E^n of plane k carried between iterations: own Ex, Ey; Ex at (i-1); Ey at (j-1)
    real ex_c = ldg(eX, o), ey_c = ldg(eY, o);
    real exm_c = ldz(eX, o - 1, xm), eym_c = ldz(eY, o - px, ym);
    real hxp = 0, hyp = 0;  // H^{n+1/2} of plane k-1 at the own cell
    const unsigned orow = o - threadIdx.x;  // row start of this warp at plane k
    const int k0 = k;
    // the x psi rows are prefetched only where the tile touches an x slab
    // (the arrays exist only for axes with slabs)
    const int i0 = tx * LX;
    const bool xt = SX && (max(i0 - 1, 0) < I.pl[0] || min(i0 + LX, nx) - 1 >= nx - I.ph[0]);
    volatile unsigned long long* lr = lane_row_park(lane_row<real, SX, SY, SZ>(I, threadIdx.x, xt, yo));
    for (; k < z1; ++k, o += plane) {
        const bool kp = !EDGE || k + 1 < nz;
        const bool store = k >= z0;
        const bool zo = SZ && (k < I.pl[2] || k >= nz - I.ph[2]);
        if (LEAN_PF > 0) {
            const int kq = k + 1 + LEAN_PF;
            prefetch_lane_row<real>(lr, orow + (unsigned)(kq - k0) * plane, kq < nz && k + LEAN_PF < z1,
                              SZ && (kq < I.pl[2] || kq >= nz - I.ph[2]));
        }
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
                const unsigned om = o - 1;
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
                const unsigned om = o - px;
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
            const real* cf = I.coef + (int)__ldg(I.combo + o) * I.ncoef;
            const bool si = !dry;
            {
                const real d1 = hz - hz_ym, d2 = hy - hyp;
                real cv = d1 - d2;
                pml_term<SY, true, false>(cv, yo, byi, cyi, d1, peY, peY, o, si);
                pml_term<SZ, false, false>(cv, zo, bzi, czi, d2, peZ, peZ, o, si);
                oEX[o] = e_new_g<0, EXTRAS>(I, cf, ex_c, cv, i, j, k, n, dry);
            }
            {
                const real d1 = hx - hxp, d2 = hz - hz_xm;
                real cv = d1 - d2;
                pml_term<SZ, true, false>(cv, zo, bzi, czi, d1, peZ + vol, peZ + vol, o, si);
                pml_term<SX, false, false>(cv, xo, bxi, cxi, d2, peX, peX, o, si);
                oEY[o] = e_new_g<1, EXTRAS>(I, cf, ey_c, cv, i, j, k, n, dry);
            }
            {
                const real d1 = hy - hy_xm, d2 = hx - hx_ym;
                real cv = d1 - d2;
                pml_term<SX, true, false>(cv, xo, bxi, cxi, d1, peX + vol, peX + vol, o, si);
                pml_term<SY, false, false>(cv, yo, byi, cyi, d2, peY + vol, peY + vol, o, si);
                oEZ[o] = e_new_g<2, EXTRAS>(I, cf, ez, cv, i, j, k, n, dry);
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

// ------------------------------------------------------ shared-halo tiles
// CPML tiles with the neighbour H passed on instead of recomputed.  A block
// of LY + 2 warps: warps 0..LY-1 the tile's rows j0..j0+LY-1 (lane l:
// column i0+l), warp LY the row j0-1 and warp LY+1 the column i0-1 (lanes
// 0..LY-1: rows j0..j0+LY-1).  On every plane each warp updates H at its
// own cells through the same pml_term / h_new calls tile_block uses (the
// halo warps store nothing: the tiles that own those cells do), so the H
// a neighbour hands over has the bits tile_block would recompute.  Hx and Hz
// go to the row above through a double-buffered shared plane (one barrier
// per plane), Hy and Hz at x-1 come from the lane on the left by shuffle,
// and lane 0 takes them from the column warp.  Against tile_block this
// drops four recomputed H components (with their E, H and psi loads) per
// cell for two H-only warps per tile.  Cells outside the grid (EDGE) run
// with clamped coordinates, store nothing and are never read, so that every
// thread reaches every barrier and shuffle.
constexpr int HALO_WARPS = 2;
constexpr int HALO_THREADS = LX * (LY + HALO_WARPS);

template <typename real>
struct HaloPlane {
    real hx[LY + 1][LX];  // Hx of rows j0-1 .. j0+LY-1 (index: row - j0 + 1)
    real hz[LY + 1][LX];
    real xy[LY];          // Hy, Hz of column i0-1, rows j0 .. j0+LY-1
    real xz[LY];
};

// The H update's inputs of one plane at a warp's cell: E of the plane and
// of the one above, the x+1 / y+1 neighbours, old H and the old H-side psi
// (Hx: y, z; Hy: z, x; Hz: x, y; 0 outside the slabs), loaded together so
// that they are all in flight at once.  o: the cell's field offset, op: its
// psi offset; ok = false loads nothing (zeros).
template <typename real>
struct HaloIn {
    real ex_n, ey_n, ez, ez_xp, ez_yp, ey_xp, ex_yp, hx, hy, hz;
    real qy0, qz0, qz1, qx0, qx1, qy1;
};
template <typename real, bool SX, bool SY, bool SZ, bool EDGE>
__device__ __forceinline__ HaloIn<real> halo_in(const InstDev<real>& I, unsigned o, unsigned op, int k, bool ok,
                                                bool xp, bool yp, bool xo, bool yo) {
    const unsigned px = (unsigned)I.px, plane = (unsigned)I.plane, vol = (unsigned)I.vol;
    const bool kp = ok && (!EDGE || k + 1 < I.nz);
    const bool zo = SZ && (k < I.pl[2] || k >= I.nz - I.ph[2]);
    HaloIn<real> r;
    r.ex_n = ldz(I.F[0][0], o + plane, kp), r.ey_n = ldz(I.F[0][1], o + plane, kp);
    r.ez = ldz(I.F[0][2], o, ok);
    r.ez_xp = ldz(I.F[0][2], o + 1, ok && xp), r.ez_yp = ldz(I.F[0][2], o + px, ok && yp);
    r.ey_xp = ldz(I.F[0][1], o + 1, ok && xp), r.ex_yp = ldz(I.F[0][0], o + px, ok && yp);
    r.hx = ldz(I.F[0][3], o, ok), r.hy = ldz(I.F[0][4], o, ok), r.hz = ldz(I.F[0][5], o, ok);
    r.qy0 = psi_old<SY, true>(ok && yo, SY ? I.psiH[0][1] : nullptr, op);
    r.qy1 = psi_old<SY, true>(ok && yo, SY ? I.psiH[0][1] : nullptr, op + vol);
    r.qz0 = psi_old<SZ, true>(ok && zo, SZ ? I.psiH[0][2] : nullptr, op);
    r.qz1 = psi_old<SZ, true>(ok && zo, SZ ? I.psiH[0][2] : nullptr, op + vol);
    r.qx0 = psi_old<SX, true>(ok && xo, SX ? I.psiH[0][0] : nullptr, op);
    r.qx1 = psi_old<SX, true>(ok && xo, SX ? I.psiH[0][0] : nullptr, op + vol);
    return r;
}

template <typename real, int ZB, int MASK, bool EDGE>
__device__ __forceinline__ void tile_halo(const InstDev<real>& I, int tx, int ty, int tz, bool dry,
                                          HaloPlane<real>* sh, unsigned qf) {
    constexpr bool SX = (MASK & 1) != 0, SY = (MASK & 2) != 0, SZ = (MASK & 4) != 0;
    const int w = threadIdx.y, lane = threadIdx.x;
    const bool own = w < LY, rowh = w == LY, colh = w == LY + 1;
    const int nx = I.nx, ny = I.ny, nz = I.nz;
    const int i0 = tx * LX, j0 = ty * LY;
    const int z0 = tz * ZB, z1 = min(nz, z0 + ZB);
    int i = colh ? i0 - 1 : i0 + lane;
    int j = own ? j0 + w : (rowh ? j0 - 1 : j0 + min(lane, LY - 1));
    // a cell of the grid whose results are used
    const bool act = (!EDGE || (i >= 0 && j >= 0 && i < nx && j < ny)) && (!colh || lane < LY);
    if (EDGE) i = imin(imax(i, 0), nx - 1), j = imin(imax(j, 0), ny - 1);

    const unsigned px = (unsigned)I.px, plane = (unsigned)I.plane, vol = (unsigned)I.vol;
    const real* eX = I.F[0][0];
    const real* eY = I.F[0][1];
    real* oEX = I.F[1][0];
    real* oEY = I.F[1][1];
    real* oEZ = I.F[1][2];
    real* oHX = I.F[1][3];
    real* oHY = I.F[1][4];
    real* oHZ = I.F[1][5];
    real* hoX = SX ? I.psiH[1][0] : nullptr;
    real* hoY = SY ? I.psiH[1][1] : nullptr;
    real* hoZ = SZ ? I.psiH[1][2] : nullptr;
    real* peX = SX ? I.psiE[0] : nullptr;
    real* peY = SY ? I.psiE[1] : nullptr;
    real* peZ = SZ ? I.psiE[2] : nullptr;

    const bool xp = !EDGE || i + 1 < nx, yp = !EDGE || j + 1 < ny;
    // the neighbours at x-1 (lane 0: the column warp) and y-1 (row 0: the row warp) exist
    const bool xm = !EDGE || i0 > 0, ym = !EDGE || j0 > 0;
    const bool xo = SX && in_slab(I, 0, i), yo = SY && in_slab(I, 1, j);
    real bxi = 1, cxi = 0, bxh = 1, cxh = 0, byi = 1, cyi = 0, byh = 1, cyh = 0;
    if (SX && xo) {
        const real* pr = I.prof[0];
        bxi = ldg(pr, i), cxi = ldg(pr, nx + i), bxh = ldg(pr, 2 * nx + i), cxh = ldg(pr, 3 * nx + i);
    }
    if (SY && yo) {
        const real* pr = I.prof[1];
        byi = ldg(pr, j), cyi = ldg(pr, ny + j), byh = ldg(pr, 2 * ny + j), cyh = ldg(pr, 3 * ny + j);
    }

    int k = z0 > 0 ? z0 - 1 : 0;
    const int k0 = k;
    // field offsets (and psi offsets, + qf) of group member blockIdx.y
    unsigned o = (unsigned)k * plane + (unsigned)j * px + (unsigned)i + qf;
    real ex_c = ldg(eX, o), ey_c = ldg(eY, o);
    real hxp = 0, hyp = 0;  // H^{n+1/2} of plane k-1 at the own cell
    // row prefetch: the tile rows and the row below them (the column warp's
    // cells are not a row)
    const bool xt = SX && (imax(i0 - 1, 0) < I.pl[0] || imin(i0 + LX, nx) - 1 >= nx - I.ph[0]);
    const unsigned orow = (unsigned)k * plane + (unsigned)j * px + (unsigned)i0 + qf;
    volatile unsigned long long* lr =
        lane_row_park(colh ? 0ull : lane_row<real, SX, SY, SZ>(I, lane, xt, yo, qf));
    for (; k < z1; ++k, o += plane) {
        const bool store = k >= z0;  // block-uniform
        const bool zo = SZ && (k < I.pl[2] || k >= nz - I.ph[2]);
        if (LEAN_PF > 0) {
            const int kq = k + 1 + LEAN_PF;
            prefetch_lane_row<real>(lr, orow + (unsigned)(kq - k0) * plane, kq < nz && k + LEAN_PF < z1,
                                    SZ && (kq < I.pl[2] || kq >= nz - I.ph[2]));
        }
        // z profile values of the plane, by select (no branch)
        real bzi = 1, czi = 0, bzh = 1, czh = 0;
        if (SZ) {
            const real* pr = I.prof[2];
            bzi = zo ? ldg(pr, k) : real(1), czi = zo ? ldg(pr, nz + k) : real(0);
            bzh = zo ? ldg(pr, 2 * nz + k) : real(1), czh = zo ? ldg(pr, 3 * nz + k) : real(0);
        }
        // every load of the H update issued together
        const unsigned op = o + qf;
        const HaloIn<real> c = halo_in<real, SX, SY, SZ, EDGE>(I, o, op, k, true, xp, yp, xo, yo);
        const real ex_n = c.ex_n, ey_n = c.ey_n, ez = c.ez;
        const bool sp = store && !dry && own && act;

        // H^{n+1/2} at the warp's cells
        real hx, hy, hz;
        {
            const real d1 = c.ez_yp - ez, d2 = ey_n - ey_c;
            real cv = d1 - d2;
            pml_term_v<SY, true>(cv, yo, byh, cyh, d1, c.qy0, hoY, op, sp);
            pml_term_v<SZ, false>(cv, zo, bzh, czh, d2, c.qz0, hoZ, op, sp);
            hx = h_new<false>(I, 3, cv, c.hx, false, i, j, k, 0);
        }
        {
            const real d1 = ex_n - ex_c, d2 = c.ez_xp - ez;
            real cv = d1 - d2;
            pml_term_v<SZ, true>(cv, zo, bzh, czh, d1, c.qz1, hoZ + vol, op, sp);
            pml_term_v<SX, false>(cv, xo, bxh, cxh, d2, c.qx0, hoX, op, sp);
            hy = h_new<false>(I, 4, cv, c.hy, false, i, j, k, 0);
        }
        {
            const real d1 = c.ey_xp - ey_c, d2 = c.ex_yp - ex_c;
            real cv = d1 - d2;
            pml_term_v<SX, true>(cv, xo, bxh, cxh, d1, c.qx1, hoX + vol, op, sp);
            pml_term_v<SY, false>(cv, yo, byh, cyh, d2, c.qy1, hoY + vol, op, sp);
            hz = h_new<false>(I, 5, cv, c.hz, false, i, j, k, 0);
        }
        if (store) {
            // the E update's loads go ahead of the barrier (which the
            // compiler does not move loads across): the combo's S eps_inf^-1
            // and the old E-side psi of the own cell (the combo loads are
            // unconditional: every warp's offset is a cell of the grid)
            const bool eo = own && act;
            const real* cf = I.coef + (int)__ldg(I.combo + o) * I.ncoef;
            const real* sv = cf + I.ncoef - 3;  // S eps_inf^-1 per component
            const real iv0 = ldg(sv, 0), iv1 = ldg(sv, 1), iv2 = ldg(sv, 2);
            const real qY0 = psi_old<SY, false>(eo && yo, peY, op), qY1 = psi_old<SY, false>(eo && yo, peY, op + vol);
            const real qZ0 = psi_old<SZ, false>(eo && zo, peZ, op), qZ1 = psi_old<SZ, false>(eo && zo, peZ, op + vol);
            const real qX0 = psi_old<SX, false>(eo && xo, peX, op), qX1 = psi_old<SX, false>(eo && xo, peX, op + vol);
            HaloPlane<real>& b = sh[k & 1];
            if ((own && w < LY - 1) || rowh) {
                b.hx[rowh ? 0 : w + 1][lane] = hx;
                b.hz[rowh ? 0 : w + 1][lane] = hz;
            }
            if (colh && lane < LY) {
                b.xy[lane] = hy;
                b.xz[lane] = hz;
            }
            __syncthreads();
            if (own) {
                real hy_xm = __shfl_up_sync(FULL, hy, 1), hz_xm = __shfl_up_sync(FULL, hz, 1);
                if (lane == 0) hy_xm = xm ? b.xy[w] : real(0), hz_xm = xm ? b.xz[w] : real(0);
                const bool yn = ym || w > 0;
                const real hx_ym = yn ? b.hx[w][lane] : real(0), hz_ym = yn ? b.hz[w][lane] : real(0);
                if (act) {
                    oHX[o] = hx;
                    oHY[o] = hy;
                    oHZ[o] = hz;
                    // E^{n+1} at the own cell
                    const bool si = !dry;
                    {
                        const real d1 = hz - hz_ym, d2 = hy - hyp;
                        real cv = d1 - d2;
                        pml_term_v<SY, true>(cv, yo, byi, cyi, d1, qY0, peY, op, si);
                        pml_term_v<SZ, false>(cv, zo, bzi, czi, d2, qZ0, peZ, op, si);
                        oEX[o] = e_new_v(iv0, ex_c, cv);
                    }
                    {
                        const real d1 = hx - hxp, d2 = hz - hz_xm;
                        real cv = d1 - d2;
                        pml_term_v<SZ, true>(cv, zo, bzi, czi, d1, qZ1, peZ + vol, op, si);
                        pml_term_v<SX, false>(cv, xo, bxi, cxi, d2, qX0, peX, op, si);
                        oEY[o] = e_new_v(iv1, ey_c, cv);
                    }
                    {
                        const real d1 = hy - hy_xm, d2 = hx - hx_ym;
                        real cv = d1 - d2;
                        pml_term_v<SX, true>(cv, xo, bxi, cxi, d1, qX1, peX + vol, op, si);
                        pml_term_v<SY, false>(cv, yo, byi, cyi, d2, qY1, peY + vol, op, si);
                        oEZ[o] = e_new_v(iv2, ez, cv);
                    }
                }
            }
        }
        hxp = hx;
        hyp = hy;
        ex_c = ex_n;
        ey_c = ey_n;
    }
}

// ------------------------------------------ two-column shared-halo tiles
// tile_halo with two columns per thread (instances whose nx is a multiple of
// 32): a block of LY/2 + 1 warps.  Warps 0..LY/2-1 take the tile's rows as
// half-warps (row 2w + half; lane l of the half: columns i0+2l, i0+2l+1);
// the last warp's first half takes the row j0-1 and its second half the
// column pair (i0-2, i0-1) of rows j0..j0+LY-1 (lane l: row j0+l).  Fields
// and psi move as pairs; the H at x-1 comes from the neighbouring lane by
// shuffle (lane 0: from the column half), the H at y-1 through the shared
// plane, the E at x+2 from the next lane (last lane and column half: loaded).
// Each element evaluates tile_halo's formulas in the same order, so both
// bodies give the same bits.
constexpr int HALO2_THREADS = LX * (LY / 2 + 1);

template <typename real>
struct HaloIn2 {
    typename Pair<real>::T ex_n, ey_n, ez, ez_yp, ex_yp, hx, hy, hz;
    typename Pair<real>::T qy0, qy1, qz0, qz1, qx0, qx1;  // H-side psi (as in HaloIn)
    real ez_x2, ey_x2;                                    // E at column i+2 of plane k
};
template <typename real>
__device__ __forceinline__ typename Pair<real>::T ld2p(bool on, const real* p, unsigned o) {
    typename Pair<real>::T v;
    if (on) return ld2(p, o);
    v.x = v.y = real(0);
    return v;
}

template <typename real, int ZB, int MASK, bool EDGE>
__device__ __forceinline__ void tile_pair_halo(const InstDev<real>& I, int tx, int ty, int tz, bool dry,
                                               HaloPlane<real>* sh, unsigned qf) {
    using V2 = typename Pair<real>::T;
    constexpr bool SX = (MASK & 1) != 0, SY = (MASK & 2) != 0, SZ = (MASK & 4) != 0;
    constexpr int NW = LY / 2;  // warps of tile rows
    const int w = threadIdx.y, l = threadIdx.x & 15, half = threadIdx.x >> 4;
    const bool own = w < NW, rowh = w == NW && half == 0, colh = w == NW && half == 1;
    const int r = 2 * w + half;  // own: tile row
    const int nx = I.nx, ny = I.ny, nz = I.nz;
    const int i0 = tx * LX, j0 = ty * LY;
    const int z0 = tz * ZB, z1 = min(nz, z0 + ZB);
    int i = colh ? i0 - 2 : i0 + 2 * l;
    int j = own ? j0 + r : (rowh ? j0 - 1 : j0 + min(l, LY - 1));
    // a cell pair of the grid whose results are used (nx even: i < nx implies i + 1 < nx)
    const bool act = (!EDGE || (i >= 0 && j >= 0 && i < nx && j < ny)) && (!colh || l < LY);
    if (EDGE) i = imin(imax(i, 0), nx - 2), j = imin(imax(j, 0), ny - 1);

    const unsigned px = (unsigned)I.px, plane = (unsigned)I.plane, vol = (unsigned)I.vol;
    const real* eX = I.F[0][0];
    const real* eY = I.F[0][1];
    const real* eZ = I.F[0][2];
    const real* hX = I.F[0][3];
    const real* hY = I.F[0][4];
    const real* hZ = I.F[0][5];
    real* oEX = I.F[1][0];
    real* oEY = I.F[1][1];
    real* oEZ = I.F[1][2];
    real* oHX = I.F[1][3];
    real* oHY = I.F[1][4];
    real* oHZ = I.F[1][5];
    const real* hiX = SX ? I.psiH[0][0] : nullptr;
    const real* hiY = SY ? I.psiH[0][1] : nullptr;
    const real* hiZ = SZ ? I.psiH[0][2] : nullptr;
    real* hoX = SX ? I.psiH[1][0] : nullptr;
    real* hoY = SY ? I.psiH[1][1] : nullptr;
    real* hoZ = SZ ? I.psiH[1][2] : nullptr;
    real* peX = SX ? I.psiE[0] : nullptr;
    real* peY = SY ? I.psiE[1] : nullptr;
    real* peZ = SZ ? I.psiE[2] : nullptr;
    const real S = I.S;

    const bool yp = !EDGE || j + 1 < ny;
    const bool xl = l == 15 || colh;             // loads the E of column i+2 itself
    const bool xp2 = xl && (!EDGE || i + 2 < nx);
    const bool xm = !EDGE || i0 > 0, ym = !EDGE || j0 > 0;
    const bool xo0 = SX && in_slab(I, 0, i), xo1 = SX && in_slab(I, 0, i + 1), xo = xo0 || xo1;
    const bool yo = SY && in_slab(I, 1, j);
    real bxi0 = 1, cxi0 = 0, bxh0 = 1, cxh0 = 0, bxi1 = 1, cxi1 = 0, bxh1 = 1, cxh1 = 0;
    real byi = 1, cyi = 0, byh = 1, cyh = 0;
    if (SX) {
        const real* pr = I.prof[0];
        if (xo0) bxi0 = ldg(pr, i), cxi0 = ldg(pr, nx + i), bxh0 = ldg(pr, 2 * nx + i), cxh0 = ldg(pr, 3 * nx + i);
        if (xo1)
            bxi1 = ldg(pr, i + 1), cxi1 = ldg(pr, nx + i + 1), bxh1 = ldg(pr, 2 * nx + i + 1),
            cxh1 = ldg(pr, 3 * nx + i + 1);
    }
    if (SY && yo) {
        const real* pr = I.prof[1];
        byi = ldg(pr, j), cyi = ldg(pr, ny + j), byh = ldg(pr, 2 * ny + j), cyh = ldg(pr, 3 * ny + j);
    }

    int k = z0 > 0 ? z0 - 1 : 0;
    const int k0 = k;
    unsigned o = (unsigned)k * plane + (unsigned)j * px + (unsigned)i + qf;  // group member blockIdx.y
    V2 ex_c = ld2(eX, o), ey_c = ld2(eY, o);
    V2 hxp, hyp;
    hxp.x = hxp.y = hyp.x = hyp.y = real(0);
    const bool xt = SX && (imax(i0 - 1, 0) < I.pl[0] || imin(i0 + LX, nx) - 1 >= nx - I.ph[0]);
    const unsigned orow = (unsigned)k * plane + (unsigned)j * px + (unsigned)i0 + qf;
    // a half-warp's 16 lanes take rows 0-15 (three-axis tiles: the z psi rows go without)
    volatile unsigned long long* lr =
        lane_row_park(colh ? 0ull : lane_row<real, SX, SY, SZ>(I, l, xt, yo, qf));
    for (; k < z1; ++k, o += plane) {
        const bool kp = !EDGE || k + 1 < nz;
        const bool store = k >= z0;  // block-uniform
        const bool zo = SZ && (k < I.pl[2] || k >= nz - I.ph[2]);
        if (LEAN_PF > 0) {
            const int kq = k + 1 + LEAN_PF;
            prefetch_lane_row<real>(lr, orow + (unsigned)(kq - k0) * plane, kq < nz && k + LEAN_PF < z1,
                                    SZ && (kq < I.pl[2] || kq >= nz - I.ph[2]));
        }
        real bzi = 1, czi = 0, bzh = 1, czh = 0;
        if (SZ) {
            const real* pr = I.prof[2];
            bzi = zo ? ldg(pr, k) : real(1), czi = zo ? ldg(pr, nz + k) : real(0);
            bzh = zo ? ldg(pr, 2 * nz + k) : real(1), czh = zo ? ldg(pr, 3 * nz + k) : real(0);
        }
        const unsigned op = o + qf;
        // every load of the H update issued together
        HaloIn2<real> c;
        c.ex_n = ld2p(kp, eX, o + plane), c.ey_n = ld2p(kp, eY, o + plane);
        c.ez = ld2(eZ, o);
        c.ez_yp = ld2p(yp, eZ, o + px), c.ex_yp = ld2p(yp, eX, o + px);
        c.hx = ld2(hX, o), c.hy = ld2(hY, o), c.hz = ld2(hZ, o);
        c.qy0 = ld2p(SY && yo, hiY, op), c.qy1 = ld2p(SY && yo, hiY, op + vol);
        c.qz0 = ld2p(SZ && zo, hiZ, op), c.qz1 = ld2p(SZ && zo, hiZ, op + vol);
        c.qx0 = ld2p(SX && xo, hiX, op), c.qx1 = ld2p(SX && xo, hiX, op + vol);
        const real ez_x2l = xp2 ? ldg(eZ, o + 2) : real(0), ey_x2l = xp2 ? ldg(eY, o + 2) : real(0);
        {
            const real a = __shfl_down_sync(FULL, c.ez.x, 1, 16), b = __shfl_down_sync(FULL, ey_c.x, 1, 16);
            c.ez_x2 = xl ? ez_x2l : a;
            c.ey_x2 = xl ? ey_x2l : b;
        }
        const bool sp = store && !dry && own && act;

        // H^{n+1/2} at the thread's two cells
        V2 hx, hy, hz;
        {
            real d1 = c.ez_yp.x - c.ez.x, d2 = c.ey_n.x - ey_c.x, cv = d1 - d2;
            pml_term_v<SY, true>(cv, yo, byh, cyh, d1, c.qy0.x, hoY, op, sp);
            pml_term_v<SZ, false>(cv, zo, bzh, czh, d2, c.qz0.x, hoZ, op, sp);
            hx.x = fma(-S, cv, c.hx.x);
            d1 = c.ez_yp.y - c.ez.y, d2 = c.ey_n.y - ey_c.y, cv = d1 - d2;
            pml_term_v<SY, true>(cv, yo, byh, cyh, d1, c.qy0.y, hoY, op + 1, sp);
            pml_term_v<SZ, false>(cv, zo, bzh, czh, d2, c.qz0.y, hoZ, op + 1, sp);
            hx.y = fma(-S, cv, c.hx.y);
        }
        {
            real d1 = c.ex_n.x - ex_c.x, d2 = c.ez.y - c.ez.x, cv = d1 - d2;
            pml_term_v<SZ, true>(cv, zo, bzh, czh, d1, c.qz1.x, hoZ + vol, op, sp);
            pml_term_v<SX, false>(cv, xo0, bxh0, cxh0, d2, c.qx0.x, hoX, op, sp);
            hy.x = fma(-S, cv, c.hy.x);
            d1 = c.ex_n.y - ex_c.y, d2 = c.ez_x2 - c.ez.y, cv = d1 - d2;
            pml_term_v<SZ, true>(cv, zo, bzh, czh, d1, c.qz1.y, hoZ + vol, op + 1, sp);
            pml_term_v<SX, false>(cv, xo1, bxh1, cxh1, d2, c.qx0.y, hoX, op + 1, sp);
            hy.y = fma(-S, cv, c.hy.y);
        }
        {
            real d1 = ey_c.y - ey_c.x, d2 = c.ex_yp.x - ex_c.x, cv = d1 - d2;
            pml_term_v<SX, true>(cv, xo0, bxh0, cxh0, d1, c.qx1.x, hoX + vol, op, sp);
            pml_term_v<SY, false>(cv, yo, byh, cyh, d2, c.qy1.x, hoY + vol, op, sp);
            hz.x = fma(-S, cv, c.hz.x);
            d1 = c.ey_x2 - ey_c.y, d2 = c.ex_yp.y - ex_c.y, cv = d1 - d2;
            pml_term_v<SX, true>(cv, xo1, bxh1, cxh1, d1, c.qx1.y, hoX + vol, op + 1, sp);
            pml_term_v<SY, false>(cv, yo, byh, cyh, d2, c.qy1.y, hoY + vol, op + 1, sp);
            hz.y = fma(-S, cv, c.hz.y);
        }
        if (store) {
            // the E update's loads ahead of the barrier: S eps_inf^-1 of both
            // combos and the old E-side psi (the combo loads are unconditional:
            // every thread's offset is a cell pair of the grid)
            const bool eo = own && act;
            const uchar2 cb = __ldg(reinterpret_cast<const uchar2*>(I.combo + o));
            const real* s0 = I.coef + (int)cb.x * I.ncoef + I.ncoef - 3;
            const real* s1 = I.coef + (int)cb.y * I.ncoef + I.ncoef - 3;
            const real a0 = ldg(s0, 0), a1 = ldg(s0, 1), a2 = ldg(s0, 2);
            const real b0 = ldg(s1, 0), b1 = ldg(s1, 1), b2 = ldg(s1, 2);
            const V2 pY0 = ld2p(SY && eo && yo, peY, op), pY1 = ld2p(SY && eo && yo, peY, op + vol);
            const V2 pZ0 = ld2p(SZ && eo && zo, peZ, op), pZ1 = ld2p(SZ && eo && zo, peZ, op + vol);
            const V2 pX0 = ld2p(SX && eo && xo, peX, op), pX1 = ld2p(SX && eo && xo, peX, op + vol);
            HaloPlane<real>& b = sh[k & 1];
            if ((own && r < LY - 1) || rowh) {
                const int row = rowh ? 0 : r + 1;
                b.hx[row][2 * l] = hx.x, b.hx[row][2 * l + 1] = hx.y;
                b.hz[row][2 * l] = hz.x, b.hz[row][2 * l + 1] = hz.y;
            }
            if (colh && l < LY) {
                b.xy[l] = hy.y;
                b.xz[l] = hz.y;
            }
            __syncthreads();
            if (own) {
                real hy_m = __shfl_up_sync(FULL, hy.y, 1, 16), hz_m = __shfl_up_sync(FULL, hz.y, 1, 16);
                if (l == 0) hy_m = xm ? b.xy[r] : real(0), hz_m = xm ? b.xz[r] : real(0);
                const bool yn = ym || r > 0;
                V2 hx_ym, hz_ym;
                hx_ym.x = yn ? b.hx[r][2 * l] : real(0), hx_ym.y = yn ? b.hx[r][2 * l + 1] : real(0);
                hz_ym.x = yn ? b.hz[r][2 * l] : real(0), hz_ym.y = yn ? b.hz[r][2 * l + 1] : real(0);
                if (!EDGE || act) {
                    st2(oHX, o, hx.x, hx.y);
                    st2(oHY, o, hy.x, hy.y);
                    st2(oHZ, o, hz.x, hz.y);
                    const bool si = !dry;
                    V2 ex, ey, ezn;
                    {
                        real d1 = hz.x - hz_ym.x, d2 = hy.x - hyp.x, cv = d1 - d2;
                        pml_term_v<SY, true>(cv, yo, byi, cyi, d1, pY0.x, peY, op, si);
                        pml_term_v<SZ, false>(cv, zo, bzi, czi, d2, pZ0.x, peZ, op, si);
                        ex.x = e_new_v(a0, ex_c.x, cv);
                        d1 = hz.y - hz_ym.y, d2 = hy.y - hyp.y, cv = d1 - d2;
                        pml_term_v<SY, true>(cv, yo, byi, cyi, d1, pY0.y, peY, op + 1, si);
                        pml_term_v<SZ, false>(cv, zo, bzi, czi, d2, pZ0.y, peZ, op + 1, si);
                        ex.y = e_new_v(b0, ex_c.y, cv);
                    }
                    {
                        real d1 = hx.x - hxp.x, d2 = hz.x - hz_m, cv = d1 - d2;
                        pml_term_v<SZ, true>(cv, zo, bzi, czi, d1, pZ1.x, peZ + vol, op, si);
                        pml_term_v<SX, false>(cv, xo0, bxi0, cxi0, d2, pX0.x, peX, op, si);
                        ey.x = e_new_v(a1, ey_c.x, cv);
                        d1 = hx.y - hxp.y, d2 = hz.y - hz.x, cv = d1 - d2;
                        pml_term_v<SZ, true>(cv, zo, bzi, czi, d1, pZ1.y, peZ + vol, op + 1, si);
                        pml_term_v<SX, false>(cv, xo1, bxi1, cxi1, d2, pX0.y, peX, op + 1, si);
                        ey.y = e_new_v(b1, ey_c.y, cv);
                    }
                    {
                        real d1 = hy.x - hy_m, d2 = hx.x - hx_ym.x, cv = d1 - d2;
                        pml_term_v<SX, true>(cv, xo0, bxi0, cxi0, d1, pX1.x, peX + vol, op, si);
                        pml_term_v<SY, false>(cv, yo, byi, cyi, d2, pY1.x, peY + vol, op, si);
                        ezn.x = e_new_v(a2, c.ez.x, cv);
                        d1 = hy.y - hy.x, d2 = hx.y - hx_ym.y, cv = d1 - d2;
                        pml_term_v<SX, true>(cv, xo1, bxi1, cxi1, d1, pX1.y, peX + vol, op + 1, si);
                        pml_term_v<SY, false>(cv, yo, byi, cyi, d2, pY1.y, peY + vol, op + 1, si);
                        ezn.y = e_new_v(b2, c.ez.y, cv);
                    }
                    st2(oEX, o, ex.x, ex.y);
                    st2(oEY, o, ey.x, ey.y);
                    st2(oEZ, o, ezn.x, ezn.y);
                }
            }
        }
        hxp = hx;
        hyp = hy;
        ex_c = c.ex_n;
        ey_c = c.ey_n;
    }
}

template <typename real, int ZB, int MASK>
__device__ __forceinline__ void tile_pair_halo_any(const InstDev<real>& I, int tx, int ty, int tz, bool dry,
                                                   HaloPlane<real>* sh, unsigned qf) {
    if (tile_edge(I, tx, ty, tz, ZB))
        tile_pair_halo<real, ZB, MASK, true>(I, tx, ty, tz, dry, sh, qf);
    else
        tile_pair_halo<real, ZB, MASK, false>(I, tx, ty, tz, dry, sh, qf);
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
    if (ms >= 0 && (n % I.save_span) == 0) monitor_store(I, n, ms, v, st);
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

// The instance descriptor travels in the launch's parameter space
// (__grid_constant__), with slot 0 of the ping-pong pairs (fields, H-side
// psi) holding the current buffers and slot 1 the next ones: the host swaps
// them by parity.  Every block reads the descriptor through the constant
// cache at fixed offsets, so pointers, extents and coefficients cost no
// per-thread registers.  Each launch takes one instance and one tile class;
// its blocks map to the class's tiles through a list built on the host.

__device__ __forceinline__ void tile_decode(unsigned code, int& tx, int& ty, int& tz, int& mask) {
    tx = (int)(code & 511u);
    ty = (int)((code >> 9) & 1023u);
    tz = (int)((code >> 19) & 1023u);
    mask = (int)(code >> 29);
}

// Only the general and correction launches read the step counter (sources,
// probes): their blocks count themselves, and the last one of the step
// (step_blocks in all) advances the step and flips the device copy of the
// parity.
__device__ __forceinline__ void finish_block(unsigned step_blocks, int dry, DevState* st) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&st->done, 1u);
        if (prev == step_blocks - 1) {
            if (!dry) {
                st->step += 1;
                st->cur ^= 1;
            }
            st->done = 0;
            __threadfence();
        }
    }
}

// Plain tiles: no CPML slab, source or dispersive voxel in the footprint.

template <typename real, int ZB>
__global__ void __launch_bounds__(LX * LY, plain_minb<real>())
k_lean_plain(const __grid_constant__ LeanTable<real> tab) {
    int tx, ty, tz, m;
    tile_decode(__ldg(tab.tiles + blockIdx.x), tx, ty, tz, m);
    const unsigned qf = blockIdx.y * tab.qvol;
    if (tile_edge(tab.inst, tx, ty, tz, ZB))
        plain_block<real, ZB, true>(tab.inst, tx, ty, tz, qf);
    else
        plain_block<real, ZB, false>(tab.inst, tx, ty, tz, qf);
}

// sh: the kernel's two shared planes (declared once per kernel, not per
// instantiation of the body)
template <typename real, int ZB, int MASK>
__device__ __forceinline__ void tile_halo_any(const InstDev<real>& I, int tx, int ty, int tz, bool dry,
                                              HaloPlane<real>* sh, unsigned qf) {
    if (tile_edge(I, tx, ty, tz, ZB))
        tile_halo<real, ZB, MASK, true>(I, tx, ty, tz, dry, sh, qf);
    else
        tile_halo<real, ZB, MASK, false>(I, tx, ty, tz, dry, sh, qf);
}

// Single-slab tiles: the footprint touches the slabs of exactly one axis.
template <typename real, int ZB>
__global__ void __launch_bounds__(HALO_THREADS, slab_minb<real>())
k_lean_slab(const __grid_constant__ LeanTable<real> tab) {
    __shared__ HaloPlane<real> sh[2];
    int tx, ty, tz, m;
    tile_decode(__ldg(tab.tiles + blockIdx.x), tx, ty, tz, m);
    const unsigned qf = blockIdx.y * tab.qvol;
    if (m == 1)
        tile_halo_any<real, ZB, 1>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else if (m == 2)
        tile_halo_any<real, ZB, 2>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else
        tile_halo_any<real, ZB, 4>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
}

// Multi-slab tiles: the slabs of two or three axes (edges and corners).
template <typename real, int ZB>
__global__ void __launch_bounds__(HALO_THREADS, multi_minb<real>())
k_lean_multi(const __grid_constant__ LeanTable<real> tab) {
    __shared__ HaloPlane<real> sh[2];
    int tx, ty, tz, m;
    tile_decode(__ldg(tab.tiles + blockIdx.x), tx, ty, tz, m);
    const unsigned qf = blockIdx.y * tab.qvol;
    if (m == 3)
        tile_halo_any<real, ZB, 3>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else if (m == 5)
        tile_halo_any<real, ZB, 5>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else if (m == 6)
        tile_halo_any<real, ZB, 6>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else
        tile_halo_any<real, ZB, 7>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
}

// Single- and multi-slab tiles with two columns per thread (instances whose
// nx is a multiple of 32), 5 warps per tile.  The single-slab body fits 64
// registers without spilling (6 blocks per SM); the multi-slab body spills a
// little at 5 blocks per SM and still runs faster there than at 4 or 6.
#ifndef SJ_LEAN_SLAB2_MINB
#define SJ_LEAN_SLAB2_MINB 6
#endif
#ifndef SJ_LEAN_MULTI2_MINB
#define SJ_LEAN_MULTI2_MINB 5
#endif
template <typename real>
constexpr int slab2_minb() { return sizeof(real) == 4 ? SJ_LEAN_SLAB2_MINB : 2; }
template <typename real>
constexpr int multi2_minb() { return sizeof(real) == 4 ? SJ_LEAN_MULTI2_MINB : 2; }

template <typename real, int ZB>
__global__ void __launch_bounds__(HALO2_THREADS, slab2_minb<real>())
k_lean_slab2(const __grid_constant__ LeanTable<real> tab) {
    __shared__ HaloPlane<real> sh[2];
    int tx, ty, tz, m;
    tile_decode(__ldg(tab.tiles + blockIdx.x), tx, ty, tz, m);
    const unsigned qf = blockIdx.y * tab.qvol;
    if (m == 1)
        tile_pair_halo_any<real, ZB, 1>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else if (m == 2)
        tile_pair_halo_any<real, ZB, 2>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else
        tile_pair_halo_any<real, ZB, 4>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
}

template <typename real, int ZB>
__global__ void __launch_bounds__(HALO2_THREADS, multi2_minb<real>())
k_lean_multi2(const __grid_constant__ LeanTable<real> tab) {
    __shared__ HaloPlane<real> sh[2];
    int tx, ty, tz, m;
    tile_decode(__ldg(tab.tiles + blockIdx.x), tx, ty, tz, m);
    const unsigned qf = blockIdx.y * tab.qvol;
    if (m == 3)
        tile_pair_halo_any<real, ZB, 3>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else if (m == 5)
        tile_pair_halo_any<real, ZB, 5>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else if (m == 6)
        tile_pair_halo_any<real, ZB, 6>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
    else
        tile_pair_halo_any<real, ZB, 7>(tab.inst, tx, ty, tz, tab.dry != 0, sh, qf);
}

// Plain tiles with two columns per thread (instances whose nx is a multiple
// of 32): the two-column shared-halo body with no CPML axis, 5 warps per tile.
template <typename real, int ZB>
__global__ void __launch_bounds__(HALO2_THREADS, pair_plain_minb<real>())
k_lean_plain2(const __grid_constant__ LeanTable<real> tab) {
    __shared__ HaloPlane<real> sh[2];
    int tx, ty, tz, m;
    tile_decode(__ldg(tab.tiles + blockIdx.x), tx, ty, tz, m);
    tile_pair_halo_any<real, ZB, 0>(tab.inst, tx, ty, tz, tab.dry != 0, sh, blockIdx.y * tab.qvol);
}

// Queued tiles (LeanQueue): resident blocks claim (group, member, tile)
// items from a counter, multi-slab tiles first; every group's descriptor
// travels in the parameter space (as the grouped launches' one does), and the
// tile runs the two-column body of its slab mask.  One register budget covers
// every mask.
#ifndef SJ_LEAN_QUEUE_MINB
#define SJ_LEAN_QUEUE_MINB 5
#endif
template <typename real, int ZB>
__global__ void __launch_bounds__(HALO2_THREADS, SJ_LEAN_QUEUE_MINB)
k_lean_queue(const __grid_constant__ LeanQueueParams<real> qp, const uint4* __restrict__ items, unsigned n_items,
             unsigned* __restrict__ ctr) {
    __shared__ HaloPlane<real> sh[2];
    __shared__ unsigned s_item;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (;;) {
        __syncthreads();  // the previous tile is done with sh
        if (tid == 0) s_item = atomicAdd(ctr, 1u);
        __syncthreads();
        const unsigned it = s_item;
        if (it >= n_items) break;
        const uint4 w = __ldg(items + it);
        const LeanTable<real>& st = qp.t[w.x];
        int tx, ty, tz, m;
        tile_decode(w.z, tx, ty, tz, m);
        const unsigned qf = w.y * st.qvol;
        const bool dry = st.dry != 0;
        switch (m) {
            case 0: tile_pair_halo_any<real, ZB, 0>(st.inst, tx, ty, tz, dry, sh, qf); break;
            case 1: tile_pair_halo_any<real, ZB, 1>(st.inst, tx, ty, tz, dry, sh, qf); break;
            case 2: tile_pair_halo_any<real, ZB, 2>(st.inst, tx, ty, tz, dry, sh, qf); break;
            case 3: tile_pair_halo_any<real, ZB, 3>(st.inst, tx, ty, tz, dry, sh, qf); break;
            case 4: tile_pair_halo_any<real, ZB, 4>(st.inst, tx, ty, tz, dry, sh, qf); break;
            case 5: tile_pair_halo_any<real, ZB, 5>(st.inst, tx, ty, tz, dry, sh, qf); break;
            case 6: tile_pair_halo_any<real, ZB, 6>(st.inst, tx, ty, tz, dry, sh, qf); break;
            default: tile_pair_halo_any<real, ZB, 7>(st.inst, tx, ty, tz, dry, sh, qf); break;
        }
    }
}

int lean_queue_blocks_per_sm(int zb) {
    int nb = 0;
    cudaError_t e = cudaSuccess;
    if (zb == 8)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lean_queue<float, 8>, HALO2_THREADS, 0);
    else if (zb == 16)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lean_queue<float, 16>, HALO2_THREADS, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_lean_queue<float, 32>, HALO2_THREADS, 0);
    return e == cudaSuccess ? nb : 0;
}

// General tiles (an H source in the footprint) and probe blocks of every
// instance, one launch per step (LeanGen).
template <typename real, int ZB>
__global__ void __launch_bounds__(LX * LY, general_minb<real>())
k_lean_general(const InstDev<real>* __restrict__ parity_tab, const int4* __restrict__ blk, long long n_blk,
               int n_inst, int cur, int dry, unsigned step_blocks, DevState* st) {
    const long long n = st->step;
    const long long b = blockIdx.x;
    if (b < n_blk) {  // beyond: the one counting block of a step without general work
        const int4 e = blk[b];
        const InstDev<real>& I = parity_tab[(long long)cur * n_inst + e.x];
        if (e.y == 0) {
            int tx, ty, tz, m;
            tile_decode((unsigned)e.z, tx, ty, tz, m);
            // tile_block returns early for columns outside the grid; every
            // thread still reaches the barrier in finish_block
            tile_block<real, ZB, 7, true, true>(I, tx, ty, tz, n, dry != 0);
        } else if (!dry) {
            lean_probe_block<real>(I, e.z, n, 0, st);
        }
    }
    finish_block(step_blocks, dry, st);
}

// ------------------------------------------------------------ corrections
// After the tile kernels of a step, on the caller's stream and in this
// order: one k_lean_esrc launch per source slot s (the instances whose
// source s is an E source), then one k_lean_disp launch (the instances with
// dispersive voxels).  Block b takes FIX_THREADS cells of one instance's box:
// blk[b] = (instance, first cell / FIX_THREADS).  Descriptors come from the
// device table; `cur` is the step's parity.

// E^{n+1} = fma(-eps_inf^{-1}, dt J_s, E^{n+1}) over source s's box
// ESRC_R cells of the box per thread, in turn (fewer, longer blocks pay
// less for the step counter's fence and atomic at the end of each block);
// box coordinates in 32 bits.
constexpr int ESRC_R = 8;
constexpr int ESRC_CELLS = ESRC_R * FIX_THREADS;
template <typename real>
__global__ void __launch_bounds__(FIX_THREADS)
k_lean_esrc(const InstDev<real>* __restrict__ insts, const int2* __restrict__ blk, int slot, int cur,
            unsigned step_blocks, int dry, DevState* st) {
    const long long n = st->step;
    const int2 e = __ldg(blk + blockIdx.x);
    const InstDev<real>& I = insts[e.x];
    const SrcDev<real>& sv = I.src[slot];
    const unsigned n0 = (unsigned)sv.n[0], n1 = (unsigned)sv.n[1];
    const unsigned cells = n0 * n1 * (unsigned)sv.n[2];
    const int lo0 = sv.lo[0], lo1 = sv.lo[1], lo2 = sv.lo[2], comp = sv.comp;
    const real tn = (real)sv.tab[n];
    real* const E = I.F[cur ^ 1][comp];
    for (int r = 0; r < ESRC_R; ++r) {
        const unsigned cell = (unsigned)e.y * ESRC_CELLS + r * FIX_THREADS + threadIdx.x;
        if (cell >= cells) break;
        const unsigned q = cell / n0, dk = q / n1;
        const int di = (int)(cell - q * n0), dj = (int)(q - dk * n1);
        const long long o = (long long)(lo2 + (int)dk) * I.plane + (long long)(lo1 + dj) * I.px + (lo0 + di);
        const long long d = design_index(I, lo0 + di, lo1 + dj, lo2 + (int)dk);
        const real cfc = d >= 0 ? I.dinv[d] : I.coef[(int)I.combo[o] * I.ncoef + comp];
        const real J = tn * sv.w[0][di] * sv.w[1][dj] * sv.w[2][dk];
        E[o] = fma(-cfc, J, E[o]);
        if (!dry)
            if (real* rr = design_rec(I, d, n, comp)) *rr -= J;
    }
    finish_block(step_blocks, dry, st);
}

// meep's Lorentz/Drude ADE over the dispersive bounding box:
// P^{n+1} = A P^n + B P^{n-1} + C sigma E^n per pole the material has at the
// E point (pmask), and E^{n+1} = fma(-eps_inf^{-1}, sum_p (P^{n+1} - P^n),
// E^{n+1}).  A pole the material does not have at the E point keeps P = 0
// and would add +0: it is neither read nor written, and neither is a
// component without poles.  One thread per voxel (its three components), a
// block per DISP_VOXELS voxels of the box (DISP_R per thread, in turn): per
// voxel the combo first, then E and P of the first two poles of every
// component together (a third and later pole of a component, which no
// material here has, follows in order).  Sixteen voxels per thread and four
// blocks per SM (64 registers): every block ends with the step counter's
// fence and atomic, so fewer, longer blocks pay less for it (16 x 192^3 Au on
// quartz, forward step: 4 voxels, 3 blocks per SM 3.21 ms; 4, 4: 2.99; 8, 4:
// 2.89; 16, 4: 2.85; 32, 4: 2.85).
#ifndef SJ_DISP_R
#define SJ_DISP_R 16
#endif
#ifndef SJ_DISP_MINB
#define SJ_DISP_MINB 4
#endif
constexpr int DISP_R = SJ_DISP_R;
constexpr int DISP_VOXELS = DISP_R * FIX_THREADS;
template <typename real>
__global__ void __launch_bounds__(FIX_THREADS, sizeof(real) == 4 ? SJ_DISP_MINB : 2)
k_lean_disp(const InstDev<real>* __restrict__ insts, const int2* __restrict__ blk, int cur, unsigned step_blocks,
            int dry, DevState* st) {
    const long long n = st->step;
    const int2 e = __ldg(blk + blockIdx.x);
    const InstDev<real>& I = insts[e.x];
    // the descriptor's fields, read once (offsets within an instance fit 32 bits)
    const unsigned dvol = (unsigned)I.dvol, d0 = (unsigned)I.dn[0], d1 = (unsigned)I.dn[1];
    const int lo0 = I.dlo[0], lo1 = I.dlo[1], lo2 = I.dlo[2];
    const unsigned plane = (unsigned)I.plane, px = (unsigned)I.px;
    const uint8_t* combo = I.combo;
    const uint32_t* pmask = I.pmask;
    const real* coef = I.coef;
    const int ncoef = I.ncoef;
    real* const P = I.P;
    const real* Eo[3] = {I.F[cur][0], I.F[cur][1], I.F[cur][2]};
    real* const En[3] = {I.F[cur ^ 1][0], I.F[cur ^ 1][1], I.F[cur ^ 1][2]};
    const long long lv = 3 * (long long)dvol;  // from level n to level n-1 of a pole
    const unsigned base = (unsigned)e.y * DISP_VOXELS + threadIdx.x;
    for (int r = 0; r < DISP_R; ++r) {
        const unsigned u = base + r * FIX_THREADS;
        if (u >= dvol) break;
        const unsigned q = u / d0, kk = q / d1;
        const int i = lo0 + (int)(u - q * d0), j = lo1 + (int)(q - kk * d1), k = lo2 + (int)kk;
        const unsigned o = (unsigned)k * plane + (unsigned)j * px + (unsigned)i;
        const int cb = combo[o];
        const unsigned mask = pmask[cb];
        if (!mask) continue;
        const real* cf = coef + cb * ncoef;
        real eo[3], ec[3], pn1[3], pq1[3], pn2[3], pq2[3], c1[3], c2[3];
        int pa[3], pb[3];
        unsigned rest[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const unsigned m = (mask >> (8 * c)) & 255u;
            const unsigned m2 = m & (m - 1);
            pa[c] = m ? __ffs(m) - 1 : -1;
            pb[c] = m2 ? __ffs(m2) - 1 : -1;
            rest[c] = m2 & (m2 - 1);
            eo[c] = m ? Eo[c][o] : real(0);
            ec[c] = m ? En[c][o] : real(0);
            const long long a1 = ((long long)pa[c] * 6 + c) * dvol + u, a2 = ((long long)pb[c] * 6 + c) * dvol + u;
            c1[c] = m ? cf[3 + 3 * pa[c] + c] : real(0);
            c2[c] = m2 ? cf[3 + 3 * pb[c] + c] : real(0);
            pn1[c] = m ? P[a1] : real(0), pq1[c] = m ? P[a1 + lv] : real(0);
            pn2[c] = m2 ? P[a2] : real(0), pq2[c] = m2 ? P[a2 + lv] : real(0);
        }
        const long long d = design_index(I, i, j, k);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (pa[c] < 0) continue;
            real corr = 0;
            {
                const real pnew = I.A[pa[c]] * pn1[c] + I.B[pa[c]] * pq1[c] + c1[c] * eo[c];
                corr += pnew - pn1[c];
                if (!dry) {
                    real* pp = P + ((long long)pa[c] * 6 + c) * dvol + u;
                    pp[lv] = pn1[c];
                    *pp = pnew;
                }
            }
            if (pb[c] >= 0) {
                const real pnew = I.A[pb[c]] * pn2[c] + I.B[pb[c]] * pq2[c] + c2[c] * eo[c];
                corr += pnew - pn2[c];
                if (!dry) {
                    real* pp = P + ((long long)pb[c] * 6 + c) * dvol + u;
                    pp[lv] = pn2[c];
                    *pp = pnew;
                }
            }
            for (unsigned m = rest[c]; m; m &= m - 1) {
                const int p = __ffs(m) - 1;
                real* pp = P + ((long long)p * 6 + c) * dvol + u;
                const real pn = *pp, pq = pp[lv];
                const real pnew = I.A[p] * pn + I.B[p] * pq + cf[3 + 3 * p + c] * eo[c];
                corr += pnew - pn;
                if (!dry) {
                    pp[lv] = pn;
                    *pp = pnew;
                }
            }
            En[c][o] = fma(-(d >= 0 ? I.dinv[d] : cf[c]), corr, ec[c]);
            if (!dry)
                if (real* rr = design_rec(I, d, n, c)) *rr -= corr;
        }
    }
    finish_block(step_blocks, dry, st);
}

long long lean_items(int nx, int ny, int nz, int zb) {
    return (long long)((nx + LX - 1) / LX) * ((ny + LY - 1) / LY) * ((nz + zb - 1) / zb);
}

template <typename real>
int lean_classify(const InstDev<real>& I, int zb, std::vector<unsigned>* lists) {
    const int ntx = (I.nx + LX - 1) / LX, nty = (I.ny + LY - 1) / LY, ntz = (I.nz + zb - 1) / zb;
    if (ntx > 512 || nty > 1024 || ntz > 1024) return -1;
    for (int c = 0; c < LEAN_CLASSES; ++c) lists[c].clear();
    for (int tz = 0; tz < ntz; ++tz)
        for (int ty = 0; ty < nty; ++ty)
            for (int tx = 0; tx < ntx; ++tx) {
                const int i0 = tx * LX, j0 = ty * LY, z0 = tz * zb, z1 = imin(I.nz, z0 + zb);
                const int m = tile_slab_mask(I, i0, j0, z0, z1);
                const int c = tile_has_hsource(I, i0, j0, z0, z1) || tile_has_design(I, i0, j0, z0, z1) ? LEAN_GENERAL
                              : m == 0                      ? LEAN_PLAIN
                              : (m == 1 || m == 2 || m == 4) ? LEAN_SLAB
                                                             : LEAN_MULTI;
                lists[c].push_back((unsigned)tx | ((unsigned)ty << 9) | ((unsigned)tz << 19) | ((unsigned)m << 29));
            }
    return 0;
}
template int lean_classify<float>(const InstDev<float>&, int, std::vector<unsigned>*);
template int lean_classify<double>(const InstDev<double>&, int, std::vector<unsigned>*);

namespace {

template <typename real>
long long probe_blocks(const InstDev<real>& I) {
    return (I.n_probe + LX * LY - 1) / (LX * LY);
}

// blocks of the step's general launch (at least one, so that every step
// has a block that advances the counter)
long long general_blocks(const LeanGen& gen, int dry) {
    return std::max(1LL, dry ? gen.n_tiles : gen.n_all);
}

}  // namespace

int lean_launches(const LeanTiles* tiles, const LeanGroup* groups, int n_groups, const LeanFix& fix) {
    int total = 1;  // the general launch
    for (int p = 0; p < LEAN_FIX_PASSES; ++p) total += fix.count[p] > 0;
    for (int g = 0; g < n_groups; ++g)
        for (int c = 0; c < LEAN_CLASSES; ++c)
            if (c != LEAN_GENERAL && tiles[groups[g].lead].count[c] > 0) ++total;
    return total;
}
template <typename real>
void lean_gen_blocks(const InstDev<real>* h_insts, const std::vector<unsigned>* general_tiles, int n_inst,
                     std::vector<int4>& blk, long long& n_tiles) {
    blk.clear();
    for (int q = 0; q < n_inst; ++q)
        for (unsigned code : general_tiles[q]) blk.push_back(make_int4(q, 0, (int)code, 0));
    n_tiles = (long long)blk.size();
    for (int q = 0; q < n_inst; ++q)
        for (long long c = 0; c < probe_blocks(h_insts[q]); ++c) blk.push_back(make_int4(q, 1, (int)c, 0));
}
template void lean_gen_blocks<float>(const InstDev<float>*, const std::vector<unsigned>*, int, std::vector<int4>&,
                                     long long&);
template void lean_gen_blocks<double>(const InstDev<double>*, const std::vector<unsigned>*, int,
                                      std::vector<int4>&, long long&);

template <typename real>
void lean_fix_blocks(const InstDev<real>* h_insts, int n_inst, std::vector<int2>* passes) {
    for (int p = 0; p < LEAN_FIX_PASSES; ++p) passes[p].clear();
    for (int q = 0; q < n_inst; ++q) {
        const InstDev<real>& I = h_insts[q];
        for (int s = 0; s < I.n_src; ++s) {
            if (I.src[s].comp >= 3) continue;
            const long long cells = (long long)I.src[s].n[0] * I.src[s].n[1] * I.src[s].n[2];
            for (long long b = 0; b * ESRC_CELLS < cells; ++b) passes[s].push_back(make_int2(q, (int)b));
        }
        if (I.n_poles > 0 && I.dvol > 0)
            for (long long b = 0; b * DISP_VOXELS < I.dvol; ++b)
                passes[SJ_MAX_SOURCES].push_back(make_int2(q, (int)b));
    }
}
template void lean_fix_blocks<float>(const InstDev<float>*, int, std::vector<int2>*);
template void lean_fix_blocks<double>(const InstDev<double>*, int, std::vector<int2>*);

// Each class of instance q goes to its own stream of set q % LEAN_SETS: the
// kernels of a step overlap and fill each other's tails.  Only as many sets
// as there are instances are forked.
template <typename real>
cudaError_t launch_lean_step(const InstDev<real>* h_insts, const InstDev<real>* d_insts,
                             const InstDev<real>* d_parity, const LeanTiles* tiles, const LeanGroup* groups,
                             int n_groups, const LeanGen& gen, const LeanFix& fix, int n_inst, int zb, int dry,
                             int cur, DevState* st, const LeanStreams& ls, int one_column,
                             const LeanQueue<real>* queue) {
    cudaError_t e = cudaSuccess;
    const bool fork = ls.side[0] != nullptr;
    const int nsets = fork ? (queue ? 1 : std::min(std::max(n_groups, 1), LEAN_SETS)) : 0;
    if (fork) {
        e = cudaEventRecord(ls.fork, ls.main);
        for (int q = 0; q < nsets * LEAN_CLASSES && e == cudaSuccess; ++q)
            e = cudaStreamWaitEvent(ls.side[q], ls.fork, 0);
        if (e != cudaSuccess) return e;
    }
    const long long gb = general_blocks(gen, dry);
    long long gtotal = gb;
    for (int p = 0; p < LEAN_FIX_PASSES; ++p) gtotal += fix.count[p];
    const dim3 block(LX, LY), halo(LX, LY + HALO_WARPS), halo2(LX, LY / 2 + 1);
    // descriptor of instance q with the step's parity applied
    auto table = [&](int q) {
        LeanTable<real> t;
        t.inst = h_insts[q];
        if (cur) {
            for (int c = 0; c < 6; ++c) std::swap(t.inst.F[0][c], t.inst.F[1][c]);
            for (int a = 0; a < 3; ++a) std::swap(t.inst.psiH[0][a], t.inst.psiH[1][a]);
        }
        t.dry = dry;
        t.step_blocks = (unsigned)gtotal;
        t.qvol = (unsigned)h_insts[q].vol;
        return t;
    };
    auto set_streams = [&](int s, cudaStream_t* sc) {
        for (int c = 0; c < LEAN_CLASSES; ++c) sc[c] = fork ? ls.side[(s % LEAN_SETS) * LEAN_CLASSES + c] : ls.main;
    };
    // queued: every group's plain, slab and multi tiles in one launch
    if (queue && queue->n_items) {
        cudaStream_t sc[LEAN_CLASSES];
        set_streams(0, sc);
        const LeanTable<real>* tabs = queue->tabs + (size_t)(dry ? 2 : 0) * queue->n_groups +
                                      (size_t)cur * queue->n_groups;
        LeanQueueParams<real> qp;
        memset(&qp, 0, sizeof(qp));
        for (int g = 0; g < queue->n_groups && g < LEAN_QUEUE_GROUPS; ++g) qp.t[g] = tabs[g];
        e = cudaMemsetAsync(queue->ctr, 0, sizeof(unsigned), sc[LEAN_MULTI]);
        const unsigned grid = (unsigned)std::min<long long>(queue->grid, queue->n_items);
        if (e == cudaSuccess) {
            if constexpr (sizeof(real) == 4) {
                switch (zb) {
                    case 8: k_lean_queue<real, 8><<<grid, halo2, 0, sc[LEAN_MULTI]>>>(qp, queue->items, queue->n_items, queue->ctr); break;
                    case 16: k_lean_queue<real, 16><<<grid, halo2, 0, sc[LEAN_MULTI]>>>(qp, queue->items, queue->n_items, queue->ctr); break;
                    case 32: k_lean_queue<real, 32><<<grid, halo2, 0, sc[LEAN_MULTI]>>>(qp, queue->items, queue->n_items, queue->ctr); break;
                    default: return cudaErrorInvalidValue;
                }
                e = cudaGetLastError();
            } else {
                e = cudaErrorInvalidValue;
            }
        }
    }
    // plain, slab and multi tiles: one launch per group and class, blockIdx.y = member
    for (int g = 0; g < n_groups && e == cudaSuccess && !queue; ++g) {
        LeanTable<real> t = table(groups[g].lead);
        const LeanTiles& T = tiles[groups[g].lead];
        const unsigned gn = (unsigned)groups[g].n;
        // plain tiles: two columns per thread where rows are whole
        const bool pairs = !one_column && t.inst.nx % LX == 0;
        // CPML tiles too in FP32; FP64 keeps one column per thread (its
        // two-column bodies need 152-168 registers: 2 blocks per SM, slower)
        const bool pairs2 = pairs && sizeof(real) == 4;
        cudaStream_t sc[LEAN_CLASSES];
        set_streams(g, sc);
#define SJ_ZB(Z)                                                                                             \
    case Z:                                                                                                  \
        t.tiles = T.list[LEAN_MULTI], t.n_tiles = T.count[LEAN_MULTI];                                       \
        if constexpr (sizeof(real) == 4)                                                                     \
            if (t.n_tiles && pairs2)                                                                         \
                k_lean_multi2<real, Z><<<dim3((unsigned)t.n_tiles, gn), halo2, 0, sc[LEAN_MULTI]>>>(t);      \
        if (t.n_tiles && !pairs2)                                                                            \
            k_lean_multi<real, Z><<<dim3((unsigned)t.n_tiles, gn), halo, 0, sc[LEAN_MULTI]>>>(t);            \
        t.tiles = T.list[LEAN_SLAB], t.n_tiles = T.count[LEAN_SLAB];                                         \
        if constexpr (sizeof(real) == 4)                                                                     \
            if (t.n_tiles && pairs2)                                                                         \
                k_lean_slab2<real, Z><<<dim3((unsigned)t.n_tiles, gn), halo2, 0, sc[LEAN_SLAB]>>>(t);        \
        if (t.n_tiles && !pairs2)                                                                            \
            k_lean_slab<real, Z><<<dim3((unsigned)t.n_tiles, gn), halo, 0, sc[LEAN_SLAB]>>>(t);              \
        t.tiles = T.list[LEAN_PLAIN], t.n_tiles = T.count[LEAN_PLAIN];                                       \
        if (t.n_tiles && pairs)                                                                              \
            k_lean_plain2<real, Z><<<dim3((unsigned)t.n_tiles, gn), halo2, 0, sc[LEAN_PLAIN]>>>(t);          \
        if (t.n_tiles && !pairs)                                                                             \
            k_lean_plain<real, Z><<<dim3((unsigned)t.n_tiles, gn), block, 0, sc[LEAN_PLAIN]>>>(t);           \
        break;
        switch (zb) {  // z-segment length
            SJ_ZB(8)
            SJ_ZB(16)
            SJ_ZB(32)
            default: return cudaErrorInvalidValue;
        }
#undef SJ_ZB
        e = cudaGetLastError();
    }
    // general tiles (H sources) and probe blocks of all instances: one launch
    if (e == cudaSuccess) {
        cudaStream_t sc[LEAN_CLASSES];
        set_streams(0, sc);
        const long long nb = dry ? gen.n_tiles : gen.n_all;
        switch (zb) {
#define SJ_GEN(Z)                                                                                       \
    case Z:                                                                                             \
        k_lean_general<real, Z><<<(unsigned)gb, block, 0, sc[LEAN_GENERAL]>>>(d_parity, gen.blk, nb, n_inst, \
                                                                             cur, dry, (unsigned)gtotal, st); \
        break;
            SJ_GEN(8)
            SJ_GEN(16)
            SJ_GEN(32)
#undef SJ_GEN
            default: return cudaErrorInvalidValue;
        }
        e = cudaGetLastError();
    }
    if (fork) {
        for (int q = 0; q < nsets * LEAN_CLASSES && e == cudaSuccess; ++q) {
            e = cudaEventRecord(ls.join[q], ls.side[q]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ls.main, ls.join[q], 0);
        }
    }
    for (int p = 0; p < LEAN_FIX_PASSES && e == cudaSuccess; ++p) {
        if (!fix.count[p]) continue;
        const unsigned nb = (unsigned)fix.count[p];
        if (p < SJ_MAX_SOURCES)
            k_lean_esrc<real><<<nb, FIX_THREADS, 0, ls.main>>>(d_insts, fix.blk[p], p, cur, (unsigned)gtotal, dry, st);
        else
            k_lean_disp<real><<<nb, FIX_THREADS, 0, ls.main>>>(d_insts, fix.blk[p], cur, (unsigned)gtotal, dry, st);
        e = cudaGetLastError();
    }
    return e;
}

template cudaError_t launch_lean_step<double>(const InstDev<double>*, const InstDev<double>*,
                                              const InstDev<double>*, const LeanTiles*, const LeanGroup*, int,
                                              const LeanGen&, const LeanFix&, int, int, int, int, DevState*,
                                              const LeanStreams&, int, const LeanQueue<double>*);
template cudaError_t launch_lean_step<float>(const InstDev<float>*, const InstDev<float>*, const InstDev<float>*,
                                             const LeanTiles*, const LeanGroup*, int, const LeanGen&,
                                             const LeanFix&, int, int, int, int, DevState*, const LeanStreams&,
                                             int, const LeanQueue<float>*);
}  // namespace sj
