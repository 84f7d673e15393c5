// Internal structures shared by the host driver (sj_host.cu) and the
// kernels (sj_step.cu, sj_raster.cu).  Nothing here crosses the C ABI.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/sj.h"

namespace sj {

constexpr int MAXP = SJ_MAX_POLES;
constexpr int MAXS = SJ_MAX_SOURCES;

// Row pitch of every per-voxel array, in elements.  Rows start on 128-byte
// boundaries for FP32 and 256-byte boundaries for FP64.
constexpr int PITCH_ALIGN = 32;

// One separable source stencil: J(i,j,k,n) = tab[n] * w0[i-lo0] * w1[j-lo1] * w2[k-lo2],
// with tab[n] = dt * Re[amp * current(t_n)] precomputed on the host in FP64.
template <typename real>
struct SrcDev {
    int comp;            // SJ_EX..SJ_HZ
    int lo[3], n[3];     // index box on the component's own Yee grid
    const real* w[3];    // per-axis weights
    const double* tab;   // [steps]
};

// The first monitor sample that tripped the divergence guard, written by the
// probe that found it into host-mapped pinned memory, so the host sees it
// without synchronising the stream.  flag is written last.
struct GuardRecord {
    int flag;                   // 1 once a sample tripped the guard
    int inst;                   // instance
    int monitor;                // monitor column
    int _pad;
    long long step;             // the step the sample was taken before
    double value;               // the sample
};

// Device-side view of one simulation instance.
template <typename real>
struct InstDev {
    int nx, ny, nz, px;         // px = row pitch (elements), >= nx
    long long plane, vol;       // px*ny, px*ny*nz
    real S;                     // Courant number dt/dx
    double dt;
    real* F[2][6];              // [ping-pong][Ex..Hz]

    // materials: one byte per voxel selects a "combo" = (class at Ex, Ey, Ez)
    const uint8_t* combo;       // [nz][ny][px]
    const real* coef;           // [n_combos][ncoef]: inv_eps[3], Csig[p][3], then S * inv_eps[3]
    const uint8_t* cflag;       // [n_combos]: bit 0 = some pole has sigma != 0
    const uint32_t* pmask;      // [n_combos]: bit 8 c + p = pole p has C sigma != 0 at E component c
    int n_combos, ncoef;
    int n_poles;
    real A[MAXP], B[MAXP];

    // polarisation storage, dense over the bounding box of dispersive voxels
    int dlo[3], dn[3];
    long long dvol;
    real* P;                    // [n_poles][2 levels: n, n-1][3 comps][dvol]

    // CPML: slab thickness (cells) per axis and face, profiles, psi storage.
    // psi arrays share the field layout ([nz][ny][px] per component) so a
    // voxel's psi sits at the same offset as its fields; only axes with a
    // slab allocate them, and only slab voxels are ever read or written.
    int pl[3], ph[3];
    const real* prof[3];        // per axis: b_int[n], c_int[n], b_half[n], c_half[n]
    real* psiE[3];              // per axis: [2 comps][vol]
    real* psiH[2][3];           // [ping-pong][axis]: [2 comps][vol]

    int n_src;
    SrcDev<real> src[MAXS];

    // probes (monitors and DFT points)
    int n_probe, n_mon, n_dft, n_freq, save_span;
    const int* probe_comp;      // [n_probe]
    const long long* probe_idx; // [n_probe][8] element offsets, -1 = outside
    const double* probe_w;      // [n_probe][8]
    const int* probe_mon;       // [n_probe] monitor column or -1
    const int* probe_dft;       // [n_probe] DFT row or -1
    const double* freqs;        // [n_freq]
    double* mon;                // [mon_cap][n_mon]
    long long mon_cap;
    double2* dft;               // [n_dft][n_freq]

    // design region (adjoint): per-voxel inverse eps at the voxel's E points,
    // and, while a segment is re-run, the E-update acc recorded there
    const real* dinv;           // [des_n2][des_n1][des_n0], null without a design region
    int des_lo[3], des_n[3];
    real* rec_acc;              // [step - rec_t0][design voxel][3], null when not recording
    long long rec_t0, rec_len;

    // fused schedule: TMA descriptors and tiling
    const void* tmap;           // 31 CUtensorMap: E[b][c], H[b][c], combo, psiE[a][p], psiH[b][a][p]
    int f_ntx, f_nty, f_nzs, f_zs;  // tiles in x, y; z segments and their length

    // divergence guard: a monitor sample with |v| > guard_bound, or not
    // finite, is recorded once per sim (guard_bound = 0: off)
    int index;                  // this instance's index in its sim
    double guard_bound;
    int* guard_flag;            // device word electing the one recorder
    GuardRecord* guard;         // host-mapped record (device address)
};

// Step counter and status kept in device memory so that graph replays need
// no per-launch arguments.
struct DevState {
    long long step;     // absolute step index n of the next step
    unsigned int done;  // blocks finished in the current launch
    int cur;            // ping-pong buffer holding E^n, H^{n-1/2}
    int status;         // sticky error code set by kernels (0 = fine)
    int _pad;
};

// Launch helpers implemented in sj_step.cu.
template <typename real>
cudaError_t launch_probe(const InstDev<real>* d_insts, const InstDev<real>* h_insts, int n_inst,
                         DevState* st, cudaStream_t s);
long long split_block_count_f64(const InstDev<double>& I);
long long split_block_count_f32(const InstDev<float>& I);
template <typename real>
cudaError_t launch_split_step(const InstDev<real>* d_insts, const InstDev<real>* h_insts,
                              int n_inst, DevState* st, cudaStream_t s);
// Fused schedule launch description (host side).
struct FusedLaunch {
    int ty;                     // TMA schedule: tile height; lean schedule: z-segment length
    int ring;                   // TMA ring depth (planes)
    long long n_items;          // stepping blocks (tiles x z segments)
    long long n_probe_blocks;   // probe blocks after them
    const long long* d_item_pre;   // [n_inst + 1] prefix of stepping blocks
    const long long* d_probe_pre;  // [n_inst + 1] prefix of probe blocks
    int dry;                    // 1 = time only: no step advance, no in-place stores
    int stall;                  // test hook: block 0 never fetches its second plane
    unsigned long long wait_ns; // limit of a wait on a TMA copy (0 = the default 100 ms)
};
template <typename real>
cudaError_t launch_fused_step(const InstDev<real>* d_insts, int n_inst, DevState* st,
                              const FusedLaunch& fl, cudaStream_t s);
// Fused (lean) schedule.  Tiles (32 x 8 columns x zb planes) fall into four
// classes by what their footprint touches: CPML slabs of no axis (plain),
// of one axis (slab) or of several (multi), or an H source (general).  E
// sources and polarisations are corrections applied after the tiles.  The
// plain, slab and multi tiles of a group of instances (LeanGroup) run as one
// launch per class, blockIdx.y = member; general tiles as one launch per
// instance.  A launch carries its descriptor as a kernel parameter.
enum { LEAN_PLAIN = 0, LEAN_SLAB = 1, LEAN_MULTI = 2, LEAN_GENERAL = 3, LEAN_CLASSES = 4 };
template <typename real>
struct LeanTable {
    InstDev<real> inst;         // slot 0 of F / psiH = current buffers, slot 1 = next
    const unsigned* tiles;      // device list: tx | ty << 9 | tz << 19 | slab mask << 29
    long long n_tiles;          // tiles of this launch (general: probe blocks follow)
    int dry;                    // 1 = time only: no step advance, no in-place stores
    unsigned step_blocks;       // general-launch blocks of the whole step
    unsigned qvol;              // group member r's fields at + r * qvol elements, psi at + 2 r * qvol
};
// Instances whose tile kernels share launches: equal grid, time step, CPML
// profiles, coefficient table and H-source boxes (hence equal tile lists),
// with every field, combo and psi array of member r at a fixed offset from
// the lead's: r * vol elements (fields, combo), r * 2 * vol (psi).  Member
// 0 is the lead; the host keeps which instance is member r.
struct LeanGroup {
    int lead;
    int n;
};
// Device tile lists of one instance, by class.
struct LeanTiles {
    const unsigned* list[LEAN_CLASSES];
    long long count[LEAN_CLASSES];
};
long long lean_items(int nx, int ny, int nz, int zb);  // tiles of one instance
template <typename real>
int lean_classify(const InstDev<real>& I, int zb, std::vector<unsigned>* lists);  // -1: grid too large
// Correction passes after the tile kernels: E sources (one pass per source
// slot), then polarisations; blk[b] = (instance, block of that instance).
constexpr int LEAN_FIX_PASSES = SJ_MAX_SOURCES + 1;
struct LeanFix {
    const int2* blk[LEAN_FIX_PASSES];
    long long count[LEAN_FIX_PASSES];
};
template <typename real>
void lean_fix_blocks(const InstDev<real>* h_insts, int n_inst, std::vector<int2>* passes);
// The general launch of a step: one block per H-source tile and per probe
// block of every instance.  blk[b] = (instance, 0, tile code) or (instance,
// 1, probe chunk); the tiles come first, so a dry launch takes the first
// n_tiles entries.  Descriptors come from a device table holding every
// instance twice, by parity (entry cur * n_inst + q has slot 0 = buffer cur).
struct LeanGen {
    const int4* blk;
    long long n_tiles, n_all;
};
template <typename real>
void lean_gen_blocks(const InstDev<real>* h_insts, const std::vector<unsigned>* general_tiles, int n_inst,
                     std::vector<int4>& blk, long long& n_tiles);
int lean_launches(const LeanTiles* tiles, const LeanGroup* groups, int n_groups, const LeanFix& fix);
// Streams of one fused step: LEAN_SETS sets of one stream per tile class,
// forked from `main` and joined back into it with the events; group g's
// launches go to set g % LEAN_SETS (instance q's general launch to set
// q % LEAN_SETS), so the launches of many groups overlap (side streams
// null: all on `main`).
constexpr int LEAN_SETS = 4;
constexpr int LEAN_STREAMS = LEAN_SETS * LEAN_CLASSES;
struct LeanStreams {
    cudaStream_t main;
    cudaStream_t side[LEAN_STREAMS];
    cudaEvent_t fork, join[LEAN_STREAMS];
};
// Queued launch of the fused schedule (FP32, every instance with whole
// 32-column rows): the plain, slab and multi-slab tiles of every group in one
// launch of resident blocks that claim tiles from a counter, multi-slab tiles
// first, then single-slab, then plain.
constexpr int LEAN_QUEUE_GROUPS = 16;  // most launch groups one queued launch takes
template <typename real>
struct LeanQueueParams {          // kernel parameter: every group's descriptor
    LeanTable<real> t[LEAN_QUEUE_GROUPS];
};
template <typename real>
struct LeanQueue {
    const LeanTable<real>* tabs;   // host [dry][parity][group]: the descriptors with the parity applied
    const uint4* items;            // (group, member, tile code, 0) in claiming order
    unsigned n_items;
    unsigned* ctr;                 // items claimed; zeroed before each launch
    int n_groups;
    int grid;                      // resident blocks per SM x SMs
};
int lean_queue_blocks_per_sm(int zb);   // occupancy of the queued kernel (FP32)
template <typename real>
cudaError_t launch_lean_step(const InstDev<real>* h_insts, const InstDev<real>* d_insts,
                             const InstDev<real>* d_parity, const LeanTiles* tiles, const LeanGroup* groups,
                             int n_groups, const LeanGen& gen, const LeanFix& fix, int n_inst, int zb, int dry,
                             int cur, DevState* st, const LeanStreams& ls, int one_column = 0,
                             const LeanQueue<real>* queue = nullptr);
template <typename real>
int fused_box_width();          // TMA box width in elements (x)
template <typename real>
int fused_box_xoff();           // box starts at i0 - xoff
int fused_block_threads(int ty);  // threads per block (= probes per probe block)
int fused_tensor_maps();          // CUtensorMap slots per instance
template <typename real>
int fused_smem_bytes(int ty, int ring);  // dynamic shared memory of a tiling, -1 if unsupported
constexpr int FUSED_MAX_SMEM = 227 * 1024;
template <typename real>
cudaError_t launch_max_abs_e(const InstDev<real>& h_inst, int buf, double* d_out, cudaStream_t s);

// Adjoint (sj_adjoint.cu): the transposed step of one instance.
template <typename real>
struct AdjDev {
    InstDev<real> I;            // coefficients, geometry, design region
    real* eb[3];                // dF/dE
    real* hb[3];                // dF/dH
    real* t1[3];                // per component: adjoint of its first difference (E update)
    real* t2[3];                // ... and of its second
    real* t3[3];                // the same for the H update's differences
    real* t4[3];
    real* psEb[3];              // [axis] -> [2 slots][vol] (null where the axis has no slab)
    real* psHb[3];
    real* pb;                   // polarisation layout: level 0 = dF/dP^n, level 1 = dF/dP^{n-1}
    const real* rec;            // E-update acc at the design points, [step - rec_t0][d][3]
    long long rec_t0;
    double* g;                  // dF/d(inverse eps) at the design points [d][3]
};
// Adjoint step n: the E update's transpose (first = false: with step n+1's
// gather into dF/dE folded in) and the H update's.
template <typename real>
cudaError_t launch_adjoint_step(const AdjDev<real>& a, long long n, bool first, cudaStream_t s);
// Objective DFT of one instance: D[q][c] += dt E_c^n(cell q) e^{i 2 pi f n dt}
// (sample = true, from buffer cur) or dF/dE^n source into eb (sample = false).
template <typename real>
cudaError_t launch_objective(const InstDev<real>& I, int cur, const int* d_cells, int n_cells, int comp_mask,
                             double freq, double2* d_D, long long n, bool sample, real* const* eb, cudaStream_t s);

// Diagnostics (sj_diag.cu): the discrete energy (scale * sum, partial sums in
// d_partial[energy_partials()]) and the flux spectrum of DFT-probe rows.
int energy_partials();
template <typename real>
cudaError_t launch_energy(const InstDev<real>& h_inst, int cur, double scale, double* d_partial, double* d_out,
                          cudaStream_t s);
cudaError_t launch_flux(const double2* d_dft, int n_freq, const int* d_rows, int n_pts, double dA, double* d_out,
                        cudaStream_t s);

// Phase extraction (sj_phases.cu): series q at d_v[q * s_series + k * s_sample],
// k < N, times d_t[N]; per-series workspace phase_workspace(N) doubles.
long long phase_workspace(int N);
cudaError_t launch_phases(const double* d_v, long long s_series, long long s_sample, int n_series, int N,
                          const double* d_t, double lowpass_inc, double* d_work, sj_phase_result* d_out,
                          cudaStream_t s);

// Monitor spectra (sj_spectrum.cu): out[monitor][np][re, im] from the
// monitor buffer mon[sample][n_mon] (n samples, np = 2^floor(log2 n)).
cudaError_t launch_spectrum(const double* d_mon, int n_mon, long long n, long long np, double* d_out, cudaStream_t s);

// Launch helpers implemented in sj_raster.cu.
cudaError_t launch_rasterize(const sj_csg_node* d_nodes, const int* d_region_start,
                             int n_regions, int nx, int ny, int nz, double dx,
                             const double* origin, uint8_t* d_masks, long long mask_pitch_elems,
                             int px, cudaStream_t s);
// smoothing: per-point region counts packed 8 bits per region (keys, pitched
// [3][pitch]), distinct keys into a set of cap slots, then key -> class byte
constexpr unsigned SMOOTH_SET_CAP = 4096;
cudaError_t launch_rasterize_counts(const sj_csg_node* d_nodes, const int* d_region_start, int n_regions,
                                    int nx, int ny, int nz, double dx, const double* origin,
                                    const double* d_offs, int n_offs, unsigned long long* d_keys,
                                    long long key_pitch_elems, int px, unsigned long long* d_set,
                                    unsigned cap, int* d_overflow, cudaStream_t s);
cudaError_t launch_class_assign(const unsigned long long* d_keys, long long pitch, int nx, int ny, int nz,
                                int px, const unsigned long long* d_sorted, int n_keys, uint8_t* d_cls,
                                cudaStream_t s);
cudaError_t launch_combo_mark(const uint8_t* d_cls, long long cpitch, int nx, int ny, int nz,
                              int px, uint32_t* d_bitmap, cudaStream_t s);
cudaError_t launch_combo_compact(const uint32_t* d_bitmap, int n_words, uint32_t* d_keys, int cap, int* d_count,
                                 cudaStream_t s);
cudaError_t launch_combo_assign(const uint8_t* d_cls, long long cpitch, int nx, int ny, int nz,
                                int px, const uint32_t* d_keys, int n_keys, uint8_t* d_combo,
                                cudaStream_t s);
cudaError_t launch_combo_hist(const uint8_t* d_combo, int nx, int ny, int nz, int px,
                              unsigned long long* d_hist, cudaStream_t s);
int rasterize_static(const sj_grid_desc* g, const sj_scene_desc* sc, uint8_t* d_out, cudaStream_t s,
                     const char** msg);
cudaError_t launch_disp_bbox(const uint8_t* d_combo, const uint8_t* d_cflag, int nx, int ny,
                             int nz, int px, int* d_box, cudaStream_t s);

}  // namespace sj
