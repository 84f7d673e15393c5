/*
 * sj.h — C ABI of the sim_juncs GB300 FDTD stepper.
 *
 * This library replaces the meep::fields object that sim_juncs' bound_geom
 * owns (src/disp.hpp:175-177) and the time loop that drives it
 * (bound_geom::run, src/disp.cpp:690-749).  Every entry point below names the
 * reference call it stands in for.
 *
 * Conventions
 *   - plain C, no exceptions cross the ABI; every call returns an int status:
 *     0 = success, negative = error (SJ_E_*), with a message from
 *     sj_last_error(sim) (or sj_last_error(NULL) after a failed create);
 *   - device memory is owned by the library, host arrays by the caller;
 *   - units are meep units: lengths in "a" (= 1/um_scale um), c = 1,
 *     frequencies in c/a, times in a/c;
 *   - field arrays exchanged with the host are [nz][ny][nx], x fastest.
 *
 * Discretisation (the definition the CPU oracle and the kernels share)
 *   Integer Yee point (i,j,k) sits at origin + (i,j,k)*dx.  Component
 *   offsets, in units of dx: Ex(1/2,0,0) Ey(0,1/2,0) Ez(0,0,1/2)
 *   Hx(0,1/2,1/2) Hy(1/2,0,1/2) Hz(1/2,1/2,0).  Values outside the
 *   nx*ny*nz arrays are zero.  mu = 1, so B = H and no B array exists.
 *   One step n -> n+1 (S = dt/dx):
 *     H^{n+1/2} = H^{n-1/2} - S*curl_fwd(E^n) [+ CPML psi] - dt*M
 *     P_p^{n+1} = A_p P_p^n + B_p P_p^{n-1} + C_p sigma_p E^n
 *     E^{n+1}   = E^n + eps_inf^{-1} ( S*curl_bwd(H^{n+1/2}) [+ CPML psi]
 *                                     - dt*J^{n+1/2} - sum_p (P_p^{n+1}-P_p^n) )
 *   with meep's Lorentzian form A_p = (2 - w^2 dt^2 L)/(1+g dt/2),
 *   B_p = -(1 - g dt/2)/(1+g dt/2), C_p = w^2 dt^2/(1+g dt/2),
 *   w = 2 pi omega_0, g = 2 pi gamma, L = 0 for Drude (no omega_0
 *   denominator) and 1 for Lorentz.  Monitors sample E^n before step n when
 *   n % save_span == 0 (src/disp.cpp:721); DFT sums accumulate
 *   dt * F(t) * exp(+i 2 pi f t) over every step, t = n dt for E probes and
 *   (n - 1/2) dt for H probes.
 */
#ifndef SJ_H
#define SJ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* raised whenever a struct layout or a signature changes; 2: sj_scene_desc
   gained smooth_n and smooth_rad; 3: the divergence guard, bounded-wait,
   energy, flux, phase-extraction and fused launch-mode entry points and
   sj_phase_result */
#define SJ_ABI_VERSION 3

/* status codes */
#define SJ_OK 0
#define SJ_E_INVALID (-1)   /* bad argument or descriptor */
#define SJ_E_CUDA (-2)      /* a CUDA runtime/driver call failed */
#define SJ_E_NOMEM (-3)     /* device or host allocation failed */
#define SJ_E_RANGE (-4)     /* index / capacity out of range */
#define SJ_E_DIVERGED (-5)  /* field exceeded the divergence guard */
#define SJ_E_TIMEOUT (-6)   /* a bounded device wait gave up */

/* field components, same order as meep's Ex..Hz (src/disp.cpp:334-344) */
enum { SJ_EX = 0, SJ_EY = 1, SJ_EZ = 2, SJ_HX = 3, SJ_HY = 4, SJ_HZ = 5 };

/* precision of fields, polarisations and CPML auxiliaries; DFT and
   monitor sums are always FP64 */
enum { SJ_F64 = 0, SJ_F32 = 1 };

/* kernel schedule: FUSED is the single-HBM-pass leapfrog kernel (tiles of
   (i,j) columns marching z, neighbour H passed between warps or recomputed,
   instances with equal grids sharing launches); SPLIT the two-pass (H then
   E) schedule; TMA the single-pass kernel that stages tiles through a
   TMA/mbarrier shared-memory ring.  Default: FUSED for both precisions (the
   fastest on GB300 for both).  FUSED and SPLIT apply design regions
   (adjoint); TMA does not, and a TMA sim moves to FUSED when a design
   region is set */
enum { SJ_SCHED_FUSED = 0, SJ_SCHED_SPLIT = 1, SJ_SCHED_TMA = 2 };

#define SJ_MAX_POLES 8
#define SJ_MAX_SOURCES 4
#define SJ_MAX_REGIONS 8
#define SJ_MAX_CSG_NODES 256

/* ---------------------------------------------------------------- grid */
/* meep::vol3d(L, L, L, res) built in structure_from_settings
   (src/disp.cpp:505-510); nx = grid_num from correct_defaults
   (src/argparse.h:171-191), dx = 1/resolution.  dt <= 0 selects
   meep's default Courant factor 0.5 (dt = dx/2). */
typedef struct {
    int32_t nx, ny, nz;
    double dx;
    double dt;
    double origin[3];
} sj_grid_desc;

/* ---------------------------------------------------------------- materials */
/* one meep::lorentzian_susceptibility (src/disp.cpp:538-547): omega_0 and
   gamma already divided by um_scale, drude != 0 for no_omega_0_denominator */
typedef struct {
    double omega_0;
    double gamma;
    int32_t drude;
    int32_t _pad;
} sj_pole;

/* Flattened CSG program of one root composite_object, in postfix order:
   leaves push in(r) (0/1), composites pop two and push the combination.
   Mirrors composite_object::in and the primitives' in()
   (src/cgs.cpp:34-120, 403-449), in the same floating-point operation
   order (matrix rows summed left to right, no fused multiply-add).
     leaf point   r' = m * r             (m = product of the ancestors'
                                          trans_mat; exact when they are
                                          identities, as in every shipped
                                          junction file)
                  q  = t * (r' - c)      (t = the primitive's own trans_mat)
     SJ_CSG_BOX      |q_a| > p[a] for any a      -> invert, else 1-invert
     SJ_CSG_SPHERE   |q| > p[0]                  -> invert, else 1-invert
     SJ_CSG_CYLINDER q_z<0 || q_z>p[0] || (qx^2+qy^2)*p[0] > (p[2]-p[1])*q_z + p[1]*p[0]
                                                 -> invert, else 1-invert
                     (p[0] = height, p[1] = r1^2, p[2] = r2^2)
     SJ_CSG_PLANE    dot(r', p[0..2]) > p[3] -> 0 else 1
                     (plane::in ignores invert and its own trans_mat)
     SJ_CSG_UNION / SJ_CSG_INTERSECT   pop b, pop a, push invert ^ (a|b) / (a&b)
     SJ_CSG_PASS     pop a, push invert ^ a     (composite with one child)
     SJ_CSG_CONST    push invert                (composite with no child)
     SJ_CSG_NOOP     push 0                     (CGS_CMB_NOOP)
   Difference is emitted as INTERSECT with the right child's invert set, as
   composite_object::add_child does. */
enum {
    SJ_CSG_BOX = 0, SJ_CSG_SPHERE = 1, SJ_CSG_CYLINDER = 2, SJ_CSG_PLANE = 3,
    SJ_CSG_UNION = 4, SJ_CSG_INTERSECT = 5, SJ_CSG_PASS = 6, SJ_CSG_CONST = 7,
    SJ_CSG_NOOP = 8
};
typedef struct {
    int32_t op;
    int32_t invert;
    double m[9];   /* row-major 3x3, ancestors' transform */
    double t[9];   /* row-major 3x3, primitive's own transform */
    double c[3];
    double p[4];
} sj_csg_node;

/* one root of the scene: the region_scale_pair of cgs_material_function
   (src/disp.hpp:44-47) plus the root's susceptibilities */
typedef struct {
    int32_t n_nodes;
    const sj_csg_node* nodes;
    double eps;                 /* the root's "eps" metadata (scale s) */
    int32_t n_poles;
    const sj_pole* poles;       /* meep units */
    const double* sigma;        /* [n_poles], already divided by thickness */
} sj_region_desc;

/* cgs_material_function semantics (src/disp.cpp:264-283).
   SJ_EPS_SUM (the reference's behaviour):
     eps(r) = sum_roots [ambient + (s_root - ambient) * f_root(r)]
     (ambient alone when there is no root), so empty space carries
     n_roots * ambient;
   SJ_EPS_FIRST (what the comment at src/disp.cpp:271 describes):
     eps(r) = s of the first root containing r, else ambient.
   In both modes sigma_{root,q}(r) = sigma * f_root(r), except that under
   SJ_EPS_FIRST only the first containing root contributes poles.

   f_root is the fill fraction.  With smooth_n = 0 it is in_root(r) (0/1).
   With smooth_n > 0 (stochastic smoothing, SJ_EPS_SUM only) it is
     f_root(r) = (in_root(r) + sum_j in_root(r + d_j)) / (N + 1),
   N = 8 smooth_n, d_j the offsets sj_smooth_points returns: smooth_n draws
   of cgs_material_function::generate_smooth_pts (src/disp.cpp:56-112,
   std::mt19937 seeded as there with DEF_SEED = 0xd9a28bf3, src/disp.hpp:34),
   each reflected through the 8 octants.  Every Yee point's class is then the
   tuple of its per-root counts; a scene whose voxels carry more than 256
   distinct (Ex, Ey, Ez) class triples is rejected (SJ_E_INVALID). */
enum { SJ_EPS_SUM = 0, SJ_EPS_FIRST = 1 };
#define SJ_MAX_SMOOTH_N 31
typedef struct {
    double ambient_eps;
    int32_t n_regions;
    int32_t combine;            /* SJ_EPS_SUM (default) or SJ_EPS_FIRST */
    const sj_region_desc* regions;
    int32_t smooth_n;           /* 0 = off (the reference's default, src/argparse.h:40);
                                   1 .. SJ_MAX_SMOOTH_N */
    double smooth_rad;          /* standard deviation of the radial draw, length units
                                   (the reference's DEFAULT_SMOOTH_RAD is 0.05) */
} sj_scene_desc;

/* Material description: either an explicit per-component class map with a
   class table, or a scene rasterised on the device (class = bitmask of the
   regions containing the component's Yee point). */
typedef struct {
    /* explicit form (used when class_map != NULL) */
    int32_t n_classes;          /* <= 255 */
    const double* eps_inf;      /* [n_classes] */
    int32_t n_poles;            /* <= SJ_MAX_POLES */
    const sj_pole* poles;       /* [n_poles] */
    const double* sigma;        /* [n_classes][n_poles] */
    const uint8_t* class_map;   /* [3][nz][ny][nx]: class at Ex, Ey, Ez points */
    /* scene form (used when class_map == NULL) */
    const sj_scene_desc* scene;
} sj_material_desc;

/* ---------------------------------------------------------------- PML */
/* meep::pml(thickness) (src/disp.cpp:527): stretched-coordinate absorber on
   every face.  sigma(u) = sigma_max (u/d)^power, sigma_max chosen so the
   round-trip reflection at normal incidence is r_asymptotic. */
typedef struct {
    double thickness[3][2];     /* [axis][low, high] in length units */
    double r_asymptotic;        /* <= 0 -> 1e-15 (meep's default) */
    double power;               /* <= 0 -> 2 (meep's quadratic profile) */
    double alpha;               /* CFS frequency shift, 0 = none */
} sj_pml_desc;

/* ---------------------------------------------------------------- sources */
/* source_info + gaussian_src_time_phase / continuous_src_time as passed to
   fields.add_volume_source (src/disp.cpp:595-620).  Times and frequency in
   meep units (the fs -> meep conversion of src/disp.cpp:604-609 is the
   caller's, as in the reference).  The current density injected is
   Re[amplitude * (d(t) - d(t - dt)) / dt] * weight(r), d the dipole
   function, evaluated at t = (n + 1/2) dt for E-components and n dt for H. */
enum { SJ_SRC_GAUSSIAN = 0, SJ_SRC_CONTINUOUS = 1 };
typedef struct {
    int32_t component;
    int32_t kind;
    double frequency;
    double width;
    double phase;
    double start_time;
    double end_time;
    double amplitude[2];        /* complex (re, im) */
    double lo[3], hi[3];        /* source volume; zero extent -> sheet */
} sj_source_desc;

/* ---------------------------------------------------------------- probes */
/* fields.get_field(component, loc) at monitor points (src/disp.cpp:724),
   trilinear interpolation between the component's Yee points. */
enum { SJ_PROBE_MONITOR = 1, SJ_PROBE_DFT = 2 };
typedef struct {
    int32_t component;
    int32_t flags;              /* SJ_PROBE_MONITOR | SJ_PROBE_DFT */
    double pos[3];
} sj_probe_desc;

/* one simulation instance (one bound_geom) */
typedef struct {
    sj_grid_desc grid;
    sj_material_desc material;
    sj_pml_desc pml;
    int32_t n_sources;
    const sj_source_desc* sources;
    int32_t n_probes;
    const sj_probe_desc* probes;
    int32_t n_freqs;
    const double* freqs;        /* DFT frequencies (meep units) */
    int32_t save_span;          /* monitor sampling period (>= 1) */
} sj_instance_desc;

typedef struct sj_sim sj_sim;

/* ---------------------------------------------------------------- lifecycle */
int sj_abi_version(void);
/* sizeof of the descriptor structs above, in declaration order
   (0 = sj_grid_desc ... 9 = sj_instance_desc, 10 = sj_design_desc,
   11 = sj_objective_desc, 12 = sj_phase_result); -1 for an unknown index */
int64_t sj_abi_struct_size(int32_t which);
const char* sj_last_error(const sj_sim* sim);

/* fields(strct) + add_volume_source + parse_monitors
   (src/disp.cpp:557-645): builds one instance on the current device. */
int sj_create(const sj_instance_desc* inst, int32_t precision, sj_sim** out);

/* many independent instances stepped together (batched CEP/amplitude
   sweeps): instances with equal grid, CPML and materials share every tile
   launch of a step; instance i keeps its own grid, materials, PML, sources
   and probes. */
int sj_batch_create(int32_t n_instances, const sj_instance_desc* insts,
                    int32_t precision, sj_sim** out);

/* ~bound_geom / ~fields (src/disp.cpp:647-649) */
int sj_destroy(sj_sim* sim);

/* stream used by every later call (a cudaStream_t); NULL = the library's own */
int sj_set_stream(sj_sim* sim, void* cuda_stream);
int sj_set_schedule(sj_sim* sim, int32_t schedule);
/* the schedule in use (SJ_SCHED_*), -1 for a null handle */
int32_t sj_get_schedule(const sj_sim* sim);
int sj_synchronize(sj_sim* sim);

/* tiling of the single-pass schedules.  FUSED: blocks of 32 x 8 columns
   march z segments of zseg in {8, 16, 32} planes (tile_y, ring ignored).
   TMA: tiles of 32 x tile_y cells, a TMA ring of `ring` planes
   ((tile_y, ring) in {(4,3), (8,3), (16,3), (4,4), (8,4)}), z segments of
   zseg planes.  Applies to the schedule selected when it is called. */
int sj_set_tiling(sj_sim* sim, int32_t tile_y, int32_t ring, int32_t zseg);
int sj_get_tiling(const sj_sim* sim, int32_t* tile_y, int32_t* ring, int32_t* zseg);
/* FUSED: columns per thread in the tile kernels.  0 (default) = two where
   rows are whole (nx a multiple of 32; CPML tiles in FP32 only), 1 = one
   everywhere.  Both evaluate the same per-cell arithmetic in the same order:
   the results do not change. */
int sj_set_fused_columns(sj_sim* sim, int32_t columns);
/* FUSED: how a step's tile kernels are launched.  GROUPED (default): one
   launch per launch group and tile class (plain, single-slab, multi-slab),
   the launches of a step concurrent on forked streams.  QUEUE: one launch of
   resident blocks for every group's tiles, which claim (group, member, tile)
   items from a counter, multi-slab tiles first; FP32 with two columns per
   thread only (every instance's nx a multiple of 32), else the grouped
   launches run.  Both evaluate the same per-cell arithmetic: the results do
   not change.  sj_autotune tries both where QUEUE applies and keeps the
   faster. */
enum { SJ_LAUNCH_GROUPED = 0, SJ_LAUNCH_QUEUE = 1 };
int sj_set_fused_launch(sj_sim* sim, int32_t mode);
/* the launch mode in use (SJ_LAUNCH_*), -1 for a null handle */
int32_t sj_get_fused_launch(const sj_sim* sim);
/* time every fused tiling with `steps` launches that leave the state
   untouched, keep the fastest and report it (any output may be NULL) */
int sj_autotune(sj_sim* sim, int32_t steps, int32_t* tile_y, int32_t* ring, int32_t* zseg,
                float* ms_per_step);

/* ---------------------------------------------------------------- stepping */
/* n_steps iterations of the loop body at src/disp.cpp:719-741: sample
   monitors when step % save_span == 0, accumulate DFTs, then fields.step().
   Asynchronous on the sim's stream. */
int sj_step(sj_sim* sim, int64_t n_steps);

/* same, recorded once into a CUDA graph of `chunk` steps and replayed */
int sj_step_graph(sj_sim* sim, int64_t n_steps, int32_t chunk);

/* ---------------------------------------------------------------- queries */
int64_t sj_steps_done(const sj_sim* sim);
int32_t sj_n_instances(const sj_sim* sim);
/* fields.time() (src/disp.cpp:733) and fields.dt (src/disp.cpp:704) */
double sj_time(const sj_sim* sim, int32_t inst);
double sj_dt(const sj_sim* sim, int32_t inst);
/* fields.last_source_time() (src/disp.cpp:625) */
double sj_last_source_time(const sj_sim* sim, int32_t inst);
/* number of monitor samples taken so far (ceil(steps / save_span)) */
int64_t sj_n_samples(const sj_sim* sim, int32_t inst);
/* bytes this sim has copied host->device and device->host so far */
int sj_transfer_bytes(const sj_sim* sim, int64_t* h2d, int64_t* d2h);
/* per-instance voxel count and algorithmic bytes per step (roofline model) */
int64_t sj_voxels(const sj_sim* sim, int32_t inst);
double sj_bytes_per_step(const sj_sim* sim, int32_t inst);
/* kernel launches one sj_step step issues under the current schedule (GB300
   query; the reference has no counterpart) */
int32_t sj_launches_per_step(const sj_sim* sim);

/* ---------------------------------------------------------------- read-back */
/* field_times (src/disp.hpp:172): out[monitor][sample], monitor = order of
   the SJ_PROBE_MONITOR probes; cap = capacity in doubles */
int sj_read_monitors(sj_sim* sim, int32_t inst, double* out, size_t cap);
/* running DFT sums: out[dft_probe][freq][re, im] */
int sj_read_dft(sj_sim* sim, int32_t inst, double* out, size_t cap);
/* The spectrum save_field_times writes per monitor (src/disp.cpp:804, the
   fft of src/data_utils.cpp:413-427), computed on the device from the
   samples so far: of N samples the first N' = 2^floor(log2 N) are used and
   F_k = sum_{m<N'} x_m e^{-i 2 pi m k / N} for k = -N'/2 .. N'/2-1, stored
   at index k mod N'.  out[monitor][N'][re, im]; sj_monitor_spectrum_length
   gives N'. */
int64_t sj_monitor_spectrum_length(const sj_sim* sim, int32_t inst);
int sj_monitor_spectrum(sj_sim* sim, int32_t inst, double* out, size_t cap);
/* full component array converted to FP64 (dump_raw, src/disp.cpp:732-737) */
int sj_read_field(sj_sim* sim, int32_t inst, int32_t component, double* out, size_t cap);
/* dump_raw streamed (src/disp.cpp:732-737, `if (dump_raw)` inside the save
   point): every `every` steps, at the monitor rule (step n with
   n % every == 0, before step n runs), component `component` of instance
   `inst` is copied on the device into a dense [nz][ny][nx] staging slot and
   from there to pinned host memory on a copy stream of its own, overlapped
   with the steps that follow.  `depth` slots form a ring that
   sj_take_snapshot drains oldest first.  When a snapshot falls due and every
   slot still holds one not taken, sj_step / sj_step_graph stop before that
   step and return SJ_E_RANGE (the steps before it are done; sj_time tells
   where).  every = 0 switches snapshots off for the instance (pending ones
   are dropped).  While any instance takes snapshots, sj_step_graph launches
   step by step instead of replaying graphs. */
int sj_set_snapshots(sj_sim* sim, int32_t inst, int32_t component, int32_t every, int32_t depth);
/* the oldest snapshot not yet taken: waits for its copy, writes nx*ny*nz
   doubles ([nz][ny][nx]) to out and the step it was taken before to *step;
   *step = -1 (out untouched) when none is pending */
int sj_take_snapshot(sj_sim* sim, int32_t inst, int64_t* step, double* out, size_t cap);
/* snapshots in the ring not yet taken (in flight or copied); -1 on error */
int32_t sj_snapshots_pending(const sj_sim* sim, int32_t inst);
/* overwrite one component (initial conditions / checkpoint restore) */
int sj_write_field(sj_sim* sim, int32_t inst, int32_t component, const double* in, size_t n);
/* per-component class map the stepper uses: out[3][nz][ny][nx] */
int sj_read_class_map(sj_sim* sim, int32_t inst, uint8_t* out, size_t cap);
/* largest |E| over the instance (a full-grid query; the step loop's own
   guard is sj_set_divergence_guard) */
int sj_max_abs_e(sj_sim* sim, int32_t inst, double* out);

/* Bounded device waits (no counterpart in the reference).  The TMA schedule's
   kernels wait on mbarriers for their tile copies; a wait that does not end
   within the limit gives up, the block waits (bounded by 100 ms) for the
   copies it still has in flight and returns, and SJ_E_TIMEOUT is recorded:
   sj_synchronize (and every call that synchronises) then returns it.  The
   fields of that step are not valid.  ns = 0 restores the default of 100 ms
   (a healthy copy takes microseconds); at most 10 s. */
int sj_set_wait_limit(sj_sim* sim, int64_t ns);
/* Test hook for the bounded waits: while on, the first tile block of every
   TMA-schedule launch never fetches its second plane, so its wait on that
   plane runs out after the limit and the launch records SJ_E_TIMEOUT.  No
   other schedule is affected.  Off by default; for tests of a host's error
   handling only. */
int sj_set_test_stall(sj_sim* sim, int32_t on);

/* Discrete energy of instance inst in FP64 (the energy-conservation check;
   the reference has no counterpart):
     W = 1/2 dx^3 [ sum_E eps E^n E^n + sum_H H^{n-1/2} H^{n+1/2} ],
   eps the stepper's own eps_inf (the design region's per-voxel value inside
   it), H^{n+1/2} = H^{n-1/2} - S curl_fwd(E^n) formed on the fly.  For a
   closed cavity (no CPML, no source) of non-dispersive material the leapfrog
   conserves W exactly; its drift measures the arithmetic's rounding.
   Polarisation energy is not included.  Synchronises the sim's stream. */
int sj_energy(sj_sim* sim, int32_t inst, double* out);
/* Flux spectrum through a surface sampled by DFT probes (the flux DFT of the
   bowtie workload; meep's flux regions, which the reference does not use):
     out[f] = dA * sum_p Re( E1_p(f) conj(H2_p(f)) - E2_p(f) conj(H1_p(f)) )
   for every DFT frequency f; rows[p][4] are the DFT rows (the order of the
   SJ_PROBE_DFT probes) of the tangential components E1, E2, H1, H2 of one
   normal axis: x (Ey, Ez, Hy, Hz), y (Ez, Ex, Hz, Hx) or z (Ex, Ey, Hx, Hy),
   each quadruple at one point.  FP64 on the device; cap >= n_freqs. */
int sj_flux(sj_sim* sim, int32_t inst, int32_t n_points, const int32_t* rows, double dA, double* out,
            size_t cap);

/* Divergence guard of the time loop (src/disp.cpp:727-729, where
   bound_geom::run prints every monitor sample whose real part exceeds 1000).
   Every monitor sample is checked as it is taken, inside the probe kernels:
   the first sample of the sim with |value| > bound, or that is NaN or
   infinite, is recorded (step, instance, monitor, value) in host-mapped
   memory.  From then on sj_step and sj_step_graph return SJ_E_DIVERGED
   without queuing further steps, and sj_synchronize returns SJ_E_DIVERGED
   once the queued steps are done; every read-back still works.  Steps queued
   before the host saw the record still run.  bound = 0 switches the guard
   off; default 1000 (the reference's threshold, applied to |value| rather
   than to the real part only).  Setting a bound clears the record. */
int sj_set_divergence_guard(sj_sim* sim, double bound);
/* 1 and the record when the guard has tripped, 0 when not, -1 for NULL
   (any output may be NULL; reads the record without synchronising) */
int sj_divergence(const sj_sim* sim, int64_t* step, int32_t* inst, int32_t* monitor, double* value);

/* ---------------------------------------------------------------- adjoint */
/* Gradient of a gap-field objective with respect to per-voxel eps (the
   adjoint item of the replacement interface; the reference has no
   counterpart).

   Design region: a box of voxels whose eps_inf is given per voxel and
   applies at the voxel's Ex, Ey and Ez points (replacing the class table's
   value there; polarisations of the voxel's class still apply).  The
   FUSED and SPLIT schedules apply it; a sim on the TMA schedule moves to
   FUSED when a design region is set.

   Objective: F = sum over cells and over the E components in comp_mask of
   |D_c|^2 with D_c = sum_{n=0}^{N-1} dt E_c^n(cell) e^{+i 2 pi f n dt}, the
   running DFT of E sampled before each of the N steps (the probes'
   convention).

   sj_adjoint_gradient restarts every instance from zero fields at t = 0,
   runs N steps forward keeping the full state every checkpoint_every steps,
   then runs the discrete adjoint of the stepper backwards (the exact
   transpose of each sub-update: H and its CPML psi, E and its psi, the
   polarisation ADE), re-running each segment forward from its checkpoint
   to regenerate what the gradient needs.  d_obj_d_eps receives, instance
   after instance, dF/d(eps) for every design voxel ([n2][n1][n0] order);
   obj receives F per instance.  On return the instances hold the state
   after N steps.  Memory: (N / checkpoint_every + 1) copies of the full
   state (fields, CPML psi, polarisations) plus the E-update bracket at the
   design points for checkpoint_every steps; the work does not depend on
   the interval (each segment is re-run once).  checkpoint_every <= 0 or
   >= N keeps one segment: two state copies and the bracket of all N steps,
   the least memory whenever the design region is small.  An interval whose
   copies do not fit the free device memory fails with SJ_E_NOMEM; an
   instance of 2^31 voxels or more (row pitch included) with SJ_E_INVALID. */
typedef struct {
    int32_t lo[3];              /* first voxel of the design box */
    int32_t n[3];               /* extent in voxels */
    const double* eps;          /* [n[2]][n[1]][n[0]] eps_inf per voxel, > 0 */
} sj_design_desc;

typedef struct {
    int32_t n_cells;            /* cells of the objective patch */
    const int32_t* cells;       /* [n_cells][3] voxel indices (i, j, k) */
    int32_t comp_mask;          /* bit c: E component c (1 = Ex, 2 = Ey, 4 = Ez) */
    int32_t _pad;
    double frequency;           /* DFT frequency (meep units) */
} sj_objective_desc;

/* set (or replace) instance inst's design region; NULL removes it */
int sj_set_design(sj_sim* sim, int32_t inst, const sj_design_desc* design);
/* objectives[n_instances]; d_obj_d_eps holds every instance's design voxels */
int sj_adjoint_gradient(sj_sim* sim, const sj_objective_desc* objectives, int64_t n_steps,
                        int32_t checkpoint_every, double* d_obj_d_eps, size_t cap, double* obj);
/* the forward half alone: F per instance after n_steps from rest */
int sj_objective(sj_sim* sim, const sj_objective_desc* objectives, int64_t n_steps, double* obj);

/* ---------------------------------------------------------------- rasteriser */
/* cgs_material_function::in_bound per E-component Yee point, on the device:
   out_masks[3][nz][ny][nx] = bitmask of the scene regions containing the
   point (composite_object::in, src/cgs.cpp:403-449).  The scene's smooth_n
   must be 0 (a smoothed scene has fill counts: sj_rasterize_counts). */
int sj_rasterize(const sj_grid_desc* grid, const sj_scene_desc* scene, uint8_t* out_masks);
/* The fill counts behind f_root on the device: out_counts[3][n_regions][nz][ny][nx]
   = in_root(r) + sum_j in_root(r + d_j) at each E-component Yee point
   (cgs_material_function::in_bound's this_ret, src/disp.cpp:272-279), so
   0 .. 8 smooth_n + 1; with smooth_n = 0 the region's bit of sj_rasterize. */
int sj_rasterize_counts(const sj_grid_desc* grid, const sj_scene_desc* scene, uint8_t* out_counts);
/* The smoothing offsets (host): out[8 smooth_n][3], the reflections of each draw
   in the order of src/disp.cpp:95-104 (x sign outermost).  cap in doubles. */
int sj_smooth_points(int32_t smooth_n, double smooth_rad, double* out, size_t cap);

/* Allocation-free rasteriser (no counterpart in the reference).
   For callers that cannot call cudaMalloc: hosts whose device memory is
   handed out by a pool or caching allocator of their own (which may hold
   nearly all of the GPU, so an allocation by this library would fail or
   fragment it), and loops that must not stall on cudaMalloc/cudaFree, which
   synchronise the device.  Same result as sj_rasterize, but the caller
   passes the output as a DEVICE buffer d_out_masks[3][nz][ny][nx] and the
   kernel is queued on `stream` (a cudaStream_t; NULL = the legacy default
   stream).  The CSG program is copied from the caller's host arrays with
   cudaMemcpyAsync; from pageable memory CUDA lets that copy start only after
   the work already queued on `stream`, so the call may wait for it.  The
   program is staged in one library-owned static device array of
   SJ_RASTER_STATIC_NODES nodes in total (about 107 KB), which every GPU that
   loads the library holds until exit; larger scenes are rejected with
   SJ_E_RANGE.  The first call on a device (and the first after that device's
   context is created anew) looks up the array's address; make that first
   call before any stream capture.  All calls share the array and it keeps
   the last call's program: calls that overlap on the GPU (e.g. on two
   streams) race.  No cudaMalloc, cudaFree or other allocating routine is
   called. */
#define SJ_RASTER_STATIC_NODES 512
int sj_rasterize_static(const sj_grid_desc* grid, const sj_scene_desc* scene, uint8_t* d_out_masks,
                        void* stream);

/* ---------------------------------------------------------------- phase extraction */
/* CEP and envelope of monitor series, on the device: the reference's analysis
   class `signal` (scripts/phases.py:94-450) on the path its sweeps take,
   signal(t, v, lowpass_inc) then get_envelope() and get_skewness(), one
   thread block per series, FP64.  Per series: the t0 guess from the peaks of
   v^2; V = 2 rfft(v rolled to t0); f0 = the trapezoid mean frequency of |V|
   below twice its peak; sinc low-passes of strength lowpass_inc, 2
   lowpass_inc, ... (at most 4) while f0 sits above half the band or |V| has
   a prominent peak above 3 f0; the band where |V| > 0.1 |V(f0)|; a linear
   regression of the unwrapped phase there (t0_corr = -slope / 2 pi, phi =
   intercept wrapped to (-pi, pi]), recentred once when |t0_corr| > 2 / band
   width; the envelope from |V| / (2 pi f) symmetrised about f0 with the
   phase's odd-polynomial fit (solved as the linear least-squares problem the
   reference's curve_fit converges to), and its moments.  Where the
   reference raises, status says why and the fields computed before that
   point are kept. */
enum {
    SJ_PHASE_OK = 0,
    SJ_PHASE_NARROW_BAND = 1,   /* fewer than 5 band bins for the phase fit (curve_fit's TypeError):
                                   f0, phi, t0_corr and the band are valid */
    SJ_PHASE_EMPTY_BAND = 2,    /* zero-width band (the recentring test divides by it) */
    SJ_PHASE_BAD_F0 = 3,        /* no finite central frequency inside the spectrum */
    SJ_PHASE_BAD_T0 = 4,        /* recentring moved t0 outside the series */
    SJ_PHASE_WIDE_BAND = 5      /* a band of more than 256 bins (the kernel's fit size; the
                                   reference has no such limit) */
};
typedef struct {
    double f0;                  /* central frequency (signal.f0) */
    double phi;                 /* CEP: signal._phi_corr */
    double t0_corr;             /* signal._t0_corr */
    double t0;                  /* time of the largest |v| after filtering */
    double amp[2];              /* the envelope at its maximum (numpy's complex argmax) */
    double mu, sig, skew;       /* get_skewness: mean, width and skewness of |envelope| */
    int32_t f0_ind;             /* f0's bin */
    int32_t band_lo, band_hi;   /* the band [lo, hi) of the regression */
    int32_t lowpass_steps;      /* low-pass strengths applied */
    int32_t status;             /* SJ_PHASE_* */
    int32_t _pad;
} sj_phase_result;

/* n_series series of n_samples (8 .. 4096) values each, v[series][sample],
   sampled at t_pts[n_samples] (evenly spaced); results out[n_series].  Host
   arrays; device memory is allocated for the call. */
int sj_extract_phases(int32_t n_series, int32_t n_samples, const double* t_pts, const double* v,
                      double lowpass_inc, sj_phase_result* out);
/* Every monitor series of every instance of a sim, read where the stepper
   keeps them (no host round trip), instance after instance, monitors in
   probe order; sample k at time k save_span dt.  cap = entries of out. */
int sj_extract_monitor_phases(sj_sim* sim, double lowpass_inc, sj_phase_result* out, size_t cap);

/* ---------------------------------------------------------------- host helpers */
/* gaussian_src_time_phase::dipole (src/disp.cpp:378-400) / meep's
   continuous_src_time, and the current the stepper injects at time t */
int sj_source_dipole(const sj_source_desc* src, double t, double* re, double* im);
int sj_source_current(const sj_source_desc* src, double t, double dt, double* re, double* im);
/* gaussian_src_time_phase::last_time (src/disp.hpp:115) */
double sj_source_last_time(const sj_source_desc* src);

#ifdef __cplusplus
}
#endif
#endif /* SJ_H */
