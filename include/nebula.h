/*
 * nebula.h — C ABI of libnebula.so, the GB300 (sm_103a) implementation of the
 * NebulaViewer simulation step: isothermal-Euler MUSCL + HLL/Rusanov RK2 hydro with the
 * ionized-fraction sound-speed mix, the ray-cast Stromgren ionization front, the
 * dust-attenuated FUV field and the wind / jet sources.
 *
 * The reference exposes this path as a Python class, `Sim` (sim.py:543-1222), whose
 * methods launch NVIDIA-Warp kernels; it has no FFI of its own.  Each entry point below
 * names the reference method or kernel it replaces.  The Python drop-in
 * (nebulaviewer_gb300.Sim) binds them with ctypes.
 *
 * Conventions
 *   - Every call returns 0 (NB_OK) or a negative NB_ERR_* code and never aborts or traps;
 *     nb_last_error() describes the last failure of a handle (thread-local text for
 *     calls made without a handle).
 *   - Field buffers are CALLER-OWNED device memory (float32, C-order [i][j][k], k
 *     fastest, shape (nx, ny, nz)); the library owns its scratch (ray-front tables, the
 *     FUV attenuation grid, tensor maps, the per-instance control block) and its CUDA
 *     graphs.  Device pointers must be 16-byte aligned and nz a multiple of 4 (the
 *     reference's grid_shape rounds every axis to a multiple of 8).
 *   - A handle is used from one host thread at a time; work is enqueued on the stream
 *     given to nb_create (0 = the legacy default stream) and is asynchronous unless
 *     the call says otherwise.
 *   - The simulation clock (t, dt, it) lives in device memory: nothing in a step waits
 *     for the host, so steps can be captured and replayed as CUDA graphs.
 */
#ifndef NEBULA_GB300_H
#define NEBULA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NB_ABI_VERSION 2

enum {
    NB_OK = 0,
    NB_ERR_ARG = -1,        /* bad argument (null pointer, size, alignment) */
    NB_ERR_CUDA = -2,       /* a CUDA runtime call failed */
    NB_ERR_STATE = -3,      /* call not valid in the handle's current state */
    NB_ERR_LIMIT = -4,      /* a stated maximum was exceeded */
    NB_ERR_TIMEOUT = -5,    /* a bounded device-side wait gave up (see nb_device_status) */
    NB_ERR_NOMEM = -6       /* device allocation refused */
};

enum { NB_SOLVER_RUSANOV = 0, NB_SOLVER_HLL = 1 };
enum { NB_LIM_MINMOD = 0, NB_LIM_VANLEER = 1, NB_LIM_MC = 2 };
enum { NB_STAR_MAIN = 0, NB_STAR_ABS = 1 };                   /* sim.py:652 star kinds */
enum { NB_JET_JET = 0, NB_JET_PROTO = 1, NB_JET_NONE = 2 };   /* sim.py:653 jet kinds */

typedef struct nb_instance* nb_handle;

/* Fields of one simulation instance (all caller-owned device memory, nx*ny*nz cells).
 * The 40 B/cell layout of sim.py:718-735: rho, mx, my, mz, xi (float32), stage
 * (4 float32 planes: the RK2 stage between the two hydro kernels, scratch between steps),
 * dfront and g0 (float16, or float32 when fields_fp32 != 0). */
typedef struct nb_fields {
    float* rho;
    float* mx;
    float* my;
    float* mz;
    float* xi;
    float* stage;           /* 4 * nx*ny*nz floats */
    void* dfront;           /* __half, or float when fields_fp32 */
    void* g0;               /* __half, or float when fields_fp32 */
} nb_fields;

/* Static description of an instance: the values sim.py:Sim.reset computes (sim.py:591-795). */
typedef struct nb_desc {
    int abi_version;        /* NB_ABI_VERSION */
    int nx, ny, nz;
    double dx;              /* cell size; cell centres at (i + 1/2) dx from the origin */
    double cn2, ci2;        /* neutral / ionized sound speed squared (sim.py:740-741) */
    double floor_rho;       /* density floor (nebula3d.py:591) */
    double vmax;            /* velocity cap (sim.py:1020) */
    double cfl;             /* CFL number (nebula3d.py:589) */
    int solver;             /* NB_SOLVER_* (sim.py:1016) */
    int limiter;            /* NB_LIM_* (sim.py:1022); Rusanov always uses minmod */
    /* ionizing rays (sim.py:743-755) */
    int nu, nphi;
    double dr;              /* ray step: dx (fast) or dx/2 (bake) */
    int nsteps;             /* int(diag / dr) + 1 */
    double diag;            /* |L| + 0.6: the no-front radius rcap */
    /* FUV grid (sim.py:756-757) */
    int fnr, fnu, fnphi;
    int fields_fp32;        /* P['fp32_fields']: dfront / g0 stored as float32 */
    int max_stars;          /* star table capacity (sim.py:745 cap) */
    nb_fields f;
    void* stream;           /* cudaStream_t; 0 = legacy default stream */
} nb_desc;

/* Live parameters (sim.py:82-83 LIVE + the fixed jet geometry), read on device every step. */
typedef struct nb_live {
    double q_main, wind, jet, jet_proto, jet_pulse, jet_period, kappa_fuv, q_ramp;
    double jet_angle_deg, jet_r;
    double dt_cap;          /* Sim.dt_cap (bake.py:113); <= 0 means none */
    int phase_main;         /* 1 once the main phase started (sim.py:786, 816) */
    /* plane-parallel source on the -x face (no reference counterpart; 0 = off): ionizing flux F
     * against the column sum n^2 dx along +x, and FUV luminosity L giving G0 += L exp(-tau) */
    double plane_flux, plane_fuv;
    /* stirring amplitude (nebula3d.py:622 pre_amp) and its main-phase factor (nebula3d.py:625
     * drive_main): the stirring phase stirs with pre_amp, the main phase with pre_amp * drive_main
     * while drive_main > 0 and nb_drive_enable(h, 1) */
    double pre_amp, drive_main;
} nb_live;

/* One star: sim.py Sim.stars entry (x, y, z, qf, t_on) with its kind, and its jet axis. */
typedef struct nb_star {
    double x, y, z;
    double qf;              /* Q / q_main for NB_STAR_MAIN, absolute Q for NB_STAR_ABS */
    double t_on;
    double ax, ay, az;      /* jet axis (sim.py:713, Sim.jets) */
    int kind;               /* NB_STAR_* */
    int jkind;              /* NB_JET_* */
} nb_star;

/* Simulation clock (device-resident; sim.py Sim.t / Sim.dt / Sim.it, and the stirring
 * phase's Sim.tp / Sim.ip). */
typedef struct nb_clock {
    double t;
    double dt;
    int64_t it;
    double tp;
    int64_t ip;
} nb_clock;

/* ---------------------------------------------------------------- lifetime */
/* Replaces Sim.__init__/reset's buffer set-up (sim.py:718-759).  NB_ERR_LIMIT: max_stars outside
 * [1, 256], ny * nz or fnu * fnphi * fnr at 2^31 or more, or nu * nphi * max_stars or
 * fnu * fnphi * max_stars at 2^32 or more (ray indices are 32-bit). */
int nb_create(const nb_desc* desc, nb_handle* out);
/* Releases library scratch and graphs (never the caller's fields). */
void nb_destroy(nb_handle h);
/* No reference counterpart (the reference allocates through Warp and charges 40 B/cell of fields,
 * sim.py:79-87): the device bytes the library holds for an instance -- control blocks, tensor
 * maps, ray directions, the ray-front and FUV tables sized for the star table, the reduction and
 * culling scratch, the stirring ring -- beyond the caller's fields.  With h: what h holds now.
 * Without (h = NULL): what nb_create(d) followed by nb_set_stars(nstars) will allocate, for an
 * admission decision made before any allocation. */
int nb_instance_bytes(nb_handle h, const nb_desc* d, int nstars, long long* out);
const char* nb_last_error(nb_handle h);
int nb_device_status(nb_handle h, int* status);     /* bounded-wait failures seen on device */

/* ---------------------------------------------------------------- configuration */
/* Sim.P live parameters; replaces set_param's effect on the next step (sim.py:1154-1166). */
int nb_set_live(nb_handle h, const nb_live* live);
/* Star list; replaces replace_stars / the star part of reset (sim.py:1120-1133, 710-714).
 * The per-step weights of _set_star_weights (sim.py:914-925) are computed on device. */
int nb_set_stars(nb_handle h, const nb_star* stars, int n);
/* Sim.t / dt / it, as written by set_state_meta (sim.py:1185-1211). */
int nb_set_clock(nb_handle h, const nb_clock* c);
/* Synchronizes the stream.  Both clock reads return NB_ERR_TIMEOUT (the clock still filled in)
 * once a hydro stage's bounded TMA wait has given up on the device: the fields are incomplete. */
int nb_get_clock(nb_handle h, nb_clock* c);
/* Enqueues a copy of the clock into pinned host memory, in stream order (asynchronous). */
int nb_mirror_clock(nb_handle h);
/* The clock as of the last nb_mirror_clock (once the stream has passed it: the caller
 * synchronizes, as Sim.step(k) does after the steps and the mirror) or nb_set_clock: no
 * synchronization and no device access here. */
int nb_peek_clock(nb_handle h, nb_clock* c);

/* ---------------------------------------------------------------- the step */
/* k main-phase steps of Sim.step (sim.py:1141-1152 -> _main_step sim.py:1099-1114):
 * ionize when it % ion_every == 0, dt from the CFL max speed on device, the two RK2
 * hydro stages, t += dt.  Asynchronous. */
int nb_step(nb_handle h, int k, int ion_every);
/* Sim.ionize (sim.py:927-947): rays per active star, front apply, smoothing, fp16 dfront. */
int nb_ionize(nb_handle h);
/* Sim.fuv_field (sim.py:949-985): FUV rays per active star, G0 into g0. */
int nb_fuv(nb_handle h);
/* Marks the CFL max speed stale after the caller rewrote rho/m/xi (timeline restore). */
int nb_invalidate(nb_handle h);

/* ---------------------------------------------------------------- turbulent stirring
 * The stirring phase before the stars switch on and the optional main-phase stirring
 * (nebula3d.py:165-179 drive; sim.py:1030-1059 _stir / _pre_step; sim.py:1110-1111).  The
 * forcing is a cross-fade of two solenoidal fields A and B on a coarse grid: each stirred step
 * adds rho * amp * dt * ((1 - blend) A + blend B) to the momenta with blend = min(clock /
 * pre_corr, 1), then clock += dt; when the clock reaches pre_corr it restarts at 0, B becomes A
 * and the next field becomes B.  The caller generates the fields (sim.py:801-804) and pushes
 * them into a device ring ahead of use; the clock, the blend and the swaps are evaluated on the
 * device, so stirred steps need no host round trip.  The next step's CFL max speed is taken
 * over the stirred state (the drive kernel computes it; stage 2 then skips its own). */
typedef struct nb_drive_desc {
    int sx, sy, sz;         /* forcing grid (sim.py:761-768) */
    int slots;              /* ring capacity in fields, >= 3 */
    double dxs;             /* forcing grid spacing; sample points (i + 1/2) dx (nebula3d.py:172) */
    double pre_corr;        /* cross-fade time (nebula3d.py:623) */
    double clock;           /* cross-fade clock to start from (sim.py drv['clock']) */
} nb_drive_desc;

typedef struct nb_drive_info {
    double clock;           /* cross-fade clock */
    int64_t swaps;          /* fields retired so far: A is field `swaps`, B field `swaps + 1` */
    int64_t pushed;         /* fields pushed since nb_drive_config */
    int status;             /* device status bits (as nb_device_status; 2 = a step found no field B) */
    int pad;
} nb_drive_info;

/* (Re)configures the stirring: allocates the ring, empties it (swaps = 0), sets the clock.
 * Synchronizes. */
int nb_drive_config(nb_handle h, const nb_drive_desc* d);
/* Appends n forcing fields (host memory, n x [3][sx][sy][sz] float32: x, y, z components) in
 * the order they are to be used.  Synchronizes; NB_ERR_LIMIT when a field still to be used
 * would be overwritten (the ring holds fields swaps .. swaps + slots - 1). */
int nb_drive_push(nb_handle h, const float* fields, int n);
/* 1: main-phase steps stir (the reference's drv is not None, sim.py:1110); 0: they do not. */
int nb_drive_enable(nb_handle h, int on);
int nb_drive_state(nb_handle h, nb_drive_info* out);    /* synchronizes */
/* k stirring-phase steps (sim.py:1044-1050 _pre_step without its end-of-phase test): dt from
 * the CFL max speed (no dt_cap), hydro without stars, wind or jets, the drive with amplitude
 * pre_amp, tp += dt, ip += 1.  NB_ERR_STATE in the main phase or before two fields were pushed.
 * Asynchronous. */
int nb_pre_step(nb_handle h, int k);
/* One nebula3d.py:165-179 drive launch with explicit arguments (fa, fb: device, [3][sx][sy][sz]
 * on the grid of nb_drive_config), for parity. */
int nb_drive_step(nb_handle h, const float* fa, const float* fb, float blend, float amp, float dt);
/* sim.py:352-363 add_torus: rho += torus, m *= 1 - torus / (torus + rho) (torus: device,
 * nx*ny*nz floats); sim.py:806-812 runs it when the stirring phase ends. */
int nb_add_torus(nb_handle h, const float* torus);
/* sim.py:501-508 mach_sums in FP64: out[0] = sum |m|^2 / rho, out[1] = sum rho.  Synchronizes. */
int nb_mach_sums(nb_handle h, double out[2]);

/* ---------------------------------------------------------------- single kernels
 * Parity and benchmarking entry points for one reference kernel launch each. */
/* One RK2 stage: nebula3d.py:76-151 hydro_stage / sim.py:423-498 hydro_stage_hll, launched
 * as in sim.py:1025/1028 (in -> out with out = a*U0 + b*(in + dt L(in))).  in/U0/out are
 * 4-plane (rho, mx, my, mz) pointers; out may alias U0 (stage 2 in place).  dt and pulse
 * are given explicitly; the star/jet weights are those of the handle's current clock. */
int nb_hydro_stage(nb_handle h, const float* const in4[4], const float* const u0_4[4], float* const out4[4],
                   float a, float b, float dt, float pulse);
/* nebula3d.py:154-162 max_speed over the handle's current fields (synchronizes). */
int nb_max_speed(nb_handle h, float* smax_out);
/* nebula3d.py:247-270 cast_rays for one star into rfront_out (device, nu*nphi floats). */
int nb_cast_rays(nb_handle h, const double star_xyz[3], double Q, float* rfront_out);
/* nebula3d.py:320-352 cast_fuv for one star into att_out (device, fnr*fnu*fnphi floats,
 * reference layout [b][iu][ip]). */
int nb_cast_fuv(nb_handle h, const double star_xyz[3], float* att_out);

/* ---------------------------------------------------------------- batches
 * No single reference counterpart: many Sim instances (sim.py:543) advanced together, each
 * with its own clock, CFL dt, stars and ionization cadence (it % ion_every, sim.py:1102).
 * A batch step = one control launch for every instance, the ionization of every instance due
 * to ionize (3 launches), and one persistent launch per RK2 stage walking a tile work-list that
 * spans all instances; the step is replayed as a CUDA graph when every slot is active and every
 * instance or none ionizes.  The instances must share solver, limiter and stream and be in the main phase
 * without stirring (NB_ERR_STATE otherwise: step those alone); the batch works on its own
 * stream, ordered after / before the instances' stream by events.  The instance handles stay
 * valid and usable between batch steps (nb_step, nb_fuv, nb_get_clock ...). */
typedef struct nb_batch_s* nb_batch;
enum { NB_BATCH_GRAPHS = 0, NB_BATCH_GRID = 1, NB_BATCH_RAY_GROUP = 2 };
int nb_batch_create(const nb_handle* instances, const int* ion_every, int n, nb_batch* out);
int nb_batch_step(nb_batch b, int k);
/* Slots of a batch (no reference counterpart; a server keeps a pool of instances in one batch): n
 * flags, one per instance in nb_batch_create's order; an idle slot (0) is not stepped -- no weights,
 * clock, rays or tiles -- and is left as it is, so instances can join and leave the stepping set
 * without rebuilding the batch or its graphs.  The work list is compacted to the active slots'
 * tiles; while a slot is idle, steps are launched as they go (on the active and due instances'
 * work only) rather than replayed.  All slots start active.  Synchronizes the batch's stream. */
int nb_batch_set_active(nb_batch b, const int* active, int n);
int nb_batch_set_option(nb_batch b, int key, int value);
int nb_batch_counters(nb_batch b, long long* launches);
void nb_batch_destroy(nb_batch b);
const char* nb_batch_last_error(nb_batch b);

/* ---------------------------------------------------------------- snapshots and frames */
/* timeline.py:19-89 k_pack / k_pack_lm: the 13 B/cell snapshot of the handle's fields into a
 * device buffer of 13*N bytes, planes [rho fp16 | mx fp16 | my fp16 | mz fp16 | xi uint8 |
 * dfront fp16 | g0 fp16] (values clamped to +-65000, xi = int(clamp(xi,0,1)*255 + 0.5)). */
int nb_snapshot_pack(nb_handle h, void* out13);
/* timeline.py k_unpack / k_unpack_lm: back into the fields (rho floored); the next step
 * recomputes the CFL max speed. */
int nb_snapshot_unpack(nb_handle h, const void* in13);
/* bake.py:95-102: one frame's fields into a device buffer of 9*N bytes, planes [g0 fp16 (min
 * 6e4) | rho fp16 | xi uint8 (round half even of clip(xi,0,1)*255) | dfront fp16 (clip +-4) |
 * shock fp16 (min 6e4)], with the shock proxy of nebula3d.py:182-191 computed inline. */
int nb_frame_pack(nb_handle h, void* out9);
/* nebula3d.py:182-191 shock_field into a device buffer of N floats (Sim.shock, sim.py:827-833). */
int nb_shock(nb_handle h, float* out);

/* ---------------------------------------------------------------- renderer pack
 * render.py:77-88 PackParams: palette colours times the line weights (c_dg multiplies
 * dust * g0eff), the FUV saturation Gs and ambient term, the box-edge fade width, 1 / L and dx. */
typedef struct nb_pack_params {
    float c_ha[3], c_o3[3], c_s2[3], c_dg[3], c_sh[3];
    float gs, ambient, edge;
    float inv_L[3];
    float dx;
} nb_pack_params;
/* render.py:176-205 pack_volume_lm: the RGBA16F voxel grid (emission r, g, b; dust) of the
 * handle's fields, the shock proxy computed inline when shock_on != 0, into `out8` (device,
 * 8 B/cell, C order [i][j][k][4] float16).  With smooth != 0 also render.py:281-298 smooth_axis
 * along x, y, z, with `tmp8` (device, 8 B/cell) as the second grid; the result is in out8
 * either way.  Renderer.pack packs into Sim.render_scratch (sim.py:821-825): the stage block. */
int nb_render_pack(nb_handle h, const nb_pack_params* pp, int shock_on, int smooth, void* out8, void* tmp8);

/* ---------------------------------------------------------------- diagnostics */
/* Kernel kinds timed by nb_profile (CUDA events on the handle's stream around each launch). */
enum {
    NB_PROF_CTRL = 0,         /* star weights / dt / pulse (sim.py:914-925, 1009-1012, 1108) */
    NB_PROF_STAGE1 = 1,       /* hydro RK2 stage 1 */
    NB_PROF_STAGE2 = 2,       /* hydro RK2 stage 2 (+ CFL max speed) */
    NB_PROF_CAST_RAYS = 3,    /* nebula3d.py:247-270 */
    NB_PROF_APPLY_FRONT = 4,  /* nebula3d.py:281-307, all stars */
    NB_PROF_SMOOTH = 5,       /* nebula3d.py:310-315 (+ CFL max speed) */
    NB_PROF_CAST_FUV = 6,     /* nebula3d.py:320-352 */
    NB_PROF_APPLY_FUV = 7,    /* nebula3d.py:355-388, all stars */
    NB_PROF_MAX_SPEED = 8,    /* nebula3d.py:154-162 stand-alone */
    NB_PROF_SNAPSHOT = 9,     /* snapshot / frame packing, shock proxy */
    NB_PROF_DRIVE = 10,       /* nebula3d.py:165-179 stirring (+ CFL max speed), add_torus */
    NB_PROF_RENDER = 11,      /* render.py:176-205, 281-298 voxel pack + prefilter */
    NB_PROF_KINDS = 16
};
/* No reference counterpart (the reference times whole calls with perf_counter, sim.py:578-579):
 * enable / disable per-kernel CUDA-event timing; nb_profile_read synchronizes, returns the
 * summed milliseconds and launch counts per kind since the last read, and resets them. */
int nb_profile(nb_handle h, int enable);
int nb_profile_read(nb_handle h, double ms[NB_PROF_KINDS], long long count[NB_PROF_KINDS]);
/* Launch-shape knobs picked by the package's autotuner (no reference counterpart): the tile depth
 * along i of the hydro march (i-chunk), the tile sweep order (0: k, j, i-chunk; 1: i-chunk, k, j),
 * and the lanes per ray (1, 2, 4, 8, 16, 32 ionizing, default 1; 8, 16, 32 FUV, default 16) of the
 * ray kernels (the defaults: i-chunk 20, order 0).  The hydro
 * result does not depend on them; the ray sums only through their rounding.  NB_TUNE_FRONT_CULL
 * (default 1; up to 32 stars): the front pass first bounds each star's front radius and then
 * leaves out, per 32-cell segment of a row, the stars that cannot change its ionized fraction or
 * front distance; NB_TUNE_FUV_CUT (default 1): a FUV ray stops once its optical depth passes 120,
 * where exp(-tau) is 0.0f for good, and writes 0 to its remaining bins.  The result is the same
 * either way, bit for bit.
 * Failure-path test keys (no reference counterpart; the reference blocks on a host read instead,
 * sim.py:1009-1012): NB_TUNE_WAIT_LIMIT (default and maximum 2^22) is the number of polls after
 * which a hydro stage's bounded TMA wait gives up; NB_TUNE_STALL_TEST = 1 makes the hydro stages
 * issue no tile copy at all, so the first wait of every tile runs out with nothing in flight: the
 * stage records NB_DEV_TMA_TIMEOUT, writes nothing and returns, and every later clock read returns
 * NB_ERR_TIMEOUT.  The handle's fields are then incomplete for good (destroy it).  A batch takes
 * both from its instances when it is created.
 * NB_TUNE_FRONT_PAIRS (default 0) and NB_TUNE_FUV_PAIRS (default 1): the ray-front table (fronts,
 * nebula3d.py:273-307) or the FUV attenuation table (nebula3d.py:355-388) holds each entry with its
 * next neighbour along u (fronts) or r (attenuation) as one float2 pair, so the bilinear or
 * trilinear lookup makes half as many gathers, for twice the table bytes and a second write per
 * entry in the ray kernel; 0 keeps one float per entry.  The result is the same either way, bit for
 * bit.  A batch takes the front layout from its instances when it is created. */
enum { NB_TUNE_CHUNK_I = 0, NB_TUNE_RAY_GROUP = 1, NB_TUNE_FUV_GROUP = 2, NB_TUNE_TILE_ORDER = 3,
       NB_TUNE_FRONT_CULL = 4, NB_TUNE_FUV_CUT = 5, NB_TUNE_WAIT_LIMIT = 6, NB_TUNE_STALL_TEST = 7,
       NB_TUNE_FRONT_PAIRS = 8, NB_TUNE_FUV_PAIRS = 9 };
int nb_set_tuning(nb_handle h, int key, int value);
int nb_get_tuning(nb_handle h, int key, int* value);
/* Number of kernels the handle has launched (a claim the benchmark reports). */
int nb_counters(nb_handle h, long long* launches);

/* ---------------------------------------------------------------- allocation-free entry point
 * No counterpart in the reference.  The FP64 totals of nb_reduce_fp64 (sum rho, mx, my, mz
 * over n cells) for callers that cannot allocate device memory -- e.g. a serving process whose
 * device memory all belongs to a pre-sized pool, or code that must not call cudaMalloc while
 * another thread captures work into a CUDA graph.  It needs no handle: the caller passes the
 * four input planes (device) and out4 (device, 4 doubles); the per-block partial sums live in
 * a library-owned static device array of 512 KiB (held by every GPU that loads the library
 * until the process exits), which caps n at 2^30 cells: larger n returns NB_ERR_LIMIT with a
 * message in nb_static_last_error().  It calls no cudaMalloc / cudaFree.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress, with the device current);
 * make that first call before any stream capture.  The address belongs to the context it was
 * looked up in: a call made in another context (after a cudaDeviceReset, or with another context
 * current on the thread) looks it up again, so the first call after such a change is a set-up
 * call too.  An error that an earlier CUDA call left pending on the thread is returned as
 * NB_ERR_CUDA before any work is enqueued, and left pending.  Every call shares the one array:
 * calls that overlap on the GPU (different streams without ordering) race.  Asynchronous on
 * `stream` (0 = legacy default stream). */
int nb_reduce_fp64_static(const float* rho, const float* mx, const float* my, const float* mz, long long n,
                          double* out4, void* stream);
const char* nb_static_last_error(void);
/* FP64 conservation totals: sum rho, sum mx, sum my, sum mz (times dx^3 = mass/momentum). */
int nb_reduce_fp64(nb_handle h, double out[4]);

#ifdef __cplusplus
}
#endif
#endif /* NEBULA_GB300_H */
