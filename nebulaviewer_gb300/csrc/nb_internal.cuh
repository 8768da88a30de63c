// Internal declarations shared by the libnebula translation units.
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nebula.h"

#define NB_FRONT_PARTS 32         // partial front-radius ranges per star (apply_front culling)
#define NB_ROW_STARS 32           // stars a per-row table holds (more: per-cell form)
#define NB_MAX_STARS 256          // star-table capacity limit (smem-resident in the kernels)
#define NB_WAIT_LIMIT (1u << 22)  // iteration cap of every device-side spin wait

// Device-status bits (NbState::status), reported by nb_device_status.
#define NB_DEV_TMA_TIMEOUT 1u
#define NB_ADV_MAIN 1             // control-kernel modes (weights only = 0)
#define NB_ADV_PRE 2
#define NB_DEV_DRIVE_EMPTY 2u    // a stirred step found no pushed field B (the step did not stir)

// ------------------------------------------------------------------ device-resident data
// Scalars written by the host (geometry, physics, live parameters).  float copies are the
// float32 kernel arguments the reference passes to Warp (Python double -> float32).
struct NbConst {
    int nx, ny, nz, nstars;
    int dx_pow2;                 // dx == 2^-m: x / dx == x * (1/dx) exactly
    int solver, limiter, fields_fp32;
    float dx, inv_dx, floor_, cn2, ci2, vmax;
    float width;                 // 1.2 * dx (sim.py:939)
    float bmax[3];               // box extent (sim.py:750)
    float diag_f, dr_f, binr_f;  // rcap, ray step, FUV bin width (sim.py:742-744, 958)
    int nu, nphi, nsteps, fnr, fnu, fnphi;
    double dx_d, cfl, diag_d;
    // live parameters (sim.py:82-83)
    double q_main, wind, jet, jet_proto, jet_pulse, jet_period, kappa_fuv, q_ramp, jet_r, jet_cos, dt_cap;
    int phase_main;
    float wind_f, jet_cos_f, jet_r_f, kappa_f;
    // plane-parallel ionizing / FUV source on the -x face (no reference counterpart)
    int plane_on;
    float plane_F_f, plane_lum_f;
    double plane_F, plane_lum;
    const float* plane_xf;      // [ny][nz] front position along +x per column
    const float* plane_g0;      // [nx][ny][nz] plane FUV term (stage plane 2, written by the FUV pass)
    // turbulent stirring (nebula3d.py:165-179, sim.py:1030-1059)
    int drive_on;                // main-phase stirring allowed (the reference's drv is not None)
    int drive_sx, drive_sy, drive_sz, drive_slots;
    long long drive_pushed;      // forcing fields pushed into the ring so far
    float drive_dxs_f;
    double drive_pre_corr, pre_amp, drive_main;
    const float* drive_ring;     // [slots][3][sx][sy][sz]
};

// Written by device kernels every step.
struct NbState {
    double t, dt;
    long long it;
    float dt_f, pulse_f;         // float32 arguments of the step's hydro stages
    unsigned smax_bits;          // CFL max speed (non-negative float bits; atomicMax on uint)
    unsigned status;             // NB_DEV_* failure bits
    double tp;                   // stirring-phase time and steps (sim.py Sim.tp / Sim.ip)
    long long ip;
    double dclock;               // stirring cross-fade clock (sim.py drv['clock'])
    long long dswaps;            // forcing fields retired: A = field dswaps, B = field dswaps + 1
    float blend_f, amp_f;        // this step's drive arguments (sim.py:1032, 1047 / 1111)
    int drive_a, drive_b;        // ring slots of A and B for this step
    int drive_go;                // this step stirs
    int pad_;
};

struct NbStarDev {
    double x, y, z, qf, t_on, ax, ay, az;
    int kind, jkind;
};

// Weights of one star for the hydro sources and the ray kernels (computed on device at t).
struct NbStarW {
    float4 w;      // (x, y, z, q_eff / q_main or 0 before t_on)   sim.py:916
    float4 jet;    // (ax, ay, az, strength)                       sim.py:923
    float q_f;     // q_eff as float32 (cast_rays Q, sim.py:937)
    float lum_f;   // q_eff / q_main as float32 (apply_fuv lum, sim.py:965)
    int active;    // t >= t_on (sim.py:934)
    int pad;
};

// Tensor maps of an instance's planes (device global memory, 64-byte aligned).
enum { NB_MAP_RHO = 0, NB_MAP_MX, NB_MAP_MY, NB_MAP_MZ, NB_MAP_XI, NB_MAP_S0, NB_MAP_S1, NB_MAP_S2, NB_MAP_S3,
       NB_NMAPS };

// ------------------------------------------------------------------ kernel argument packs
struct HydroLaunch {
    const NbConst* c;
    const NbState* st;
    const NbStarW* sw;
    const CUtensorMap* maps;     // device array of NB_NMAPS maps; null: the failure-path test
                                 // (NB_TUNE_STALL_TEST) -- no tile copy is issued, so the first wait
                                 // of every tile runs out with nothing in flight
    int map_in;                  // NB_MAP_RHO (stage 1) or NB_MAP_S0 (stage 2)
    const float* in[4];
    const float* u0[4];
    float* out[4];
    const float* xi;
    float a, b;
    float dt_override, pulse_override;   // used when use_override (single-stage entry point)
    int use_override;
    unsigned* smax_bits;         // non-null: accumulate the CFL max speed of `out`
    unsigned* status;
    int tiles_k, tiles_j, chunk_i, n_chunks;
    int nstars_host;             // == c->nstars (sizes the dynamic shared memory)
    int no_sources;              // stirring-phase hydro: no stars, wind or jets (sim.py:1046)
    int order;                   // tile sweep order (NB_TUNE_TILE_ORDER)
    int idx32;                   // fewer than 2^31 cells: 32-bit cell offsets (single-instance stage)
    unsigned wait_limit;         // polls of each bounded TMA wait (NB_TUNE_WAIT_LIMIT)
    int active;                  // batched stage: 0 = the instance's slot is idle (its tiles are skipped)
};

// One instance of a batch, as the batched control kernel sees it.
struct NbBatchInst {
    const NbConst* c;
    NbState* st;
    const NbStarDev* stars;
    NbStarW* sw;
    int nstars;
    int active;           // 0: an idle slot of the batch (no weights, no clock advance)
};

// One instance of a batched ionization (nebula3d.py:247-315 over many instances in 3 launches).
struct NbRayJob {
    const NbConst* c;
    const NbStarW* sw;
    const float4* dirs;
    const float* rho;
    const float* mx;
    const float* my;
    const float* mz;
    float* rfront;
    float* xi_raw;
    float* xi;
    void* dfront;
    unsigned* smax;
    long long ray0;       // first ray group of this job (prefix over listed instances)
    long long blk0;       // first row block of this job (8 rows per block)
    int nstars;
    int half;
    float2* front_parts;  // the instance's front-radius partials when apply_front culls, else null
    long long nray;       // rays per star (nu * nphi)
    int pairs;            // the front table holds (u, u + 1) pairs (NB_TUNE_FRONT_PAIRS)
    int active;           // 0: an idle slot of the batch (its rays, fronts and smoothing are skipped)
};

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ float fmaxr(float a, float b) { return a > b ? a : b; }   // Warp max
__device__ __forceinline__ float fminr(float a, float b) { return a < b ? a : b; }   // Warp min
// fmaxr / fminr in the exact build; one min / max instruction in the fast build (fmaxr is a compare
// and a select): the same value for every operand pair without a NaN, but for the sign of a zero
#if defined(NB_ARITH_FAST) && NB_ARITH_FAST
__device__ __forceinline__ float fmaxq(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float fminq(float a, float b) { return fminf(a, b); }
#else
__device__ __forceinline__ float fmaxq(float a, float b) { return fmaxr(a, b); }
__device__ __forceinline__ float fminq(float a, float b) { return fminr(a, b); }
#endif
__device__ __forceinline__ int iclampd(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }
// The calling warp's slot on its SM (%warpid).  Slot w is issued by scheduler w mod 4; the slot
// may change on preemption, so it only ever steers work placement, never correctness.
__device__ __forceinline__ unsigned warp_slot() {
    unsigned w;
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(w));
    return w;
}

// ---- mbarrier / TMA (sm_90+ PTX; every wait is bounded)
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Returns false when the wait gave up after NB_WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    for (unsigned n = 0; n < NB_WAIT_LIMIT; ++n)
        if (mbar_test(bar, parity)) return true;
    return false;
}
// The same wait with a lower limit read from memory (a handle's NB_TUNE_WAIT_LIMIT): the limit is
// read only on the slow path, after each 64 polls that found the phase still open, so a wait that
// completes at once keeps no register for it.
__device__ __forceinline__ bool mbar_wait_limited(uint64_t* bar, unsigned parity, const unsigned* limit) {
    for (unsigned n = 0; n < NB_WAIT_LIMIT; ++n) {
        if (mbar_test(bar, parity)) return true;
        if ((n & 63u) == 63u && n + 1u >= *limit) return false;
    }
    return false;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// 3D tiled TMA load (non-multicast, this GPU's own memory).  c0 is the innermost (k)
// coordinate and must be a multiple of 4 floats (16 bytes).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// ------------------------------------------------------------------ launchers (nb_*.cu)
cudaError_t nb_launch_hydro(const HydroLaunch& L, int solver, int limiter, cudaStream_t s);
int nb_hydro_tile_j();
// Batches of up to NB_BATCH_PARAM_MAX instances (32-bit cell offsets) hand the persistent stage
// kernel their stage records as one kernel parameter (28 KB of the 32 KB parameter space): the
// kernel then reads a record's fields from the constant bank, as the single-instance kernel reads
// its own, and fits 64 registers (4 blocks / SM) where records read from global memory need 80.
#define NB_BATCH_PARAM_MAX 128
struct NbBatchRecords {
    HydroLaunch L[NB_BATCH_PARAM_MAX];
};
// idx32: every listed instance has fewer than 2^31 cells (32-bit cell offsets); params: the
// records go in the kernel parameter (idx32 and at most NB_BATCH_PARAM_MAX instances)
int nb_hydro_batch_blocks_per_sm(int solver, int limiter, int max_stars, int idx32, int params);
// Ls: the device copy of the records (the active flags and status words are read there); rec: the
// same records on the host, passed as the kernel parameter, or null
cudaError_t nb_launch_hydro_batch(const HydroLaunch* Ls, const NbBatchRecords* rec, const int2* work, int n_work,
                                  unsigned* counter, int max_stars, int stage2, int idx32, int solver, int limiter,
                                  int grid, cudaStream_t s);
cudaError_t nb_launch_ctrl(const NbConst* c, NbState* st, const NbStarDev* stars, NbStarW* sw, int nstars,
                           int advance, cudaStream_t s);
cudaError_t nb_launch_ctrl_batch(const NbBatchInst* insts, int n, int advance, unsigned* counters, cudaStream_t s);
cudaError_t nb_launch_weights(const NbConst* c, const NbState* st, const NbStarDev* stars, NbStarW* sw,
                              int nstars, cudaStream_t s);
cudaError_t nb_launch_max_speed(const NbConst* c, const float* rho, const float* mx, const float* my,
                                const float* mz, const float* xi, unsigned* smax_bits, long n, cudaStream_t s);
cudaError_t nb_launch_drive(const NbConst* c, const NbState* st, const float* rho, float* mx, float* my, float* mz,
                            const float* xi, unsigned* smax_bits, int nx, int ny, int sz, cudaStream_t s);
cudaError_t nb_launch_drive_explicit(const NbConst* c, const float* rho, float* mx, float* my, float* mz,
                                     const float* fa, const float* fb, float blend, float amp, float dt, int nx,
                                     int ny, int sz, cudaStream_t s);
cudaError_t nb_launch_add_torus(const float* torus, float* rho, float* mx, float* my, float* mz, long long n,
                                cudaStream_t s);
int nb_mach_scratch_doubles();
cudaError_t nb_launch_mach_sums(const float* rho, const float* mx, const float* my, const float* mz, long long n,
                                double* scratch, cudaStream_t s);
cudaError_t nb_launch_render_pack(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                                  const float* xi, const void* dfront, const void* g0, int half,
                                  const nb_pack_params& pp, int shock_on, int smooth, void* out8, void* tmp8, int nx,
                                  int ny, cudaStream_t s);
cudaError_t nb_launch_ray_dirs(int nu, int nphi, float4* dirs, cudaStream_t s);
// pairs: the instance's front table holds (rf(u), rf(u + 1)) float2 pairs (2 * nu * nphi floats per
// star); a star_override launch writes the reference layout [u][phi] (pairs = 0)
cudaError_t nb_launch_cast_rays(const NbConst* c, const NbStarW* sw, const float4* dirs, const float* rho,
                                float* rfront, int nstars, int group, const float* star_override, float q_override,
                                cudaStream_t s, int nu, int nphi, int pairs);
// with front_parts (NB_ROW_STARS * NB_FRONT_PARTS float2 scratch) and 1 <= nstars <= NB_ROW_STARS:
// first each star's front-radius range (one more launch), then segments skip the stars that
// cannot change them
cudaError_t nb_launch_apply_front(const NbConst* c, const NbStarW* sw, const float* rfront, int nstars,
                                  float* xi_raw, void* dfront, unsigned* smax_reset, cudaStream_t s, int nx, int ny,
                                  int half, float2* front_parts, long long nray, int pairs);
cudaError_t nb_launch_smooth(const NbConst* c, const float* xi_raw, float* xi, const float* rho, const float* mx,
                             const float* my, const float* mz, unsigned* smax_bits, cudaStream_t s, int nx, int ny);
// The ray cast of a batch of at most NB_BATCH_PARAM_MAX jobs takes the job records as one kernel
// parameter (host_jobs, the host copy of `jobs`), as the batched hydro stage does; the active
// flags are read from the device copy.  host_jobs null: the records are read from `jobs`.
struct NbRayJobs {
    NbRayJob J[NB_BATCH_PARAM_MAX];
};
cudaError_t nb_launch_ionize_batch(const NbRayJob* jobs, const NbRayJob* host_jobs, int n_jobs, long long n_groups,
                                   long long n_blocks, int group, cudaStream_t s);
cudaError_t nb_launch_plane_front(const NbConst* c, const float* rho, float* xf, int ny, int nz, cudaStream_t s);
cudaError_t nb_launch_plane_fuv(const NbConst* c, const float* rho, const float* xi, float* g, int ny, int nz,
                                cudaStream_t s);
// packs (rho, xi) pairs into rx_scratch (ncell float2, 8-byte aligned) first
cudaError_t nb_launch_cast_fuv(const NbConst* c, const NbStarW* sw, const float4* dirs, const float* rho,
                               const float* xi, float* att, int nstars, int group, const float* star_override,
                               int ref_layout, cudaStream_t s, int fnu, int fnphi, void* rx_scratch, long long ncell,
                               float tau_cut, int pairs);
#define NB_FUV_TAU_CUT 120.0f            // optical depth past which a FUV ray's remaining bins are 0
cudaError_t nb_launch_apply_fuv(const NbConst* c, const NbStarW* sw, const float* att, int nstars, void* g0,
                                cudaStream_t s, int nx, int ny, int half, int pairs);
cudaError_t nb_launch_pack(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                           const float* xi, const void* df, const void* g0, int half, void* out, long long n,
                           cudaStream_t s);
cudaError_t nb_launch_unpack(const NbConst* c, const void* in, long long n, float* rho, float* mx, float* my,
                             float* mz, float* xi, void* df, void* g0, int half, cudaStream_t s);
cudaError_t nb_launch_shock(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                            float* out, int nx, int ny, cudaStream_t s);
cudaError_t nb_launch_frame(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                            const float* xi, const void* df, const void* g0, int half, void* out, long long n, int nx,
                            int ny, cudaStream_t s);
cudaError_t nb_launch_reduce_fp64(const float* rho, const float* mx, const float* my, const float* mz, long n,
                                  double* scratch, cudaStream_t s);   // totals at scratch[4*608 .. +4)
int nb_reduce_scratch_doubles();
