// The C ABI of include/nebula.h: instance set-up, the step sequencing of sim.py (_main_step,
// ionize, fuv_field) over the device kernels, and single-kernel entry points for parity.
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <memory>
#include <vector>

#include "nb_internal.cuh"

#define NB_EXPORT extern "C" __attribute__((visibility("default")))

struct nb_instance {
    nb_desc d{};
    cudaStream_t stream = nullptr;
    NbConst hc{};                       // host copy of the device constants
    NbConst* c = nullptr;
    NbState* st = nullptr;
    NbStarDev* stars = nullptr;
    NbStarW* sw = nullptr;
    CUtensorMap* maps = nullptr;        // NB_NMAPS maps of the instance's planes
    CUtensorMap* tmp_maps = nullptr;    // maps for nb_hydro_stage on foreign planes
    float4* dirs = nullptr;             // ionizing-ray directions (nu * nphi)
    float4* dirs_fuv = nullptr;         // FUV-ray directions (fnu * fnphi)
    float* rfront = nullptr;            // [star][nphi][nu] (float2 (u, u + 1) pairs with front_pairs)
    float* att = nullptr;               // [star][fnu][fnphi][fnr] (float2 (r, r + 1) pairs with fuv_pairs)
    float* scratch3 = nullptr;          // 3 floats: a single star position for the one-star kernels
    float* plane_xf = nullptr;          // [ny][nz] front of the -x plane source
    double* red = nullptr;              // FP64 reduction partials
    float2* front_parts = nullptr;      // per-star front-radius ranges (apply_front)
    float* drive_ring = nullptr;        // stirring fields [slots][3][sx][sy][sz]
    NbState* state_mirror = nullptr;    // pinned host copy of the control block (nb_mirror_clock, nb_set_clock)
    long long drive_field = 0;          // floats per forcing field (3 components)
    int nstars = 0, star_alloc = 0;
    long long host_it = 0;
    int smax_valid = 0;
    int chunk_i = 20, ray_group = 1, fuv_group = 16;      // measured best at 192^3-256^3 (nb_set_tuning)
    int tile_order = 0;
    int front_cull = 1;                 // apply_front skips the stars that cannot change a segment
    int fuv_cut = 1;                    // FUV rays stop where exp(-tau) has reached 0.0f
    unsigned wait_limit = NB_WAIT_LIMIT; // polls of each bounded TMA wait in the hydro stages
    int stall_test = 0;                 // failure-path test: the hydro stages issue no tile copies
    int front_pairs = 0;                // ray-front table as float2 (u, u + 1) pairs (measured: no gain at 256^3)
    int fuv_pairs = 1;                  // FUV attenuation table as float2 (r, r + 1) pairs
    long long ncell = 0;
    long long launches = 0;             // kernels this handle launched (nb_counters)
    int profiling = 0;                  // CUDA-event timing per kernel kind (nb_profile)
    struct ProfRec { int kind; cudaEvent_t a, b; };
    std::vector<ProfRec> recs;
    std::vector<cudaEvent_t> pool;
    std::string err;
};

static thread_local std::string g_err;

namespace {

int fail(nb_instance* h, int code, const std::string& msg) {
    if (h) h->err = msg; else g_err = msg;
    return code;
}
int cuda_fail(nb_instance* h, cudaError_t e, const char* what) {
    return fail(h, NB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(h, call)                                                          \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call);             \
    } while (0)

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda needed)
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    return fn;
}

// A (nx, ny, nz) float32 plane, k fastest, read as (40 x (TJ+4) x 1) boxes.
bool encode_plane(CUtensorMap* m, const float* ptr, int nx, int ny, int nz) {
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    const int tj = nb_hydro_tile_j();
    cuuint64_t dims[3] = {(cuuint64_t)nz, (cuuint64_t)ny, (cuuint64_t)nx};
    cuuint64_t strides[2] = {(cuuint64_t)nz * 4, (cuuint64_t)ny * nz * 4};
    cuuint32_t box[3] = {40, (cuuint32_t)(tj + 4), 1};
    cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(ptr), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaEvent_t ev_get(nb_instance* h) {
    if (!h->pool.empty()) {
        cudaEvent_t e = h->pool.back();
        h->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets the launches of one kernel kind with CUDA events on the handle's stream.
struct Prof {
    nb_instance* h;
    int kind;
    cudaEvent_t a = nullptr;
    Prof(nb_instance* h_, int kind_, int nlaunch) : h(h_), kind(kind_) {
        h->launches += nlaunch;
        if (h->profiling) {
            a = ev_get(h);
            cudaEventRecord(a, h->stream);
        }
    }
    ~Prof() {
        if (a) {
            cudaEvent_t b = ev_get(h);
            cudaEventRecord(b, h->stream);
            h->recs.push_back({kind, a, b});
        }
    }
};

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

bool is_pow2(double x) {
    int e;
    return x > 0.0 && std::frexp(x, &e) == 0.5;
}

int upload_const(nb_instance* h) {
    CK(h, cudaMemcpyAsync(h->c, &h->hc, sizeof(NbConst), cudaMemcpyHostToDevice, h->stream));
    return NB_OK;
}

float* plane(nb_instance* h, int p) { return h->d.f.stage + (long long)p * h->ncell; }

int launch_stage(nb_instance* h, const float* const in[4], const float* const u0[4], float* const out[4], int map_in,
                 const CUtensorMap* maps, float a, float b, bool override_, float dt, float pulse, bool smax,
                 bool stage2 = false, bool no_sources = false) {
    HydroLaunch L{};
    L.c = h->c;
    L.st = h->st;
    L.sw = h->sw;
    L.maps = maps;
    L.map_in = map_in;
    for (int f = 0; f < 4; ++f) {
        L.in[f] = in[f];
        L.u0[f] = u0[f];
        L.out[f] = out[f];
    }
    L.xi = h->d.f.xi;
    L.a = a;
    L.b = b;
    L.use_override = override_ ? 1 : 0;
    L.dt_override = dt;
    L.pulse_override = pulse;
    L.smax_bits = smax ? &h->st->smax_bits : nullptr;
    L.status = &h->st->status;
    const int tj = nb_hydro_tile_j();
    L.tiles_k = (h->d.nz + 31) / 32;
    L.tiles_j = (h->d.ny + tj - 1) / tj;
    L.chunk_i = h->chunk_i < h->d.nx ? h->chunk_i : h->d.nx;
    L.n_chunks = (h->d.nx + L.chunk_i - 1) / L.chunk_i;
    L.nstars_host = h->nstars;
    L.order = h->tile_order;
    L.no_sources = no_sources ? 1 : 0;
    L.idx32 = h->ncell < (1LL << 31) ? 1 : 0;
    L.wait_limit = h->wait_limit;
    if (h->stall_test) L.maps = nullptr;
    Prof pf(h, (smax || stage2) ? NB_PROF_STAGE2 : NB_PROF_STAGE1, 1);
    CK(h, nb_launch_hydro(L, h->d.solver, h->d.limiter, h->stream));
    return NB_OK;
}

int do_ionize(nb_instance* h) {
    const nb_fields& f = h->d.f;
    {
        Prof pf(h, NB_PROF_CTRL, 1);
        CK(h, nb_launch_weights(h->c, h->st, h->stars, h->sw, h->nstars, h->stream));
    }
    if (h->nstars > 0) {
        Prof pf(h, NB_PROF_CAST_RAYS, 1);
        CK(h, nb_launch_cast_rays(h->c, h->sw, h->dirs, f.rho, h->rfront, h->nstars, h->ray_group, nullptr, 0.0f,
                                  h->stream, h->d.nu, h->d.nphi, h->front_pairs));
    }
    if (h->hc.plane_on) {
        Prof pf(h, NB_PROF_CAST_RAYS, 1);
        CK(h, nb_launch_plane_front(h->c, f.rho, h->plane_xf, h->d.ny, h->d.nz, h->stream));
    }
    float* xi_raw = plane(h, 0);            // sim.py:928-941: xi_tmp lives in the stage block
    {
        const bool cull = h->front_cull && h->nstars >= 1 && h->nstars <= NB_ROW_STARS;
        Prof pf(h, NB_PROF_APPLY_FRONT, cull ? 2 : 1);
        CK(h, nb_launch_apply_front(h->c, h->sw, h->rfront, h->nstars, xi_raw, f.dfront, &h->st->smax_bits,
                                    h->stream, h->d.nx, h->d.ny, h->d.fields_fp32 ? 0 : 1,
                                    cull ? h->front_parts : nullptr,
                                    (long long)h->d.nu * h->d.nphi, h->front_pairs));
    }
    {
        Prof pf(h, NB_PROF_SMOOTH, 1);
        CK(h, nb_launch_smooth(h->c, xi_raw, f.xi, f.rho, f.mx, f.my, f.mz, &h->st->smax_bits, h->stream, h->d.nx, h->d.ny));
    }
    h->smax_valid = 1;
    return NB_OK;
}

bool stirring_main(const nb_instance* h) { return h->hc.drive_on && h->hc.drive_main > 0.0; }

// the control block into pinned host memory, in stream order (read by nb_peek_clock)
int mirror_state(nb_instance* h) {
    CK(h, cudaMemcpyAsync(h->state_mirror, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    return NB_OK;
}

// The two RK2 stages of sim.py:1014-1028 and, when the step stirs, the drive of sim.py:1030-1042;
// the step's last kernel leaves the next step's CFL max speed in st->smax_bits.
int hydro_and_stir(nb_instance* h, bool stir, bool no_sources) {
    const nb_fields& f = h->d.f;
    int rc;
    const float* U[4] = {f.rho, f.mx, f.my, f.mz};
    float* Uw[4] = {f.rho, f.mx, f.my, f.mz};
    float* S[4] = {plane(h, 0), plane(h, 1), plane(h, 2), plane(h, 3)};
    const float* Sc[4] = {S[0], S[1], S[2], S[3]};
    // sim.py:1025: U -> U1 (a = 0, b = 1);  sim.py:1028: U1 -> U in place (a = b = 1/2) + max speed
    if ((rc = launch_stage(h, U, U, S, NB_MAP_RHO, h->maps, 0.0f, 1.0f, false, 0.f, 0.f, false, false, no_sources)) !=
        NB_OK)
        return rc;
    if ((rc = launch_stage(h, Sc, U, Uw, NB_MAP_S0, h->maps, 0.5f, 0.5f, false, 0.f, 0.f, !stir, true, no_sources)) !=
        NB_OK)
        return rc;
    if (stir) {
        Prof pf(h, NB_PROF_DRIVE, 2);
        CK(h, nb_launch_drive(h->c, h->st, f.rho, f.mx, f.my, f.mz, f.xi, &h->st->smax_bits, h->d.nx, h->d.ny,
                              h->hc.drive_sz, h->stream));
    }
    h->smax_valid = 1;
    return NB_OK;
}

int ensure_smax(nb_instance* h) {
    if (h->smax_valid) return NB_OK;
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_MAX_SPEED, 2);
    CK(h, nb_launch_max_speed(h->c, f.rho, f.mx, f.my, f.mz, f.xi, &h->st->smax_bits, h->ncell, h->stream));
    h->smax_valid = 1;
    return NB_OK;
}

int do_step(nb_instance* h, int ion_every) {
    int rc;
    if (ion_every > 0 && h->host_it % ion_every == 0) {           // sim.py:1102-1103
        if ((rc = do_ionize(h)) != NB_OK) return rc;
    } else if ((rc = ensure_smax(h)) != NB_OK) {
        return rc;
    }
    // sim.py:1104-1108: star weights at t, dt from the max speed (dt_cap), pulse; t += dt
    {
        Prof pf(h, NB_PROF_CTRL, 1);
        CK(h, nb_launch_ctrl(h->c, h->st, h->stars, h->sw, h->nstars, NB_ADV_MAIN, h->stream));
    }
    if ((rc = hydro_and_stir(h, stirring_main(h), false)) != NB_OK) return rc;
    h->host_it += 1;
    return NB_OK;
}

// sim.py:1044-1050 _pre_step (the end-of-phase test is the caller's)
int do_pre_step(nb_instance* h) {
    int rc;
    if ((rc = ensure_smax(h)) != NB_OK) return rc;
    {
        Prof pf(h, NB_PROF_CTRL, 1);
        CK(h, nb_launch_ctrl(h->c, h->st, h->stars, h->sw, h->nstars, NB_ADV_PRE, h->stream));
    }
    return hydro_and_stir(h, true, true);
}

}  // namespace

// ============================================================================ C ABI
NB_EXPORT const char* nb_last_error(nb_handle h) { return h ? h->err.c_str() : g_err.c_str(); }

NB_EXPORT int nb_create(const nb_desc* d, nb_handle* out) {
    if (!d || !out) return fail(nullptr, NB_ERR_ARG, "null argument");
    *out = nullptr;
    if (d->abi_version != NB_ABI_VERSION) return fail(nullptr, NB_ERR_ARG, "abi_version mismatch");
    if (d->nx < 1 || d->ny < 1 || d->nz < 4 || d->nz % 4 != 0)
        return fail(nullptr, NB_ERR_ARG, "grid must be nx, ny >= 1 and nz a positive multiple of 4");
    if (!(d->dx > 0.0) || d->nu < 1 || d->nphi < 1 || d->fnr < 1 || d->fnu < 1 || d->fnphi < 1 || d->nsteps < 1 ||
        !(d->dr > 0.0))
        return fail(nullptr, NB_ERR_ARG, "bad geometry / ray budget");
    if (d->max_stars < 1 || d->max_stars > NB_MAX_STARS)
        return fail(nullptr, NB_ERR_LIMIT, "max_stars must be in [1, 256]");
    if ((long long)d->nu * d->nphi * d->max_stars >= (1LL << 32) ||
        (long long)d->fnu * d->fnphi * d->max_stars >= (1LL << 32))    // ray indices in 32 bits
        return fail(nullptr, NB_ERR_LIMIT, "rays per star times max_stars must stay below 2^32");
    const nb_fields& f = d->f;
    const void* ptrs[] = {f.rho, f.mx, f.my, f.mz, f.xi, f.stage, f.dfront, f.g0};
    for (const void* p : ptrs)
        if (!p || !aligned16(p)) return fail(nullptr, NB_ERR_ARG, "field pointers must be non-null and 16-byte aligned");
    if (d->solver != NB_SOLVER_RUSANOV && d->solver != NB_SOLVER_HLL) return fail(nullptr, NB_ERR_ARG, "bad solver");
    if (d->limiter < 0 || d->limiter > 2) return fail(nullptr, NB_ERR_ARG, "bad limiter");
    if (!encode_fn()) return fail(nullptr, NB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");

    nb_instance* h = new nb_instance();
    h->d = *d;
    h->stream = static_cast<cudaStream_t>(d->stream);
    h->ncell = (long long)d->nx * d->ny * d->nz;
    if (h->ncell * 4 > (1LL << 62) || (long long)d->ny * d->nz >= (1LL << 31) ||
        (long long)d->fnu * d->fnphi * d->fnr >= (1LL << 31)) {
        delete h;
        return fail(nullptr, NB_ERR_LIMIT, "grid too large (ny * nz and fnu * fnphi * fnr must stay below 2^31)");
    }
    NbConst& c = h->hc;
    c.nx = d->nx; c.ny = d->ny; c.nz = d->nz; c.nstars = 0;
    c.dx_pow2 = is_pow2(d->dx) ? 1 : 0;
    c.solver = d->solver; c.limiter = d->limiter; c.fields_fp32 = d->fields_fp32;
    c.dx = (float)d->dx;
    c.inv_dx = (float)(1.0 / d->dx);
    c.floor_ = (float)d->floor_rho;
    c.cn2 = (float)d->cn2;
    c.ci2 = (float)d->ci2;
    c.vmax = (float)d->vmax;
    c.width = (float)(1.2 * d->dx);                               // sim.py:939
    c.bmax[0] = (float)(d->nx * d->dx);                           // sim.py:621, 750
    c.bmax[1] = (float)(d->ny * d->dx);
    c.bmax[2] = (float)(d->nz * d->dx);
    c.diag_f = (float)d->diag;
    c.dr_f = (float)d->dr;
    c.binr_f = (float)(d->diag / d->fnr);                         // sim.py:958
    c.nu = d->nu; c.nphi = d->nphi; c.nsteps = d->nsteps;
    c.fnr = d->fnr; c.fnu = d->fnu; c.fnphi = d->fnphi;
    c.dx_d = d->dx; c.cfl = d->cfl; c.diag_d = d->diag;
    c.q_main = 1.0; c.jet_period = 1.0; c.phase_main = 1;
    c.jet_cos = 1.0; c.jet_cos_f = 1.0f;

    auto bail = [&](int rc) { nb_destroy(h); return rc; };
    cudaError_t e;
#define CKC(call)                                                          \
    do {                                                                   \
        e = (call);                                                        \
        if (e != cudaSuccess) {                                            \
            g_err = std::string(#call) + ": " + cudaGetErrorString(e);     \
            return bail(e == cudaErrorMemoryAllocation ? NB_ERR_NOMEM : NB_ERR_CUDA); \
        }                                                                  \
    } while (0)
    CKC(cudaMalloc(&h->c, sizeof(NbConst)));
    CKC(cudaMalloc(&h->st, sizeof(NbState)));
    CKC(cudaMalloc(&h->stars, sizeof(NbStarDev) * d->max_stars));
    CKC(cudaMalloc(&h->sw, sizeof(NbStarW) * d->max_stars));
    CKC(cudaMalloc(&h->maps, sizeof(CUtensorMap) * NB_NMAPS));
    CKC(cudaMalloc(&h->tmp_maps, sizeof(CUtensorMap) * NB_NMAPS));
    CKC(cudaMalloc(&h->dirs, sizeof(float4) * (size_t)d->nu * d->nphi));
    CKC(cudaMalloc(&h->dirs_fuv, sizeof(float4) * (size_t)d->fnu * d->fnphi));
    CKC(cudaMalloc(&h->scratch3, 4 * sizeof(float)));
    CKC(cudaMalloc(&h->plane_xf, sizeof(float) * (size_t)d->ny * d->nz));
    c.plane_xf = h->plane_xf;
    c.plane_g0 = f.stage + 2 * h->ncell;
    CKC(cudaMalloc(&h->red, sizeof(double) * nb_reduce_scratch_doubles()));
    CKC(cudaMalloc(&h->front_parts, sizeof(float2) * NB_ROW_STARS * NB_FRONT_PARTS));
    CKC(cudaMallocHost(&h->state_mirror, sizeof(NbState)));
    std::memset(h->state_mirror, 0, sizeof(NbState));
    CKC(cudaMemsetAsync(h->st, 0, sizeof(NbState), h->stream));
    CKC(cudaMemsetAsync(h->sw, 0, sizeof(NbStarW) * d->max_stars, h->stream));
    CUtensorMap hm[NB_NMAPS];
    const float* planes[NB_NMAPS] = {f.rho, f.mx, f.my, f.mz, f.xi, f.stage, f.stage + h->ncell,
                                     f.stage + 2 * h->ncell, f.stage + 3 * h->ncell};
    for (int m = 0; m < NB_NMAPS; ++m)
        if (!encode_plane(&hm[m], planes[m], d->nx, d->ny, d->nz)) {
            g_err = "cuTensorMapEncodeTiled failed";
            return bail(NB_ERR_CUDA);
        }
    CKC(cudaMemcpyAsync(h->maps, hm, sizeof(hm), cudaMemcpyHostToDevice, h->stream));
    CKC(nb_launch_ray_dirs(d->nu, d->nphi, h->dirs, h->stream));
    CKC(nb_launch_ray_dirs(d->fnu, d->fnphi, h->dirs_fuv, h->stream));
    CKC(cudaMemcpyAsync(h->c, &h->hc, sizeof(NbConst), cudaMemcpyHostToDevice, h->stream));
    CKC(cudaStreamSynchronize(h->stream));
#undef CKC
    *out = h;
    return NB_OK;
}

// Device bytes an instance of `d` holds with a star table for `star_alloc` stars and a stirring ring
// of `ring_bytes`: the allocations of nb_create, nb_set_stars and nb_drive_config (not the caller's
// fields).  One formula for the estimate and for the live count, so they agree by construction.
static long long instance_bytes(const nb_desc& d, long long star_alloc, long long ring_bytes) {
    const long long ncell_plane = (long long)d.ny * d.nz;
    long long b = 0;
    b += sizeof(NbConst) + sizeof(NbState);
    b += (long long)(sizeof(NbStarDev) + sizeof(NbStarW)) * d.max_stars;
    b += 2LL * sizeof(CUtensorMap) * NB_NMAPS;
    b += (long long)sizeof(float4) * ((long long)d.nu * d.nphi + (long long)d.fnu * d.fnphi);
    b += 4 * sizeof(float) + sizeof(float) * ncell_plane;
    b += (long long)sizeof(double) * nb_reduce_scratch_doubles();
    b += (long long)sizeof(float2) * NB_ROW_STARS * NB_FRONT_PARTS;
    b += 2LL * sizeof(float) * star_alloc * ((long long)d.nu * d.nphi + (long long)d.fnr * d.fnu * d.fnphi);
    return b + ring_bytes;
}

NB_EXPORT int nb_instance_bytes(nb_handle h, const nb_desc* d, int nstars, long long* out) {
    if (!out || (!h && !d)) return fail(h, NB_ERR_ARG, "null argument");
    if (h) {
        *out = instance_bytes(h->d, h->star_alloc, (long long)sizeof(float) * h->drive_field * h->hc.drive_slots);
        return NB_OK;
    }
    if (nstars < 0 || nstars > d->max_stars) return fail(nullptr, NB_ERR_LIMIT, "nstars must be in [0, max_stars]");
    *out = instance_bytes(*d, nstars, 0);
    return NB_OK;
}

NB_EXPORT void nb_destroy(nb_handle h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    else cudaDeviceSynchronize();
    void* ps[] = {h->c, h->st, h->stars, h->sw, h->maps, h->tmp_maps, h->dirs, h->dirs_fuv,
                  h->rfront, h->att, h->scratch3, h->red, h->plane_xf, h->drive_ring, h->front_parts};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (h->state_mirror) cudaFreeHost(h->state_mirror);
    for (auto& r : h->recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : h->pool) cudaEventDestroy(e);
    delete h;
}

NB_EXPORT int nb_set_live(nb_handle h, const nb_live* L) {
    if (!h || !L) return fail(h, NB_ERR_ARG, "null argument");
    NbConst& c = h->hc;
    c.q_main = L->q_main;
    c.wind = L->wind;
    c.jet = L->jet;
    c.jet_proto = L->jet_proto;
    c.jet_pulse = L->jet_pulse;
    c.jet_period = L->jet_period;
    c.kappa_fuv = L->kappa_fuv;
    c.q_ramp = L->q_ramp;
    c.jet_r = L->jet_r;
    c.jet_cos = std::cos(L->jet_angle_deg * (3.141592653589793 / 180.0));   // sim.py:1018 math.cos(math.radians(.))
    c.dt_cap = L->dt_cap;
    c.phase_main = L->phase_main;
    c.wind_f = (float)L->wind;
    c.jet_cos_f = (float)c.jet_cos;
    c.jet_r_f = (float)L->jet_r;
    c.kappa_f = (float)L->kappa_fuv;
    c.plane_F = L->plane_flux;
    c.plane_lum = L->plane_fuv;
    c.plane_on = L->plane_flux > 0.0 ? 1 : 0;
    c.plane_F_f = (float)L->plane_flux;
    c.plane_lum_f = (float)L->plane_fuv;
    c.pre_amp = L->pre_amp;
    c.drive_main = L->drive_main;
    return upload_const(h);
}

NB_EXPORT int nb_set_stars(nb_handle h, const nb_star* s, int n) {
    if (!h || (n > 0 && !s)) return fail(h, NB_ERR_ARG, "null argument");
    if (n < 0 || n > h->d.max_stars) return fail(h, NB_ERR_LIMIT, "more stars than max_stars");
    if (n > h->star_alloc) {
        CK(h, cudaStreamSynchronize(h->stream));
        if (h->rfront) cudaFree(h->rfront);
        if (h->att) cudaFree(h->att);
        h->rfront = nullptr;
        h->att = nullptr;
        h->star_alloc = 0;
        // room for the float2 pair layouts (NB_TUNE_FRONT_PAIRS / NB_TUNE_FUV_PAIRS may switch at any time)
        const size_t rf = 2 * sizeof(float) * (size_t)n * h->d.nu * h->d.nphi;
        const size_t at = 2 * sizeof(float) * (size_t)n * h->d.fnr * h->d.fnu * h->d.fnphi;
        if (cudaMalloc(&h->rfront, rf) != cudaSuccess || cudaMalloc(&h->att, at) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, NB_ERR_NOMEM, "ray scratch allocation refused");
        }
        h->star_alloc = n;
    }
    NbStarDev tmp[NB_MAX_STARS];
    for (int i = 0; i < n; ++i) {
        tmp[i].x = s[i].x; tmp[i].y = s[i].y; tmp[i].z = s[i].z;
        tmp[i].qf = s[i].qf; tmp[i].t_on = s[i].t_on;
        tmp[i].ax = s[i].ax; tmp[i].ay = s[i].ay; tmp[i].az = s[i].az;
        tmp[i].kind = s[i].kind; tmp[i].jkind = s[i].jkind;
    }
    if (n > 0) CK(h, cudaMemcpyAsync(h->stars, tmp, sizeof(NbStarDev) * n, cudaMemcpyHostToDevice, h->stream));
    h->nstars = n;
    h->hc.nstars = n;
    return upload_const(h);
}

NB_EXPORT int nb_set_clock(nb_handle h, const nb_clock* c) {
    if (!h || !c) return fail(h, NB_ERR_ARG, "null argument");
    NbState s{};
    CK(h, cudaMemcpyAsync(&s, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    s.t = c->t;
    s.dt = c->dt;
    s.it = c->it;
    s.tp = c->tp;
    s.ip = c->ip;
    CK(h, cudaMemcpyAsync(h->st, &s, sizeof(NbState), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *h->state_mirror = s;
    h->host_it = c->it;
    h->smax_valid = 0;
    return NB_OK;
}

// A hydro stage whose bounded TMA wait gave up left the rest of its tile unwritten, so every
// clock read after it reports NB_ERR_TIMEOUT (the clock itself is still returned).  The device
// status bit stays set for the life of the handle.
static int clock_status(nb_instance* h, const NbState& s) {
    if (s.status & NB_DEV_TMA_TIMEOUT)
        return fail(h, NB_ERR_TIMEOUT, "a bounded TMA wait in a hydro stage gave up on the device: the fields "
                                       "are incomplete since then (nb_device_status)");
    return NB_OK;
}

NB_EXPORT int nb_mirror_clock(nb_handle h) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    return mirror_state(h);
}

NB_EXPORT int nb_peek_clock(nb_handle h, nb_clock* c) {
    if (!h || !c) return fail(h, NB_ERR_ARG, "null argument");
    const NbState& s = *h->state_mirror;
    c->t = s.t;
    c->dt = s.dt;
    c->it = s.it;
    c->tp = s.tp;
    c->ip = s.ip;
    return clock_status(h, s);
}

NB_EXPORT int nb_get_clock(nb_handle h, nb_clock* c) {
    if (!h || !c) return fail(h, NB_ERR_ARG, "null argument");
    NbState s{};
    CK(h, cudaMemcpyAsync(&s, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    c->t = s.t;
    c->dt = s.dt;
    c->it = s.it;
    c->tp = s.tp;
    c->ip = s.ip;
    return clock_status(h, s);
}

NB_EXPORT int nb_device_status(nb_handle h, int* status) {
    if (!h || !status) return fail(h, NB_ERR_ARG, "null argument");
    NbState s{};
    CK(h, cudaMemcpyAsync(&s, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    *status = (int)s.status;
    return NB_OK;
}

NB_EXPORT int nb_invalidate(nb_handle h) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    h->smax_valid = 0;
    return NB_OK;
}

NB_EXPORT int nb_step(nb_handle h, int k, int ion_every) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    if (k < 0 || ion_every < 1) return fail(h, NB_ERR_ARG, "k >= 0 and ion_every >= 1 required");
    if (!h->hc.phase_main) return fail(h, NB_ERR_STATE, "the main phase has not started");
    for (int s = 0; s < k; ++s) {
        int rc = do_step(h, ion_every);
        if (rc != NB_OK) return rc;
    }
    return NB_OK;
}

NB_EXPORT int nb_pre_step(nb_handle h, int k) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    if (k < 0) return fail(h, NB_ERR_ARG, "k >= 0 required");
    if (h->hc.phase_main) return fail(h, NB_ERR_STATE, "the stirring phase is over");
    if (!h->drive_ring || h->hc.drive_pushed < 2)
        return fail(h, NB_ERR_STATE, "stirring needs nb_drive_config and two pushed forcing fields");
    for (int s = 0; s < k; ++s) {
        int rc = do_pre_step(h);
        if (rc != NB_OK) return rc;
    }
    return NB_OK;
}

// ============================================================================ stirring
NB_EXPORT int nb_drive_config(nb_handle h, const nb_drive_desc* d) {
    if (!h || !d) return fail(h, NB_ERR_ARG, "null argument");
    if (d->sx < 1 || d->sy < 1 || d->sz < 1 || d->slots < 3 || !(d->dxs > 0.0) || !(d->pre_corr > 0.0) ||
        !(d->clock >= 0.0))
        return fail(h, NB_ERR_ARG, "forcing grid >= 1 cell per axis, slots >= 3, dxs > 0, pre_corr > 0, clock >= 0");
    const long long field = 3LL * d->sx * d->sy * d->sz;
    if (field * d->slots > (1LL << 31)) return fail(h, NB_ERR_LIMIT, "forcing ring above 2^31 floats");
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->drive_ring) cudaFree(h->drive_ring);
    h->drive_ring = nullptr;
    if (cudaMalloc(&h->drive_ring, sizeof(float) * field * d->slots) != cudaSuccess) {
        cudaGetLastError();
        h->hc.drive_ring = nullptr;
        h->hc.drive_slots = 0;
        h->hc.drive_pushed = 0;
        upload_const(h);
        return fail(h, NB_ERR_NOMEM, "forcing ring allocation refused");
    }
    h->drive_field = field;
    NbConst& c = h->hc;
    c.drive_ring = h->drive_ring;
    c.drive_sx = d->sx; c.drive_sy = d->sy; c.drive_sz = d->sz;
    c.drive_slots = d->slots;
    c.drive_pushed = 0;
    c.drive_dxs_f = (float)d->dxs;
    c.drive_pre_corr = d->pre_corr;
    NbState s{};
    CK(h, cudaMemcpyAsync(&s, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    s.dclock = d->clock;
    s.dswaps = 0;
    s.drive_go = 0;
    CK(h, cudaMemcpyAsync(h->st, &s, sizeof(NbState), cudaMemcpyHostToDevice, h->stream));
    int rc = upload_const(h);
    if (rc != NB_OK) return rc;
    CK(h, cudaStreamSynchronize(h->stream));
    return NB_OK;
}

NB_EXPORT int nb_drive_push(nb_handle h, const float* fields, int n) {
    if (!h || (n > 0 && !fields)) return fail(h, NB_ERR_ARG, "null argument");
    if (n < 0) return fail(h, NB_ERR_ARG, "n >= 0 required");
    if (!h->drive_ring) return fail(h, NB_ERR_STATE, "nb_drive_config first");
    if (n == 0) return NB_OK;
    NbState s{};
    CK(h, cudaMemcpyAsync(&s, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    NbConst& c = h->hc;
    // the ring holds fields dswaps .. dswaps + slots - 1; A and B (fields dswaps, dswaps + 1) stay
    if (c.drive_pushed + n > s.dswaps + c.drive_slots)
        return fail(h, NB_ERR_LIMIT, "forcing ring full: the fields in it are still to be used");
    for (int m = 0; m < n; ++m) {
        const long long slot = (c.drive_pushed + m) % c.drive_slots;
        CK(h, cudaMemcpyAsync(h->drive_ring + slot * h->drive_field, fields + (long long)m * h->drive_field,
                              sizeof(float) * h->drive_field, cudaMemcpyHostToDevice, h->stream));
    }
    c.drive_pushed += n;
    int rc = upload_const(h);
    if (rc != NB_OK) return rc;
    CK(h, cudaStreamSynchronize(h->stream));
    return NB_OK;
}

NB_EXPORT int nb_drive_enable(nb_handle h, int on) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    h->hc.drive_on = on ? 1 : 0;
    return upload_const(h);
}

NB_EXPORT int nb_drive_state(nb_handle h, nb_drive_info* out) {
    if (!h || !out) return fail(h, NB_ERR_ARG, "null argument");
    NbState s{};
    CK(h, cudaMemcpyAsync(&s, h->st, sizeof(NbState), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    out->clock = s.dclock;
    out->swaps = s.dswaps;
    out->pushed = h->hc.drive_pushed;
    out->status = (int)s.status;
    return NB_OK;
}

NB_EXPORT int nb_drive_step(nb_handle h, const float* fa, const float* fb, float blend, float amp, float dt) {
    if (!h || !fa || !fb) return fail(h, NB_ERR_ARG, "null argument");
    if (!h->drive_ring) return fail(h, NB_ERR_STATE, "nb_drive_config first (it sets the forcing grid)");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_DRIVE, 1);
    CK(h, nb_launch_drive_explicit(h->c, f.rho, f.mx, f.my, f.mz, fa, fb, blend, amp, dt, h->d.nx, h->d.ny,
                                   h->hc.drive_sz, h->stream));
    return NB_OK;
}

NB_EXPORT int nb_add_torus(nb_handle h, const float* torus) {
    if (!h || !torus) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_DRIVE, 1);
    CK(h, nb_launch_add_torus(torus, f.rho, f.mx, f.my, f.mz, h->ncell, h->stream));
    h->smax_valid = 0;
    return NB_OK;
}

NB_EXPORT int nb_mach_sums(nb_handle h, double out[2]) {
    if (!h || !out) return fail(h, NB_ERR_ARG, "null argument");
    if (nb_mach_scratch_doubles() > nb_reduce_scratch_doubles()) return fail(h, NB_ERR_LIMIT, "reduction scratch");
    const nb_fields& f = h->d.f;
    CK(h, nb_launch_mach_sums(f.rho, f.mx, f.my, f.mz, h->ncell, h->red, h->stream));
    CK(h, cudaMemcpyAsync(out, h->red + nb_mach_scratch_doubles() - 2, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return NB_OK;
}

NB_EXPORT int nb_render_pack(nb_handle h, const nb_pack_params* pp, int shock_on, int smooth, void* out8,
                             void* tmp8) {
    if (!h || !pp || !out8 || (smooth && !tmp8)) return fail(h, NB_ERR_ARG, "null argument");
    if (!aligned16(out8) || (smooth && !aligned16(tmp8))) return fail(h, NB_ERR_ARG, "voxel grids must be 16-byte aligned");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_RENDER, smooth ? 4 : 1);
    CK(h, nb_launch_render_pack(h->c, f.rho, f.mx, f.my, f.mz, f.xi, f.dfront, f.g0, h->d.fields_fp32 ? 0 : 1, *pp,
                                shock_on, smooth, out8, tmp8, h->d.nx, h->d.ny, h->stream));
    return NB_OK;
}

NB_EXPORT int nb_ionize(nb_handle h) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    return do_ionize(h);
}

NB_EXPORT int nb_fuv(nb_handle h) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    const size_t es = h->d.fields_fp32 ? 4 : 2;
    if (!h->hc.phase_main) {                                         // sim.py:952-954
        CK(h, cudaMemsetAsync(h->d.f.g0, 0, es * h->ncell, h->stream));
        return NB_OK;
    }
    {
        Prof pf(h, NB_PROF_CTRL, 1);
        CK(h, nb_launch_weights(h->c, h->st, h->stars, h->sw, h->nstars, h->stream));
    }
    if (h->nstars > 0) {
        Prof pf(h, NB_PROF_CAST_FUV, 2);                // the (rho, xi) pack into stage planes 0-1 + the rays
        CK(h, nb_launch_cast_fuv(h->c, h->sw, h->dirs_fuv, h->d.f.rho, h->d.f.xi, h->att, h->nstars, h->fuv_group,
                                 nullptr, 0, h->stream, h->d.fnu, h->d.fnphi, plane(h, 0), h->ncell,
                                 h->fuv_cut ? NB_FUV_TAU_CUT : 0.0f, h->fuv_pairs));
    }
    if (h->hc.plane_on) {
        Prof pf(h, NB_PROF_CAST_FUV, 1);
        CK(h, nb_launch_plane_fuv(h->c, h->d.f.rho, h->d.f.xi, plane(h, 2), h->d.ny, h->d.nz, h->stream));
    }
    {
        Prof pf(h, NB_PROF_APPLY_FUV, 1);
        CK(h, nb_launch_apply_fuv(h->c, h->sw, h->att, h->nstars, h->d.f.g0, h->stream, h->d.nx,
                                  h->d.ny, h->d.fields_fp32 ? 0 : 1, h->fuv_pairs));
    }
    return NB_OK;
}

NB_EXPORT int nb_hydro_stage(nb_handle h, const float* const in4[4], const float* const u0_4[4],
                             float* const out4[4], float a, float b, float dt, float pulse) {
    if (!h || !in4 || !u0_4 || !out4) return fail(h, NB_ERR_ARG, "null argument");
    for (int f = 0; f < 4; ++f)
        if (!in4[f] || !u0_4[f] || !out4[f] || !aligned16(in4[f]))
            return fail(h, NB_ERR_ARG, "plane pointers must be non-null (inputs 16-byte aligned)");
    CUtensorMap hm[NB_NMAPS];
    for (int f = 0; f < 4; ++f)
        if (!encode_plane(&hm[f], in4[f], h->d.nx, h->d.ny, h->d.nz)) return fail(h, NB_ERR_CUDA, "tensor map");
    if (!encode_plane(&hm[NB_MAP_XI], h->d.f.xi, h->d.nx, h->d.ny, h->d.nz)) return fail(h, NB_ERR_CUDA, "tensor map");
    CK(h, cudaMemcpyAsync(h->tmp_maps, hm, sizeof(CUtensorMap) * 5, cudaMemcpyHostToDevice, h->stream));
    CK(h, nb_launch_weights(h->c, h->st, h->stars, h->sw, h->nstars, h->stream));
    int rc = launch_stage(h, in4, u0_4, out4, 0, h->tmp_maps, a, b, true, dt, pulse, false);
    if (rc != NB_OK) return rc;
    CK(h, cudaStreamSynchronize(h->stream));        // tmp_maps is reused by the next call
    return NB_OK;
}

NB_EXPORT int nb_max_speed(nb_handle h, float* smax_out) {
    if (!h || !smax_out) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    CK(h, nb_launch_max_speed(h->c, f.rho, f.mx, f.my, f.mz, f.xi, &h->st->smax_bits, h->ncell, h->stream));
    unsigned bits = 0;
    CK(h, cudaMemcpyAsync(&bits, &h->st->smax_bits, 4, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    std::memcpy(smax_out, &bits, 4);
    h->smax_valid = 1;
    return NB_OK;
}

NB_EXPORT int nb_cast_rays(nb_handle h, const double xyz[3], double Q, float* rfront_out) {
    if (!h || !xyz || !rfront_out) return fail(h, NB_ERR_ARG, "null argument");
    float s3[4] = {(float)xyz[0], (float)xyz[1], (float)xyz[2], 0.f};
    CK(h, cudaMemcpyAsync(h->scratch3, s3, sizeof(s3), cudaMemcpyHostToDevice, h->stream));
    CK(h, nb_launch_cast_rays(h->c, h->sw, h->dirs, h->d.f.rho, rfront_out, 1, h->ray_group, h->scratch3, (float)Q,
                              h->stream, h->d.nu, h->d.nphi, 0));
    CK(h, cudaStreamSynchronize(h->stream));
    return NB_OK;
}

NB_EXPORT int nb_cast_fuv(nb_handle h, const double xyz[3], float* att_out) {
    if (!h || !xyz || !att_out) return fail(h, NB_ERR_ARG, "null argument");
    float s3[4] = {(float)xyz[0], (float)xyz[1], (float)xyz[2], 0.f};
    CK(h, cudaMemcpyAsync(h->scratch3, s3, sizeof(s3), cudaMemcpyHostToDevice, h->stream));
    CK(h, nb_launch_cast_fuv(h->c, h->sw, h->dirs_fuv, h->d.f.rho, h->d.f.xi, att_out, 1, 32, h->scratch3, 1,
                             h->stream, h->d.fnu, h->d.fnphi, plane(h, 0), h->ncell, h->fuv_cut ? NB_FUV_TAU_CUT : 0.0f,
                             0));
    CK(h, cudaStreamSynchronize(h->stream));
    return NB_OK;
}

NB_EXPORT int nb_reduce_fp64(nb_handle h, double out[4]) {
    if (!h || !out) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    CK(h, nb_launch_reduce_fp64(f.rho, f.mx, f.my, f.mz, h->ncell, h->red, h->stream));
    CK(h, cudaMemcpyAsync(out, h->red + nb_reduce_scratch_doubles() - 4, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return NB_OK;
}

NB_EXPORT int nb_profile(nb_handle h, int enable) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    h->profiling = enable ? 1 : 0;
    return NB_OK;
}

NB_EXPORT int nb_profile_read(nb_handle h, double ms[NB_PROF_KINDS], long long count[NB_PROF_KINDS]) {
    if (!h || !ms || !count) return fail(h, NB_ERR_ARG, "null argument");
    CK(h, cudaStreamSynchronize(h->stream));
    for (int k = 0; k < NB_PROF_KINDS; ++k) {
        ms[k] = 0.0;
        count[k] = 0;
    }
    for (auto& r : h->recs) {
        float t = 0.0f;
        CK(h, cudaEventElapsedTime(&t, r.a, r.b));
        if (r.kind >= 0 && r.kind < NB_PROF_KINDS) {
            ms[r.kind] += t;
            count[r.kind] += 1;
        }
        h->pool.push_back(r.a);
        h->pool.push_back(r.b);
    }
    h->recs.clear();
    return NB_OK;
}

NB_EXPORT int nb_counters(nb_handle h, long long* launches) {
    if (!h || !launches) return fail(h, NB_ERR_ARG, "null argument");
    *launches = h->launches;
    return NB_OK;
}

NB_EXPORT int nb_snapshot_pack(nb_handle h, void* out13) {
    if (!h || !out13) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_SNAPSHOT, 1);
    CK(h, nb_launch_pack(h->c, f.rho, f.mx, f.my, f.mz, f.xi, f.dfront, f.g0, h->d.fields_fp32 ? 0 : 1, out13,
                         h->ncell, h->stream));
    return NB_OK;
}

NB_EXPORT int nb_snapshot_unpack(nb_handle h, const void* in13) {
    if (!h || !in13) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_SNAPSHOT, 1);
    CK(h, nb_launch_unpack(h->c, in13, h->ncell, f.rho, f.mx, f.my, f.mz, f.xi, f.dfront, f.g0,
                           h->d.fields_fp32 ? 0 : 1, h->stream));
    h->smax_valid = 0;                     // the state changed outside a step
    return NB_OK;
}

NB_EXPORT int nb_frame_pack(nb_handle h, void* out9) {
    if (!h || !out9) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_SNAPSHOT, 1);
    CK(h, nb_launch_frame(h->c, f.rho, f.mx, f.my, f.mz, f.xi, f.dfront, f.g0, h->d.fields_fp32 ? 0 : 1, out9,
                          h->ncell, h->d.nx, h->d.ny, h->stream));
    return NB_OK;
}

NB_EXPORT int nb_shock(nb_handle h, float* out) {
    if (!h || !out) return fail(h, NB_ERR_ARG, "null argument");
    const nb_fields& f = h->d.f;
    Prof pf(h, NB_PROF_SNAPSHOT, 1);
    CK(h, nb_launch_shock(h->c, f.rho, f.mx, f.my, f.mz, out, h->d.nx, h->d.ny, h->stream));
    return NB_OK;
}

NB_EXPORT int nb_get_tuning(nb_handle h, int key, int* value) {
    if (!h || !value) return fail(h, NB_ERR_ARG, "null argument");
    switch (key) {
        case NB_TUNE_CHUNK_I: *value = h->chunk_i; return NB_OK;
        case NB_TUNE_RAY_GROUP: *value = h->ray_group; return NB_OK;
        case NB_TUNE_FUV_GROUP: *value = h->fuv_group; return NB_OK;
        case NB_TUNE_TILE_ORDER: *value = h->tile_order; return NB_OK;
        case NB_TUNE_FRONT_CULL: *value = h->front_cull; return NB_OK;
        case NB_TUNE_FUV_CUT: *value = h->fuv_cut; return NB_OK;
        case NB_TUNE_WAIT_LIMIT: *value = (int)h->wait_limit; return NB_OK;
        case NB_TUNE_STALL_TEST: *value = h->stall_test; return NB_OK;
        case NB_TUNE_FRONT_PAIRS: *value = h->front_pairs; return NB_OK;
        case NB_TUNE_FUV_PAIRS: *value = h->fuv_pairs; return NB_OK;
        default: return fail(h, NB_ERR_ARG, "unknown tuning key");
    }
}

NB_EXPORT int nb_set_tuning(nb_handle h, int key, int value) {
    if (!h) return fail(h, NB_ERR_ARG, "null handle");
    switch (key) {
        case NB_TUNE_CHUNK_I:
            if (value < 1) return fail(h, NB_ERR_ARG, "chunk_i must be >= 1");
            h->chunk_i = value;
            return NB_OK;
        case NB_TUNE_TILE_ORDER:
            if (value != 0 && value != 1) return fail(h, NB_ERR_ARG, "tile order must be 0 or 1");
            h->tile_order = value;
            return NB_OK;
        case NB_TUNE_FRONT_CULL:
            if (value != 0 && value != 1) return fail(h, NB_ERR_ARG, "front culling must be 0 or 1");
            h->front_cull = value;
            return NB_OK;
        case NB_TUNE_FUV_CUT:
            if (value != 0 && value != 1) return fail(h, NB_ERR_ARG, "FUV cut must be 0 or 1");
            h->fuv_cut = value;
            return NB_OK;
        case NB_TUNE_WAIT_LIMIT:
            if (value < 1 || (unsigned)value > NB_WAIT_LIMIT)
                return fail(h, NB_ERR_ARG, "the wait limit must be in [1, 2^22] polls");
            h->wait_limit = (unsigned)value;
            return NB_OK;
        case NB_TUNE_STALL_TEST:
            if (value != 0 && value != 1) return fail(h, NB_ERR_ARG, "the stall test switch must be 0 or 1");
            h->stall_test = value;
            return NB_OK;
        case NB_TUNE_FRONT_PAIRS:
        case NB_TUNE_FUV_PAIRS:
            if (value != 0 && value != 1) return fail(h, NB_ERR_ARG, "a pair-table switch must be 0 or 1");
            (key == NB_TUNE_FRONT_PAIRS ? h->front_pairs : h->fuv_pairs) = value;
            return NB_OK;
        case NB_TUNE_RAY_GROUP:
        case NB_TUNE_FUV_GROUP:
            if (value != 8 && value != 16 && value != 32 &&
                !((value == 1 || value == 2 || value == 4) && key == NB_TUNE_RAY_GROUP))
                return fail(h, NB_ERR_ARG, "lanes per ray must be 1, 2, 4 (ionizing rays only), 8, 16 or 32");
            (key == NB_TUNE_RAY_GROUP ? h->ray_group : h->fuv_group) = value;
            return NB_OK;
        default:
            return fail(h, NB_ERR_ARG, "unknown tuning key");
    }
}

// ============================================================================ batches
// Many instances advanced together: one persistent launch per RK2 stage over a tile work-list
// spanning all of them (largest instances first), one launch for every instance's control
// block, three launches for the ionization of every instance due to ionize, and each whole
// step replayed as a CUDA graph.  Every instance keeps its own clock, CFL dt and cadence.
struct nb_batch_s {
    std::vector<nb_instance*> inst;
    std::vector<int> ion_every;
    cudaStream_t user = nullptr;        // the instances' stream
    cudaStream_t bs = nullptr;          // the batch's own stream (capturable)
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    int solver = 0, limiter = 0, max_stars = 1, grid = 0, ray_group = 1;
    int idx32 = 1;                      // every instance below 2^31 cells: 32-bit cell offsets
    NbBatchInst* d_inst = nullptr;
    HydroLaunch* d_L1 = nullptr;
    HydroLaunch* d_L2 = nullptr;
    int2* d_work = nullptr;             // the work items of the active instances, in list order
    int n_work = 0;                     // ... their count
    std::vector<int2> h_work;           // every instance's items, in list order
    unsigned* d_counters = nullptr;
    NbRayJob* d_jobs_all = nullptr;     // every instance ionizes (the lockstep case)
    long long all_groups = 0, all_blocks = 0;
    NbRayJob* d_jobs = nullptr;         // a per-step subset
    std::vector<NbRayJob> h_all;
    std::vector<NbBatchInst> h_inst;    // host copies of the descriptors (nb_batch_set_active re-uploads them)
    std::vector<HydroLaunch> h_L1, h_L2;
    // the stage records as the persistent kernel's parameter (at most NB_BATCH_PARAM_MAX instances,
    // 32-bit offsets; their active flags are not read: the kernel takes those from d_L1 / d_L2)
    std::unique_ptr<NbBatchRecords> rec1, rec2;
    std::vector<int> active;            // per instance: 1 = its slot steps, 0 = idle
    int n_active = 0;
    std::vector<const float*> rfront0;  // each instance's ray scratch when the batch was built
    std::vector<int> nstars0;
    int use_graphs = 1;
    int n_plane = 0;                    // instances with the plane source (one extra launch each)
    cudaGraphExec_t g_plain = nullptr, g_ion = nullptr;
    int warm_plain = 0, warm_ion = 0;
    long long launches = 0;
    std::string err;
};

namespace {

int bfail(nb_batch_s* b, int code, const std::string& m) {
    b->err = m;
    return code;
}
#define BCK(b, call)                                                                        \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return bfail((b), NB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

HydroLaunch stage_desc(nb_instance* h, bool stage2) {
    HydroLaunch L{};
    const nb_fields& f = h->d.f;
    L.c = h->c;
    L.st = h->st;
    L.sw = h->sw;
    L.maps = h->maps;
    L.map_in = stage2 ? NB_MAP_S0 : NB_MAP_RHO;
    for (int c = 0; c < 4; ++c) {
        float* S = plane(h, c);
        float* U[4] = {f.rho, f.mx, f.my, f.mz};
        L.in[c] = stage2 ? S : U[c];
        L.u0[c] = U[c];
        L.out[c] = stage2 ? U[c] : S;
    }
    L.xi = f.xi;
    L.a = stage2 ? 0.5f : 0.0f;
    L.b = stage2 ? 0.5f : 1.0f;
    L.smax_bits = stage2 ? &h->st->smax_bits : nullptr;
    L.status = &h->st->status;
    const int tj = nb_hydro_tile_j();
    L.tiles_k = (h->d.nz + 31) / 32;
    L.tiles_j = (h->d.ny + tj - 1) / tj;
    L.chunk_i = h->chunk_i < h->d.nx ? h->chunk_i : h->d.nx;
    L.n_chunks = (h->d.nx + L.chunk_i - 1) / L.chunk_i;
    L.nstars_host = h->nstars;
    L.order = h->tile_order;
    L.wait_limit = h->wait_limit;
    if (h->stall_test) L.maps = nullptr;
    L.active = 1;
    return L;
}

NbRayJob ray_job(nb_instance* h) {
    NbRayJob J{};
    const nb_fields& f = h->d.f;
    J.c = h->c;
    J.sw = h->sw;
    J.dirs = h->dirs;
    J.rho = f.rho;
    J.mx = f.mx;
    J.my = f.my;
    J.mz = f.mz;
    J.rfront = h->rfront;
    J.xi_raw = plane(h, 0);
    J.xi = f.xi;
    J.dfront = f.dfront;
    J.smax = &h->st->smax_bits;
    J.nstars = h->nstars;
    J.half = h->d.fields_fp32 ? 0 : 1;
    J.front_parts = (h->front_cull && h->nstars >= 1 && h->nstars <= NB_ROW_STARS) ? h->front_parts : nullptr;
    J.nray = (long long)h->d.nu * h->d.nphi;
    J.pairs = h->front_pairs;
    J.active = 1;
    return J;
}

// prefix sums of ray groups and row blocks over a job list; returns (groups, blocks)
void job_prefix(std::vector<NbRayJob>& jobs, const std::vector<nb_instance*>& hs, long long& groups, long long& blocks) {
    groups = 0;
    blocks = 0;
    for (size_t e = 0; e < jobs.size(); ++e) {
        jobs[e].ray0 = groups;
        jobs[e].blk0 = blocks;
        groups += (long long)hs[e]->nstars * hs[e]->d.nu * hs[e]->d.nphi;
        blocks += ((long long)hs[e]->d.nx * hs[e]->d.ny + 7) / 8;
    }
}

int batch_hydro(nb_batch_s* b) {
    b->launches += 3;
    BCK(b, nb_launch_ctrl_batch(b->d_inst, (int)b->inst.size(), 1, b->d_counters, b->bs));
    BCK(b, nb_launch_hydro_batch(b->d_L1, b->rec1.get(), b->d_work, b->n_work, b->d_counters + 0, b->max_stars, 0,
                                 b->idx32, b->solver, b->limiter, b->grid, b->bs));
    BCK(b, nb_launch_hydro_batch(b->d_L2, b->rec2.get(), b->d_work, b->n_work, b->d_counters + 1, b->max_stars, 1,
                                 b->idx32, b->solver, b->limiter, b->grid, b->bs));
    return NB_OK;
}

int batch_ionize(nb_batch_s* b, const NbRayJob* jobs, const NbRayJob* host_jobs, int n_jobs, long long groups,
                 long long blocks, const std::vector<int>& listed) {
    b->launches += 5;                       // control, rays, front ranges, front apply, smoothing
    BCK(b, nb_launch_ctrl_batch(b->d_inst, (int)b->inst.size(), 0, nullptr, b->bs));
    for (int i : listed) {
        nb_instance* h = b->inst[i];
        if (!h->hc.plane_on) continue;
        b->launches += 1;
        BCK(b, nb_launch_plane_front(h->c, h->d.f.rho, h->plane_xf, h->d.ny, h->d.nz, b->bs));
    }
    BCK(b, nb_launch_ionize_batch(jobs, host_jobs, n_jobs, groups, blocks, b->ray_group, b->bs));
    return NB_OK;
}

int batch_run_graph(nb_batch_s* b, cudaGraphExec_t* g, int ion) {
    if (!*g) {
        cudaGraph_t graph = nullptr;
        BCK(b, cudaStreamBeginCapture(b->bs, cudaStreamCaptureModeRelaxed));
        std::vector<int> all(b->inst.size());
        for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
        int rc = ion ? batch_ionize(b, b->d_jobs_all, b->h_all.data(), (int)b->inst.size(), b->all_groups, b->all_blocks, all) : NB_OK;
        if (rc == NB_OK) rc = batch_hydro(b);
        cudaError_t e = cudaStreamEndCapture(b->bs, &graph);
        if (rc != NB_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return bfail(b, NB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(g, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return bfail(b, NB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        b->launches -= ion ? 8 + b->n_plane : 3;       // captured, not launched
    }
    b->launches += ion ? 8 + b->n_plane : 3;
    BCK(b, cudaGraphLaunch(*g, b->bs));
    return NB_OK;
}

}  // namespace

NB_EXPORT const char* nb_batch_last_error(nb_batch b) { return b ? b->err.c_str() : g_err.c_str(); }

NB_EXPORT int nb_batch_create(const nb_handle* hs, const int* ion_every, int n, nb_batch* out) {
    if (!hs || !ion_every || !out || n < 1) return fail(nullptr, NB_ERR_ARG, "nb_batch_create: bad arguments");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!hs[i] || ion_every[i] < 1) return fail(nullptr, NB_ERR_ARG, "nb_batch_create: null handle / ion_every < 1");
        if (hs[i]->d.solver != hs[0]->d.solver || hs[i]->d.limiter != hs[0]->d.limiter)
            return fail(nullptr, NB_ERR_ARG, "nb_batch_create: all instances need the same solver and limiter");
        if (hs[i]->stream != hs[0]->stream)
            return fail(nullptr, NB_ERR_ARG, "nb_batch_create: all instances need the same stream");
        if (!hs[i]->hc.phase_main) return fail(nullptr, NB_ERR_STATE, "nb_batch_create: main phase not started");
        for (int j = 0; j < i; ++j)
            if (hs[j] == hs[i]) return fail(nullptr, NB_ERR_ARG, "nb_batch_create: an instance appears twice");
    }
    nb_batch_s* b = new nb_batch_s();
    auto bail = [&](int rc, const std::string& m) {
        g_err = m;
        nb_batch_destroy(b);
        return rc;
    };
    b->inst.assign(hs, hs + n);
    b->ion_every.assign(ion_every, ion_every + n);
    for (int i = 0; i < n; ++i) {
        b->rfront0.push_back(hs[i]->rfront);
        b->nstars0.push_back(hs[i]->nstars);
    }
    b->user = hs[0]->stream;
    b->solver = hs[0]->d.solver;
    b->limiter = hs[0]->d.limiter;
    b->ray_group = hs[0]->ray_group;
    for (auto* h : b->inst) {
        b->max_stars = std::max(b->max_stars, h->nstars);
        b->n_plane += h->hc.plane_on ? 1 : 0;
        if (h->ncell >= (1LL << 31)) b->idx32 = 0;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int params = b->idx32 && n <= NB_BATCH_PARAM_MAX;
    b->grid = (sms > 0 ? sms : 152) * nb_hydro_batch_blocks_per_sm(b->solver, b->limiter, b->max_stars, b->idx32, params);
    if (cudaStreamCreateWithFlags(&b->bs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming) != cudaSuccess)
        return bail(NB_ERR_CUDA, "nb_batch_create: stream / event creation failed");
    // descriptors
    std::vector<NbBatchInst>& bi = b->h_inst;
    std::vector<HydroLaunch>& L1 = b->h_L1;
    std::vector<HydroLaunch>& L2 = b->h_L2;
    bi.resize(n);
    L1.resize(n);
    L2.resize(n);
    b->active.assign(n, 1);
    b->n_active = n;
    for (int i = 0; i < n; ++i) {
        nb_instance* h = b->inst[i];
        bi[i] = NbBatchInst{h->c, h->st, h->stars, h->sw, h->nstars, 1};
        L1[i] = stage_desc(h, false);
        L2[i] = stage_desc(h, true);
    }
    if (params) {                                // the records as the persistent kernel's parameter
        b->rec1.reset(new NbBatchRecords());
        b->rec2.reset(new NbBatchRecords());
        for (int i = 0; i < n; ++i) {
            b->rec1->L[i] = L1[i];
            b->rec2->L[i] = L2[i];
        }
    }
    // work list: largest instances first, each instance's tiles in order
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->inst[a]->ncell > b->inst[c]->ncell; });
    std::vector<int2> work;
    for (int i : order) {
        const int tiles = L1[i].tiles_k * L1[i].tiles_j * L1[i].n_chunks;
        for (int t = 0; t < tiles; ++t) work.push_back(make_int2(i, t));
    }
    b->n_work = (int)work.size();
    b->h_work = work;
    b->h_all.resize(n);
    for (int i = 0; i < n; ++i) b->h_all[i] = ray_job(b->inst[i]);
    job_prefix(b->h_all, b->inst, b->all_groups, b->all_blocks);
    if (cudaMalloc(&b->d_inst, sizeof(NbBatchInst) * n) != cudaSuccess ||
        cudaMalloc(&b->d_L1, sizeof(HydroLaunch) * n) != cudaSuccess ||
        cudaMalloc(&b->d_L2, sizeof(HydroLaunch) * n) != cudaSuccess ||
        cudaMalloc(&b->d_work, sizeof(int2) * work.size()) != cudaSuccess ||
        cudaMalloc(&b->d_counters, 2 * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&b->d_jobs_all, sizeof(NbRayJob) * n) != cudaSuccess ||
        cudaMalloc(&b->d_jobs, sizeof(NbRayJob) * n) != cudaSuccess) {
        cudaGetLastError();
        return bail(NB_ERR_NOMEM, "nb_batch_create: device allocation refused");
    }
    cudaStream_t s = b->bs;
    if (cudaMemcpyAsync(b->d_inst, bi.data(), sizeof(NbBatchInst) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_L1, L1.data(), sizeof(HydroLaunch) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_L2, L2.data(), sizeof(HydroLaunch) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_work, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->d_jobs_all, b->h_all.data(), sizeof(NbRayJob) * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(b->d_counters, 0, 2 * sizeof(unsigned), s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return bail(NB_ERR_CUDA, "nb_batch_create: upload failed");
    *out = b;
    return NB_OK;
}

NB_EXPORT void nb_batch_destroy(nb_batch b) {
    if (!b) return;
    if (b->bs) cudaStreamSynchronize(b->bs);
    if (b->g_plain) cudaGraphExecDestroy(b->g_plain);
    if (b->g_ion) cudaGraphExecDestroy(b->g_ion);
    void* ps[] = {b->d_inst, b->d_L1, b->d_L2, b->d_work, b->d_counters, b->d_jobs_all, b->d_jobs};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (b->ev_in) cudaEventDestroy(b->ev_in);
    if (b->ev_out) cudaEventDestroy(b->ev_out);
    if (b->bs) cudaStreamDestroy(b->bs);
    delete b;
}

NB_EXPORT int nb_batch_set_option(nb_batch b, int key, int value) {
    if (!b) return fail(nullptr, NB_ERR_ARG, "null batch");
    switch (key) {
        case NB_BATCH_GRAPHS: b->use_graphs = value ? 1 : 0; return NB_OK;
        case NB_BATCH_GRID:
            if (value < 1) return bfail(b, NB_ERR_ARG, "grid must be >= 1");
            b->grid = value;
            break;
        case NB_BATCH_RAY_GROUP:
            if (value != 1 && value != 2 && value != 4 && value != 8 && value != 16 && value != 32)
                return bfail(b, NB_ERR_ARG, "bad ray group");
            b->ray_group = value;
            break;
        default: return bfail(b, NB_ERR_ARG, "unknown batch option");
    }
    // launch shapes are baked into captured graphs: drop them
    if (b->bs) cudaStreamSynchronize(b->bs);
    if (b->g_plain) cudaGraphExecDestroy(b->g_plain);
    if (b->g_ion) cudaGraphExecDestroy(b->g_ion);
    b->g_plain = b->g_ion = nullptr;
    b->warm_plain = b->warm_ion = 0;
    return NB_OK;
}

NB_EXPORT int nb_batch_set_active(nb_batch b, const int* active, int n) {
    if (!b || !active) return fail(nullptr, NB_ERR_ARG, "null argument");
    if (n != (int)b->inst.size()) return bfail(b, NB_ERR_ARG, "one flag per instance of the batch");
    int na = 0;
    for (int i = 0; i < n; ++i) {
        const int a = active[i] ? 1 : 0;
        b->active[i] = a;
        b->h_inst[i].active = a;
        b->h_L1[i].active = a;
        b->h_L2[i].active = a;
        b->h_all[i].active = a;
        na += a;
    }
    b->n_active = na;
    // the work list of the active instances only: an idle instance's tiles are not walked at all
    std::vector<int2> work;
    work.reserve(b->h_work.size());
    for (const int2& w : b->h_work)
        if (b->active[w.x]) work.push_back(w);
    b->n_work = (int)work.size();
    // in stream order before the next step; the captured graphs read these arrays when they run
    cudaStream_t s = b->bs;
    if (!work.empty())
        BCK(b, cudaMemcpyAsync(b->d_work, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, s));
    BCK(b, cudaMemcpyAsync(b->d_inst, b->h_inst.data(), sizeof(NbBatchInst) * n, cudaMemcpyHostToDevice, s));
    BCK(b, cudaMemcpyAsync(b->d_L1, b->h_L1.data(), sizeof(HydroLaunch) * n, cudaMemcpyHostToDevice, s));
    BCK(b, cudaMemcpyAsync(b->d_L2, b->h_L2.data(), sizeof(HydroLaunch) * n, cudaMemcpyHostToDevice, s));
    BCK(b, cudaMemcpyAsync(b->d_jobs_all, b->h_all.data(), sizeof(NbRayJob) * n, cudaMemcpyHostToDevice, s));
    BCK(b, cudaStreamSynchronize(s));            // the host arrays may change again at once
    return NB_OK;
}

NB_EXPORT int nb_batch_step(nb_batch b, int k) {
    if (!b) return fail(nullptr, NB_ERR_ARG, "null batch");
    if (k < 0) return bfail(b, NB_ERR_ARG, "k >= 0 required");
    const int n = (int)b->inst.size();
    for (int i = 0; i < n; ++i)
        if (b->active[i] && (b->inst[i]->rfront != b->rfront0[i] || b->inst[i]->nstars != b->nstars0[i]))
            return bfail(b, NB_ERR_STATE, "an instance's star table changed size since nb_batch_create: rebuild the batch");
    for (int i = 0; i < n; ++i)
        if (b->active[i] && (!b->inst[i]->hc.phase_main || stirring_main(b->inst[i])))
            return bfail(b, NB_ERR_STATE, "batched steps are main-phase steps without stirring: step stirred instances alone");
    if (b->n_active == 0) return NB_OK;          // every slot idle: nothing to step
    BCK(b, cudaEventRecord(b->ev_in, b->user));
    BCK(b, cudaStreamWaitEvent(b->bs, b->ev_in, 0));
    // an instance whose CFL max speed is stale and that does not ionize first needs a fresh one
    for (int i = 0; i < n; ++i) {
        nb_instance* h = b->inst[i];
        if (!b->active[i]) continue;
        if (!h->smax_valid && h->host_it % b->ion_every[i] != 0) {
            const nb_fields& f = h->d.f;
            BCK(b, nb_launch_max_speed(h->c, f.rho, f.mx, f.my, f.mz, f.xi, &h->st->smax_bits, h->ncell, b->bs));
            h->smax_valid = 1;
            b->launches += 2;
        }
    }
    for (int s = 0; s < k; ++s) {
        std::vector<int> due;
        for (int i = 0; i < n; ++i)
            if (b->active[i] && b->inst[i]->host_it % b->ion_every[i] == 0) due.push_back(i);
        int rc = NB_OK;
        // every slot active and every or no slot ionizing: the captured graphs.  With idle slots the
        // step is launched as it goes, on the active instances' work list and the due instances'
        // ray jobs only (a captured step would walk the idle instances' rays and cells too).
        const bool full = b->n_active == n;
        const bool all = (int)due.size() == n, none = due.empty();       // all: every slot active and due
        if (b->use_graphs && full && (all || none) && (all ? b->warm_ion : b->warm_plain)) {
            rc = batch_run_graph(b, all ? &b->g_ion : &b->g_plain, all ? 1 : 0);
        } else {
            if (all) {                           // every slot ionizes: the whole job list
                rc = batch_ionize(b, b->d_jobs_all, b->h_all.data(), n, b->all_groups, b->all_blocks, due);
                b->warm_ion = 1;
            } else if (!none) {
                std::vector<NbRayJob> jobs;
                std::vector<nb_instance*> hs;
                for (int i : due) {
                    jobs.push_back(b->h_all[i]);
                    hs.push_back(b->inst[i]);
                }
                long long groups = 0, blocks = 0;
                job_prefix(jobs, hs, groups, blocks);
                BCK(b, cudaMemcpyAsync(b->d_jobs, jobs.data(), sizeof(NbRayJob) * jobs.size(), cudaMemcpyHostToDevice,
                                       b->bs));
                rc = batch_ionize(b, b->d_jobs, jobs.data(), (int)jobs.size(), groups, blocks, due);
            } else {
                b->warm_plain = 1;
            }
            if (rc == NB_OK) rc = batch_hydro(b);
        }
        if (rc != NB_OK) return rc;
        for (int i = 0; i < n; ++i) {
            if (!b->active[i]) continue;
            b->inst[i]->host_it += 1;
            b->inst[i]->smax_valid = 1;
        }
    }
    BCK(b, cudaEventRecord(b->ev_out, b->bs));
    BCK(b, cudaStreamWaitEvent(b->user, b->ev_out, 0));
    return NB_OK;
}

NB_EXPORT int nb_batch_counters(nb_batch b, long long* launches) {
    if (!b || !launches) return fail(nullptr, NB_ERR_ARG, "null argument");
    *launches = b->launches;
    return NB_OK;
}
