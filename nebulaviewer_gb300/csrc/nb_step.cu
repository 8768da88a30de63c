// Device-side step control: the star weights of sim.py:880-925 (_set_star_weights, q_eff,
// ramp), the CFL time step of sim.py:1009-1012 / 1105-1107 and the jet pulse of sim.py:1108,
// all evaluated in FP64 exactly as the reference's Python floats are, then rounded to the
// float32 kernel arguments.  Keeping them on the device removes the per-step blocking
// device->host read of the reference (sim.py:1012), so a whole step can be replayed as a
// CUDA graph.  Also: the stand-alone CFL max-speed reduction (nebula3d.py:154-162) and the
// deterministic FP64 conservation totals.
#include <mutex>
#include <string>

#include "nb_internal.cuh"

namespace {

// sim.py:885-895 ramp(i) (the turn-on smoothstep^3), in IEEE double with no contraction
__device__ double ramp_of(const NbConst& c, const NbStarDev& s, double t) {
    const double age = __dsub_rn(t, s.t_on);
    if (!c.phase_main || age < 0.0) return 0.0;
    const double tr = c.q_ramp;
    if (tr <= 0.0 || age >= tr) return 1.0;
    const double x = __ddiv_rn(age, tr);
    const double sm = __dmul_rn(__dmul_rn(x, x), __dsub_rn(3.0, __dmul_rn(2.0, x)));
    const double s3 = __dmul_rn(__dmul_rn(sm, sm), sm);
    return (1e-4 > s3) ? 1e-4 : s3;                       // Python max(s*s*s, 1e-4)
}

__device__ void star_weight(const NbConst& c, const NbStarDev& s, double t, NbStarW& w) {
    const double q_of = s.kind == NB_STAR_MAIN ? __dmul_rn(s.qf, c.q_main) : s.qf;      // sim.py:880-883
    const double q_eff = __dmul_rn(q_of, ramp_of(c, s, t));                              // sim.py:897-898
    const bool on = t >= s.t_on;
    const double qn = __ddiv_rn(q_eff, c.q_main);
    w.w = make_float4((float)s.x, (float)s.y, (float)s.z, on ? (float)qn : 0.0f);       // sim.py:916
    const double js = s.jkind == NB_JET_JET ? c.jet : (s.jkind == NB_JET_PROTO ? c.jet_proto : 0.0);  // sim.py:900-902
    w.jet = make_float4((float)s.ax, (float)s.ay, (float)s.az, (float)js);               // sim.py:923
    w.q_f = (float)q_eff;                                                                // sim.py:937
    w.lum_f = (float)qn;                                                                 // sim.py:965
    w.active = on ? 1 : 0;                                                               // sim.py:934
    w.pad = 0;
}

// advance: 0 = star weights only; NB_ADV_MAIN = a main-phase step (sim.py:1104-1113);
// NB_ADV_PRE = a stirring-phase step (sim.py:1044-1050: dt without dt_cap, tp += dt)
__device__ __forceinline__ void ctrl_body(const NbConst* __restrict__ c, NbState* __restrict__ st,
                                          const NbStarDev* __restrict__ stars, NbStarW* __restrict__ sw, int nstars,
                                          int advance) {
    const double t = st->t;
    for (int s = threadIdx.x; s < nstars; s += blockDim.x) star_weight(*c, stars[s], t, sw[s]);
    __syncthreads();                                      // every thread has read t before it moves
    if (!advance || threadIdx.x != 0) return;
    const bool pre = advance == NB_ADV_PRE;
    // sim.py:1012: P['cfl'] * dx / float(smax)
    const double smax = (double)__uint_as_float(st->smax_bits);
    double dt = __ddiv_rn(__dmul_rn(c->cfl, c->dx_d), smax);
    double pulse = 0.0;
    if (!pre) {
        if (c->dt_cap > 0.0 && c->dt_cap < dt) dt = c->dt_cap;                           // sim.py:1106-1107
        // sim.py:1108: max(0, 1 + jet_pulse * sin(2 pi t / jet_period)).  Only the jet source reads
        // it; with jet == jet_proto == 0 every star's jet strength is 0 (sim.py:900-902) and the
        // FP64 sine is skipped
        if (c->jet != 0.0 || c->jet_proto != 0.0) {
            const double arg = __ddiv_rn(__dmul_rn(6.283185307179586, t), c->jet_period);
            pulse = __dadd_rn(1.0, __dmul_rn(c->jet_pulse, sin(arg)));
            if (!(pulse > 0.0)) pulse = 0.0;
        } else {
            pulse = 1.0;
        }
    }
    st->dt = dt;
    st->dt_f = (float)dt;
    st->pulse_f = (float)pulse;
    st->smax_bits = 0u;                                   // the step's last kernel accumulates the next max
    // sim.py:1030-1042 _stir: blend from the clock before this step, then clock += dt and, at
    // pre_corr, B becomes A and the next pushed field becomes B
    st->drive_go = 0;
    if (pre || (c->drive_on && c->drive_main > 0.0)) {
        const double q = __ddiv_rn(st->dclock, c->drive_pre_corr);
        st->blend_f = (float)(1.0 < q ? 1.0 : q);                                      // min(clock / pre_corr, 1)
        st->amp_f = (float)(pre ? c->pre_amp : __dmul_rn(c->pre_amp, c->drive_main));   // sim.py:1047, 1111
        if (st->dswaps + 1 < c->drive_pushed && c->drive_slots > 0) {
            st->drive_a = (int)(st->dswaps % c->drive_slots);
            st->drive_b = (int)((st->dswaps + 1) % c->drive_slots);
            st->drive_go = 1;
            const double clk = __dadd_rn(st->dclock, dt);
            if (clk >= c->drive_pre_corr) {
                st->dswaps = st->dswaps + 1;
                st->dclock = 0.0;
            } else {
                st->dclock = clk;
            }
        } else {
            st->status |= NB_DEV_DRIVE_EMPTY;
        }
    }
    if (pre) {
        st->tp = __dadd_rn(st->tp, dt);                   // sim.py:1048-1049
        st->ip = st->ip + 1;
    } else {
        st->t = __dadd_rn(t, dt);                         // sim.py:1112-1113
        st->it = st->it + 1;
    }
}

__global__ void ctrl_kernel(const NbConst* __restrict__ c, NbState* __restrict__ st,
                            const NbStarDev* __restrict__ stars, NbStarW* __restrict__ sw, int nstars,
                            int advance) {
    ctrl_body(c, st, stars, sw, nstars, advance);
}

// one block per instance of a batch; block 0 also resets the persistent stage kernels' counters
__global__ void ctrl_batch_kernel(const NbBatchInst* __restrict__ insts, int n, int advance, unsigned* counters) {
    const NbBatchInst& I = insts[blockIdx.x];
    if (counters && blockIdx.x == 0 && threadIdx.x == 0) {
        counters[0] = 0u;
        counters[1] = 0u;
    }
    if (!I.active) return;                       // an idle slot: its clock stays
    ctrl_body(I.c, I.st, I.stars, I.sw, I.nstars, advance);
}

// nebula3d.py:154-162 max_speed, as an exact max reduction (atomicMax on the bits of a
// non-negative float orders like the float)
__global__ void max_speed_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                 const float* __restrict__ mx, const float* __restrict__ my,
                                 const float* __restrict__ mz, const float* __restrict__ xi,
                                 unsigned* smax_bits, long n) {
    const float cn2 = c->cn2, ci2 = c->ci2;
    float m = 0.0f;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const float r = rho[q];
        const float vx = mx[q] / r, vy = my[q] / r, vz = mz[q] / r;
        const float cc = sqrtf(cn2 + xi[q] * (ci2 - cn2));
        const float v = fabsf(vx) + fabsf(vy) + fabsf(vz) + cc;
        m = fmaxr(v, m);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxr(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = fmaxr(b, red[w]);
        atomicMax(smax_bits, __float_as_uint(b));
    }
}

__global__ void zero_u32(unsigned* p) { *p = 0u; }

// Deterministic FP64 totals: every block sums a fixed contiguous range in a fixed order.
constexpr int RED_BLOCKS = 608;     // 4 x 152 SMs
constexpr int RED_THREADS = 256;

__global__ void reduce_partials(const float* __restrict__ rho, const float* __restrict__ mx,
                                const float* __restrict__ my, const float* __restrict__ mz, long n,
                                double* __restrict__ part) {
    const long per = (n + gridDim.x - 1) / gridDim.x;
    const long lo = blockIdx.x * per, hi = min(n, lo + per);
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (long q = lo + threadIdx.x; q < hi; q += blockDim.x) {
        s0 += (double)rho[q];
        s1 += (double)mx[q];
        s2 += (double)my[q];
        s3 += (double)mz[q];
    }
    __shared__ double red[4][RED_THREADS];
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    red[2][threadIdx.x] = s2;
    red[3][threadIdx.x] = s3;
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int f = 0; f < 4; ++f) red[f][threadIdx.x] += red[f][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 4) part[blockIdx.x * 4 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void reduce_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += part[b * 4 + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

}  // namespace

cudaError_t nb_launch_ctrl(const NbConst* c, NbState* st, const NbStarDev* stars, NbStarW* sw, int nstars,
                           int advance, cudaStream_t s) {
    ctrl_kernel<<<1, 128, 0, s>>>(c, st, stars, sw, nstars, advance);
    return cudaGetLastError();
}

cudaError_t nb_launch_weights(const NbConst* c, const NbState* st, const NbStarDev* stars, NbStarW* sw,
                              int nstars, cudaStream_t s) {
    ctrl_kernel<<<1, 128, 0, s>>>(c, const_cast<NbState*>(st), stars, sw, nstars, 0);
    return cudaGetLastError();
}

cudaError_t nb_launch_max_speed(const NbConst* c, const float* rho, const float* mx, const float* my,
                                const float* mz, const float* xi, unsigned* smax_bits, long n, cudaStream_t s) {
    zero_u32<<<1, 1, 0, s>>>(smax_bits);
    max_speed_kernel<<<1216, 256, 0, s>>>(c, rho, mx, my, mz, xi, smax_bits, n);
    return cudaGetLastError();
}

cudaError_t nb_launch_ctrl_batch(const NbBatchInst* insts, int n, int advance, unsigned* counters, cudaStream_t s) {
    if (n > 0) ctrl_batch_kernel<<<n, 128, 0, s>>>(insts, n, advance, counters);
    return cudaGetLastError();
}

int nb_reduce_scratch_doubles() { return RED_BLOCKS * 4 + 4; }

cudaError_t nb_launch_reduce_fp64(const float* rho, const float* mx, const float* my, const float* mz, long n,
                                  double* scratch, cudaStream_t s) {
    reduce_partials<<<RED_BLOCKS, RED_THREADS, 0, s>>>(rho, mx, my, mz, n, scratch);
    reduce_final<<<1, 32, 0, s>>>(scratch, RED_BLOCKS, scratch + RED_BLOCKS * 4);
    return cudaGetLastError();
}

// ============================================================================ allocation-free totals
// nb_reduce_fp64_static: the FP64 conservation totals for callers that cannot allocate device
// memory (a process whose allocations all come from a pre-sized pool or arena owned by someone
// else, or code that must not call cudaMalloc while other work is being captured into a CUDA
// graph).  The per-block partial sums live in this file-scope device array instead of handle
// scratch, so the caller passes only the input planes and a device output.
#define NB_STATIC_RED_CELLS_PER_BLOCK (1LL << 16)          // cells summed by one block
#define NB_STATIC_RED_MAX_BLOCKS (1 << 14)                  // 16384 blocks -> n <= 2^30 cells
static __device__ __align__(256) double g_static_red[NB_STATIC_RED_MAX_BLOCKS * 4 + 4];   // 512 KiB + 32 B

namespace {

#define NB_MAX_DEVICES 64
// The device address of g_static_red per device, with the ID of the context it was looked up in:
// an address belongs to one context (a cudaDeviceReset destroys it), so a call made in another
// context (a different one current on this thread, or the device's primary context re-created
// after a reset) looks it up again.
struct StaticSlot {
    unsigned long long ctx_id;
    double* ptr;
};
std::mutex g_static_mu;
StaticSlot g_static_slot[NB_MAX_DEVICES];

thread_local std::string g_static_err;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// The process-unique ID of the context current on this thread (cuCtxGetId, through the runtime's
// driver entry points); 0 when no context is current or the driver cannot tell, which makes the
// caller look the address up again.
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) const char* nb_static_last_error(void) {
    return g_static_err.c_str();
}

extern "C" __attribute__((visibility("default"))) int nb_reduce_fp64_static(const float* rho, const float* mx,
                                                                         const float* my, const float* mz,
                                                                         long long n, double* out4, void* stream) {
    if (!rho || !mx || !my || !mz || !out4) {
        g_static_err = "nb_reduce_fp64_static: null pointer";
        return NB_ERR_ARG;
    }
    if (n < 1 || n > (long long)NB_STATIC_RED_MAX_BLOCKS * NB_STATIC_RED_CELLS_PER_BLOCK) {
        g_static_err = "nb_reduce_fp64_static: n must be in [1, 2^30] cells (the static scratch holds 16384 "
                       "block partials of 65536 cells each)";
        return NB_ERR_LIMIT;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        g_static_err = std::string("nb_reduce_fp64_static: cudaGetDevice: ") + cudaGetErrorString(e);
        return NB_ERR_CUDA;
    }
    if (dev < 0 || dev >= NB_MAX_DEVICES) {
        g_static_err = "nb_reduce_fp64_static: device index " + std::to_string(dev) + " beyond the " +
                       std::to_string(NB_MAX_DEVICES) + " devices this entry point keeps an address for";
        return NB_ERR_LIMIT;
    }
    // an error left by an earlier call on this thread is the caller's, not this call's: report it
    // without clearing it, before any work is enqueued
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        g_static_err = std::string("nb_reduce_fp64_static: an earlier CUDA call left an error pending: ") +
                       cudaGetErrorString(e);
        return NB_ERR_CUDA;
    }
    double* part = nullptr;
    {
        // set-up, once per device and context, with that device current: the device address of the
        // array (the lookup itself makes the device's primary context current if none was)
        std::lock_guard<std::mutex> lock(g_static_mu);
        StaticSlot& slot = g_static_slot[dev];
        const unsigned long long id = current_ctx_id();
        if (!slot.ptr || id == 0 || slot.ctx_id != id) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_static_red);
            if (e != cudaSuccess || !p) {
                slot.ptr = nullptr;
                g_static_err = std::string("nb_reduce_fp64_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
                return NB_ERR_CUDA;
            }
            slot.ptr = static_cast<double*>(p);
            slot.ctx_id = current_ctx_id();
        }
        part = slot.ptr;
    }
    const int blocks = (int)((n + NB_STATIC_RED_CELLS_PER_BLOCK - 1) / NB_STATIC_RED_CELLS_PER_BLOCK);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // every partial the final pass reads is written by this call's first pass: nothing to clear
    reduce_partials<<<blocks, RED_THREADS, 0, s>>>(rho, mx, my, mz, n, part);
    reduce_final<<<1, 32, 0, s>>>(part, blocks, out4);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_static_err = std::string("nb_reduce_fp64_static: launch: ") + cudaGetErrorString(e);
        return NB_ERR_CUDA;
    }
    return NB_OK;
}
