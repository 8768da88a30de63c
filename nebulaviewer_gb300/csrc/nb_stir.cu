// Turbulent stirring and the end of the stirring phase.
//
//  * drive (nebula3d.py:165-179, launched by sim.py:1030-1042 _stir): every cell adds
//    rho * amp * dt * ((1 - blend) F_A + blend F_B) to its momenta, F_A / F_B trilinear samples
//    (nebula3d.py:195-226 sample_n) of two solenoidal fields on a coarse grid of spacing dxs.
//    The blend, the amplitude, dt and which ring slots hold A and B come from the control block
//    the step's control kernel wrote, so a stirred step needs no host round trip.  The CFL max
//    speed of the stirred state (nebula3d.py:154-162, what the next step's _compute_dt reads) is
//    folded into the same pass: stage 2 then skips its own.
//    The trilinear sample interpolates along x, then y, then z (sample_n's order).  Along one
//    (i, j) row of cells the x and y weights and corner indices are the same for every cell, so
//    the x-then-y interpolated value at each coarse z level is a property of the row: a warp
//    (one row) evaluates it once per level and field into shared memory, and each cell then
//    does only the z interpolation between its two levels -- the same float operations on the
//    same operands as the direct form, so the same bits, with 12 shared loads per cell instead
//    of 48 gathers.
//  * add_torus (sim.py:352-363): the dense torus joins the turbulent envelope at the start of
//    the main phase (sim.py:806-812).
//  * mach_sums (sim.py:501-508): sum |m|^2 / rho and sum rho, here in FP64 with a fixed
//    summation order (the reference sums in FP32 atomics, whose order is unspecified).
#include "nb_rayutil.cuh"

namespace {

// Trilinear weights of one coordinate of nebula3d.py:195-226 sample_n on an n-cell axis:
// g = p / d - 1/2, clamped corner indices, fraction; `out` when g lies outside [-1/2, n - 1/2].
struct Axis {
    int a, b;
    float f;
    bool out;
    __device__ __forceinline__ Axis(float p, float d, int n) {
        const float g = p / d - 0.5f;
        out = g < -0.5f || g > (float)n - 0.5f;
        const int i0 = out ? 0 : (int)floorf(g);
        f = g - (float)i0;
        a = iclampd(i0, 0, n - 1);
        b = iclampd(i0 + 1, 0, n - 1);
    }
};

// sample_n's interpolation order: along x, then y, then z
__device__ __forceinline__ float trilerp(const float* __restrict__ g, int sy, int sz, const Axis& X, const Axis& Y,
                                         const Axis& Z) {
    const float* pa = g + (long long)X.a * sy * sz;
    const float* pb = g + (long long)X.b * sy * sz;
    const int ya = Y.a * sz, yb = Y.b * sz;
    const float c000 = __ldg(pa + ya + Z.a), c100 = __ldg(pb + ya + Z.a);
    const float c010 = __ldg(pa + yb + Z.a), c110 = __ldg(pb + yb + Z.a);
    const float c001 = __ldg(pa + ya + Z.b), c101 = __ldg(pb + ya + Z.b);
    const float c011 = __ldg(pa + yb + Z.b), c111 = __ldg(pb + yb + Z.b);
    const float c00 = c000 + (c100 - c000) * X.f;
    const float c10 = c010 + (c110 - c010) * X.f;
    const float c01 = c001 + (c101 - c001) * X.f;
    const float c11 = c011 + (c111 - c011) * X.f;
    const float c0 = c00 + (c10 - c00) * Y.f;
    const float c1 = c01 + (c11 - c01) * Y.f;
    return c0 + (c1 - c0) * Z.f;
}

// x-then-y interpolated value of one coarse z level of one field (the c0 / c1 of sample_n)
__device__ __forceinline__ float xy_level(const float* __restrict__ g, int sy, int sz, const Axis& X, const Axis& Y,
                                          int kz) {
    const float* pa = g + (long long)X.a * sy * sz;
    const float* pb = g + (long long)X.b * sy * sz;
    const float c_a = __ldg(pa + Y.a * sz + kz), c_b = __ldg(pb + Y.a * sz + kz);
    const float d_a = __ldg(pa + Y.b * sz + kz), d_b = __ldg(pb + Y.b * sz + kz);
    const float cx = c_a + (c_b - c_a) * X.f;
    const float dxv = d_a + (d_b - d_a) * X.f;
    return cx + (dxv - cx) * Y.f;
}

__device__ __forceinline__ void block_max_to(float m, unsigned* dst) {
    for (int o = 16; o > 0; o >>= 1) m = fmaxr(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float red[32];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    if ((t & 31) == 0) red[t >> 5] = m;
    __syncthreads();
    if (t == 0) {
        float b = 0.0f;
        const int nw = (blockDim.x * blockDim.y + 31) >> 5;
        for (int w = 0; w < nw; ++w) b = fmaxr(b, red[w]);
        atomicMax(dst, __float_as_uint(b));
    }
}

// One warp per row (i, j), cells k = lane + 32 m (RowWalk).  With `explicit_args` the
// blend / amp / dt / fields come from the arguments (the single-kernel parity entry point).
// STAGED: the per-row x-y levels in shared memory (6 fields x sz floats per warp); otherwise
// every cell gathers its 48 corners (forcing grids too tall for shared memory).
template <bool STAGED>
__global__ void __launch_bounds__(256) drive_kernel(const NbConst* __restrict__ c, const NbState* __restrict__ st,
                                                    const float* __restrict__ rho, float* __restrict__ mx,
                                                    float* __restrict__ my, float* __restrict__ mz,
                                                    const float* __restrict__ xi, unsigned* smax_bits,
                                                    const float* __restrict__ fa_arg,
                                                    const float* __restrict__ fb_arg, float blend_arg,
                                                    float amp_arg, float dt_arg, int explicit_args) {
    extern __shared__ float levels[];                       // [warp][6][sz] when STAGED
    const NbConst& C = *c;
    const RowWalk w(C.nx, C.ny, C.nz);
    float vm = 0.0f;
    if (w.valid) {
        const int sx = C.drive_sx, sy = C.drive_sy, sz = C.drive_sz;
        const long long S = (long long)sx * sy * sz;
        bool go;
        float blend, amp, dt;
        const float *fa, *fb;
        if (explicit_args) {
            go = true;
            blend = blend_arg; amp = amp_arg; dt = dt_arg;
            fa = fa_arg; fb = fb_arg;
        } else {
            go = st->drive_go != 0;
            blend = st->blend_f; amp = st->amp_f; dt = st->dt_f;
            fa = C.drive_ring + (long long)st->drive_a * 3 * S;
            fb = C.drive_ring + (long long)st->drive_b * 3 * S;
        }
        const float dx = C.dx, dxs = C.drive_dxs_f, cn2 = C.cn2, ci2 = C.ci2;
        const float wa = 1.0f - blend;
        const Axis X(((float)w.i + 0.5f) * dx, dxs, sx);
        const Axis Y(((float)w.j + 0.5f) * dx, dxs, sy);
        float* lv = levels + threadIdx.y * 6 * sz;
        if (STAGED && go && !(X.out || Y.out)) {
            for (int t = threadIdx.x; t < 6 * sz; t += 32) {
                const int f = t / sz, kz = t - f * sz;
                const float* g = (f < 3 ? fa : fb) + (long long)(f < 3 ? f : f - 3) * S;
                lv[t] = xy_level(g, sy, sz, X, Y, kz);
            }
        }
        if (STAGED) __syncwarp();
#pragma unroll 4
        for (int k = w.k0; k < C.nz; k += 32) {     // unrolled: four cells' loads in flight per lane
            const long long q = w.base + k;
            const float r = rho[q];
            float m0 = mx[q], m1 = my[q], m2 = mz[q];
            if (go) {
                const Axis Z(((float)k + 0.5f) * dx, dxs, sz);
                float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, b0 = 0.0f, b1 = 0.0f, b2 = 0.0f;
                if (!(X.out || Y.out || Z.out)) {
                    if (STAGED) {
                        auto zl = [&](int f) {
                            const float c0 = lv[f * sz + Z.a], c1 = lv[f * sz + Z.b];
                            return c0 + (c1 - c0) * Z.f;
                        };
                        a0 = zl(0); a1 = zl(1); a2 = zl(2);
                        b0 = zl(3); b1 = zl(4); b2 = zl(5);
                    } else {
                        a0 = trilerp(fa, sy, sz, X, Y, Z);
                        a1 = trilerp(fa + S, sy, sz, X, Y, Z);
                        a2 = trilerp(fa + 2 * S, sy, sz, X, Y, Z);
                        b0 = trilerp(fb, sy, sz, X, Y, Z);
                        b1 = trilerp(fb + S, sy, sz, X, Y, Z);
                        b2 = trilerp(fb + 2 * S, sy, sz, X, Y, Z);
                    }
                }
                const float f0 = wa * a0 + blend * b0, f1 = wa * a1 + blend * b1, f2 = wa * a2 + blend * b2;
                const float s = r * amp * dt;
                m0 = m0 + s * f0;
                m1 = m1 + s * f1;
                m2 = m2 + s * f2;
                mx[q] = m0;
                my[q] = m1;
                mz[q] = m2;
            }
            if (smax_bits) {                     // nebula3d.py:158-162 on the stirred state
                const float cc = sqrtf(cn2 + xi[q] * (ci2 - cn2));
#if NB_ARITH_FAST
                const float ri = 1.0f / r;           // one division for the three velocities
                const float v = fabsf(m0 * ri) + fabsf(m1 * ri) + fabsf(m2 * ri) + cc;
#else
                const float v = fabsf(m0 / r) + fabsf(m1 / r) + fabsf(m2 / r) + cc;
#endif
                vm = fmaxr(v, vm);
            }
        }
    }
    if (smax_bits) block_max_to(vm, smax_bits);
}

__global__ void __launch_bounds__(256) add_torus_kernel(const float* __restrict__ torus, float* __restrict__ rho,
                                                        float* __restrict__ mx, float* __restrict__ my,
                                                        float* __restrict__ mz, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const float r = rho[q];
        const float tq = torus[q];
        const float f = 1.0f - tq / (tq + r);
        rho[q] = r + tq;
        mx[q] = mx[q] * f;
        my[q] = my[q] * f;
        mz[q] = mz[q] * f;
    }
}

constexpr int MACH_BLOCKS = 608;      // 4 x 152 SMs; fixed, so the FP64 sums are reproducible
constexpr int MACH_THREADS = 256;

__global__ void __launch_bounds__(MACH_THREADS) mach_partials(const float* __restrict__ rho,
                                                              const float* __restrict__ mx,
                                                              const float* __restrict__ my,
                                                              const float* __restrict__ mz, long long n,
                                                              double* __restrict__ part) {
    const long long per = (n + gridDim.x - 1) / gridDim.x;
    const long long lo = blockIdx.x * per, hi = min(n, lo + per);
    double s0 = 0.0, s1 = 0.0;
    for (long long q = lo + threadIdx.x; q < hi; q += blockDim.x) {
        const float r = rho[q];
        const float m2 = mx[q] * mx[q] + my[q] * my[q] + mz[q] * mz[q];
        s0 += (double)(m2 / r);
        s1 += (double)r;
    }
    __shared__ double red[2][MACH_THREADS];
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    __syncthreads();
    for (int w = MACH_THREADS / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < 2) part[blockIdx.x * 2 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void mach_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
    if (threadIdx.x < 2) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += part[b * 2 + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

int grid_n(long long n) {
    const long long b = (n + 255) / 256;
    return (int)(b < 152LL * 16 ? (b < 1 ? 1 : b) : 152LL * 16);
}

}  // namespace

namespace {
constexpr int DRIVE_STAGED_MAX_SZ = 1024;           // 8 warps x 6 x 1024 floats = 192 KiB of shared memory

cudaError_t launch_drive(const NbConst* c, const NbState* st, const float* rho, float* mx, float* my, float* mz,
                         const float* xi, unsigned* smax_bits, const float* fa, const float* fb, float blend, float amp,
                         float dt, int explicit_args, int nx, int ny, int sz, cudaStream_t s) {
    const dim3 grid(rowwalk_blocks(nx, ny)), block(32, 8);
    if (sz <= DRIVE_STAGED_MAX_SZ) {
        const int smem = 8 * 6 * sz * (int)sizeof(float);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(drive_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        drive_kernel<true><<<grid, block, smem, s>>>(c, st, rho, mx, my, mz, xi, smax_bits, fa, fb, blend, amp, dt,
                                                     explicit_args);
    } else {
        drive_kernel<false><<<grid, block, 0, s>>>(c, st, rho, mx, my, mz, xi, smax_bits, fa, fb, blend, amp, dt,
                                                   explicit_args);
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t nb_launch_drive(const NbConst* c, const NbState* st, const float* rho, float* mx, float* my, float* mz,
                            const float* xi, unsigned* smax_bits, int nx, int ny, int sz, cudaStream_t s) {
    if (smax_bits) cudaMemsetAsync(smax_bits, 0, sizeof(unsigned), s);
    return launch_drive(c, st, rho, mx, my, mz, xi, smax_bits, nullptr, nullptr, 0.f, 0.f, 0.f, 0, nx, ny, sz, s);
}

cudaError_t nb_launch_drive_explicit(const NbConst* c, const float* rho, float* mx, float* my, float* mz,
                                     const float* fa, const float* fb, float blend, float amp, float dt, int nx,
                                     int ny, int sz, cudaStream_t s) {
    return launch_drive(c, nullptr, rho, mx, my, mz, nullptr, nullptr, fa, fb, blend, amp, dt, 1, nx, ny, sz, s);
}

cudaError_t nb_launch_add_torus(const float* torus, float* rho, float* mx, float* my, float* mz, long long n,
                                cudaStream_t s) {
    add_torus_kernel<<<grid_n(n), 256, 0, s>>>(torus, rho, mx, my, mz, n);
    return cudaGetLastError();
}

int nb_mach_scratch_doubles() { return MACH_BLOCKS * 2 + 2; }

cudaError_t nb_launch_mach_sums(const float* rho, const float* mx, const float* my, const float* mz, long long n,
                                double* scratch, cudaStream_t s) {
    mach_partials<<<MACH_BLOCKS, MACH_THREADS, 0, s>>>(rho, mx, my, mz, n, scratch);
    mach_final<<<1, 32, 0, s>>>(scratch, MACH_BLOCKS, scratch + MACH_BLOCKS * 2);
    return cudaGetLastError();
}
