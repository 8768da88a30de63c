// CPU oracle: a line-by-line restatement of the reference's simulation-step kernels.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls this file;
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it to check results.
//
// Each function follows one NVIDIA-Warp kernel of the reference (file:line cited) with
// the same operation order, evaluated op by op (built with -ffp-contract=off, no
// fast-math).  Warp's builtin semantics are restated as:
//   vec / s  -> component-wise division;  dot(a,b) = 0 + a0*b0 + a1*b1 + ... ;
//   length   = sqrt(dot(a,a));  max(a,b) = a > b ? a : b;  min(a,b) = a < b ? a : b;
//   clamp(x,lo,hi) = min(max(lo,x),hi);  int(x) truncates toward zero.
// Every routine is a template over the real type T: T=float is the FP32 oracle that the
// CUDA path is checked against; T=double is the FP64 re-run of the same scheme used to
// state each FP32 result's error.  Arrays are C-order [i][j][k] (k fastest), the
// reference's (nx, ny, nz) layout, one plane per field (rho, mx, my, mz).
//
// Pinned against the golden fixtures of tests/golden/ (the reference's own kernel source
// run under a float32 restatement of the Warp builtins): the hydro kernels agree bit for
// bit; ray/FUV results agree to float32 rounding of the transcendental functions.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T> inline T tmax(T a, T b) { return a > b ? a : b; }
template <class T> inline T tmin(T a, T b) { return a < b ? a : b; }
inline int imax(int a, int b) { return a > b ? a : b; }
inline int imin(int a, int b) { return a < b ? a : b; }
inline int iclamp(int x, int lo, int hi) { return imin(imax(lo, x), hi); }
template <class T> inline T tclamp(T x, T lo, T hi) { return tmin(tmax(lo, x), hi); }

template <class T> struct V4 { T c[4]; };
template <class T> struct V3 { T c[3]; };

template <class T> inline T pi_t() { return T(3.14159265358979323846); }

struct Grid {
    int nx, ny, nz;
    inline long idx(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }
    inline long idxc(int i, int j, int k) const {            // clamped (outflow) index: nebula3d.py:23-25 ldc
        return idx(iclamp(i, 0, nx - 1), iclamp(j, 0, ny - 1), iclamp(k, 0, nz - 1));
    }
};

// nebula3d.py:28-32 prim
template <class T>
inline V4<T> prim(const Grid& g, const T* rho, const T* mx, const T* my, const T* mz, int i, int j, int k, T floor_) {
    long q = g.idxc(i, j, k);
    T r = tmax(rho[q], floor_);
    return V4<T>{{r, mx[q] / r, my[q] / r, mz[q] / r}};
}

// nebula3d.py:35-37 csq
template <class T>
inline T csq(const Grid& g, const T* xi, int i, int j, int k, T cn2, T ci2) {
    return cn2 + xi[g.idxc(i, j, k)] * (ci2 - cn2);
}

// nebula3d.py:40-46 minmod; sim.py:366-380 mc_lim / vl_lim; sim.py:383-389 slope
template <class T> inline T minmod(T a, T b) {
    if (a * b <= T(0)) return T(0);
    if (std::fabs(a) < std::fabs(b)) return a;
    return b;
}
template <class T> inline T mc_lim(T a, T b) {
    if (a * b <= T(0)) return T(0);
    T s = a > T(0) ? T(1) : T(-1);
    return s * tmin(tmin(T(2) * std::fabs(a), T(2) * std::fabs(b)), T(0.5) * std::fabs(a + b));
}
template <class T> inline T vl_lim(T a, T b) {
    if (a * b <= T(0)) return T(0);
    return T(2) * a * b / (a + b);
}
template <class T> inline T slope(T a, T b, int lim) {
    if (lim == 2) return mc_lim(a, b);
    if (lim == 1) return vl_lim(a, b);
    return minmod(a, b);
}

template <class T> inline T dot4(const V4<T>& a, const V4<T>& b) {
    T r = T(0);
    for (int c = 0; c < 4; ++c) r = r + a.c[c] * b.c[c];
    return r;
}
template <class T> inline T dot3(const V3<T>& a, const V3<T>& b) {
    T r = T(0);
    for (int c = 0; c < 3; ++c) r = r + a.c[c] * b.c[c];
    return r;
}
template <class T> inline T len3(const V3<T>& a) { return std::sqrt(dot3(a, a)); }

// nebula3d.py:54-72 face_flux (Rusanov, minmod) when hll == false;
// sim.py:397-420 flux_hll (HLL, Davis speeds, limiter lim) when hll == true.
template <class T>
inline V4<T> face_flux(const V4<T>& qa, const V4<T>& qb, const V4<T>& qc, const V4<T>& qd, T c2b, T c2c,
                       const V4<T>& e, T floor_, bool hll, int lim) {
    V4<T> L, R;
    for (int c = 0; c < 4; ++c) {
        T sl = hll ? slope(qb.c[c] - qa.c[c], qc.c[c] - qb.c[c], lim) : minmod(qb.c[c] - qa.c[c], qc.c[c] - qb.c[c]);
        T sr = hll ? slope(qc.c[c] - qb.c[c], qd.c[c] - qc.c[c], lim) : minmod(qc.c[c] - qb.c[c], qd.c[c] - qc.c[c]);
        L.c[c] = qb.c[c] + T(0.5) * sl;
        R.c[c] = qc.c[c] - T(0.5) * sr;
    }
    T rL = tmax(L.c[0], floor_);
    T rR = tmax(R.c[0], floor_);
    V4<T> vL{{T(0), L.c[1], L.c[2], L.c[3]}};
    V4<T> vR{{T(0), R.c[1], R.c[2], R.c[3]}};
    T unL = dot4(vL, e);
    T unR = dot4(vR, e);
    V4<T> UL{{rL, rL * L.c[1], rL * L.c[2], rL * L.c[3]}};
    V4<T> UR{{rR, rR * R.c[1], rR * R.c[2], rR * R.c[3]}};
    V4<T> FL, FR, F;
    T pL = rL * c2b, pR = rR * c2c;
    for (int c = 0; c < 4; ++c) {
        FL.c[c] = UL.c[c] * unL + e.c[c] * pL;
        FR.c[c] = UR.c[c] * unR + e.c[c] * pR;
    }
    if (!hll) {
        T amax = tmax(std::fabs(unL) + std::sqrt(c2b), std::fabs(unR) + std::sqrt(c2c));
        T ha = T(0.5) * amax;
        for (int c = 0; c < 4; ++c) F.c[c] = T(0.5) * (FL.c[c] + FR.c[c]) - ha * (UR.c[c] - UL.c[c]);
        return F;
    }
    T cb = std::sqrt(c2b), cc = std::sqrt(c2c);
    T SL = tmin(unL - cb, unR - cc);
    T SR = tmax(unL + cb, unR + cc);
    if (SL >= T(0)) return FL;
    if (SR <= T(0)) return FR;
    T slsr = SL * SR, den = SR - SL;
    for (int c = 0; c < 4; ++c) F.c[c] = (SR * FL.c[c] - SL * FR.c[c] + slsr * (UR.c[c] - UL.c[c])) / den;
    return F;
}

// nebula3d.py:195-226 sample_n: trilinear, 0 outside the domain
template <class T>
inline T sample_n(const Grid& g, const T* a, const V3<T>& p, T dx) {
    T gx = p.c[0] / dx - T(0.5), gy = p.c[1] / dx - T(0.5), gz = p.c[2] / dx - T(0.5);
    if (gx < T(-0.5) || gy < T(-0.5) || gz < T(-0.5)) return T(0);
    if (gx > T(g.nx) - T(0.5) || gy > T(g.ny) - T(0.5) || gz > T(g.nz) - T(0.5)) return T(0);
    int i0 = (int)std::floor(gx), j0 = (int)std::floor(gy), k0 = (int)std::floor(gz);
    T fx = gx - T(i0), fy = gy - T(j0), fz = gz - T(k0);
    T c000 = a[g.idxc(i0, j0, k0)], c100 = a[g.idxc(i0 + 1, j0, k0)];
    T c010 = a[g.idxc(i0, j0 + 1, k0)], c110 = a[g.idxc(i0 + 1, j0 + 1, k0)];
    T c001 = a[g.idxc(i0, j0, k0 + 1)], c101 = a[g.idxc(i0 + 1, j0, k0 + 1)];
    T c011 = a[g.idxc(i0, j0 + 1, k0 + 1)], c111 = a[g.idxc(i0 + 1, j0 + 1, k0 + 1)];
    T c00 = c000 + (c100 - c000) * fx;
    T c10 = c010 + (c110 - c010) * fx;
    T c01 = c001 + (c101 - c001) * fx;
    T c11 = c011 + (c111 - c011) * fx;
    T c0 = c00 + (c10 - c00) * fy;
    T c1 = c01 + (c11 - c01) * fy;
    return c0 + (c1 - c0) * fz;
}

// nebula3d.py:229-244 box_range
template <class T>
inline void box_range(const V3<T>& o, const V3<T>& d, const V3<T>& bmax, T& t0, T& t1) {
    t0 = T(0);
    t1 = T(1e9);
    for (int a = 0; a < 3; ++a) {
        T da = d.c[a];
        if (std::fabs(da) < T(1e-9)) {
            if (o.c[a] < T(0) || o.c[a] > bmax.c[a]) t1 = T(-1);
        } else {
            T ta = (T(0) - o.c[a]) / da;
            T tb = (bmax.c[a] - o.c[a]) / da;
            t0 = tmax(t0, tmin(ta, tb));
            t1 = tmin(t1, tmax(ta, tb));
        }
    }
}

// ray direction of nebula3d.py:253-256 (cast_rays) and 329-332 (cast_fuv)
template <class T>
inline V3<T> ray_dir(int iu, int ip, int nu, int nphi) {
    T u = T(-1) + (T(iu) + T(0.5)) * T(2) / T(nu);
    T s = std::sqrt(tmax(T(1) - u * u, T(0)));
    T phi = (T(ip) + T(0.5)) * T(2) * pi_t<T>() / T(nphi);
    return V3<T>{{s * std::cos(phi), s * std::sin(phi), u}};
}

// python int() of a float, guarded against values beyond the int range
template <class T> inline long trunc_l(T x) {
    if (x > T(2e9)) return 2000000000L;
    if (x < T(-2e9)) return -2000000000L;
    return (long)x;
}

template <class T>
inline void cell_dir(int i, int j, int k, T dx, const V3<T>& star, T& r, T& u, T& phi) {
    V3<T> p{{(T(i) + T(0.5)) * dx, (T(j) + T(0.5)) * dx, (T(k) + T(0.5)) * dx}};
    V3<T> rel{{p.c[0] - star.c[0], p.c[1] - star.c[1], p.c[2] - star.c[2]}};
    r = tmax(len3(rel), T(1e-6));
    u = rel.c[2] / r;
    phi = std::atan2(rel.c[1], rel.c[0]);
    if (phi < T(0)) phi = phi + T(2) * pi_t<T>();
}

}  // namespace

// ==================================================================================== kernels
template <class T>
static void hydro_stage_t(int nx, int ny, int nz, const T* rho, const T* mx, const T* my, const T* mz, const T* xi,
                          const T* r0, const T* mx0, const T* my0, const T* mz0,
                          T* o_r, T* o_mx, T* o_my, T* o_mz,
                          const T* stars, int nstars, T wind, const T* jets, T jet_cos, T jet_r, T pulse,
                          T dt, T dx, T a, T b, T floor_, T cn2, T ci2, T vmax, int solver, int lim) {
    // nebula3d.py:76-151 hydro_stage (solver 0) / sim.py:423-498 hydro_stage_hll (solver 1)
    Grid g{nx, ny, nz};
    const bool hll = solver == 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                V4<T> div{{T(0), T(0), T(0), T(0)}};
                for (int axis = 0; axis < 3; ++axis) {
                    int oi = axis == 0, oj = axis == 1, ok = axis == 2;
                    V4<T> e{{T(0), T(oi), T(oj), T(ok)}};
                    V4<T> qm2 = prim(g, rho, mx, my, mz, i - 2 * oi, j - 2 * oj, k - 2 * ok, floor_);
                    V4<T> qm1 = prim(g, rho, mx, my, mz, i - oi, j - oj, k - ok, floor_);
                    V4<T> q0 = prim(g, rho, mx, my, mz, i, j, k, floor_);
                    V4<T> qp1 = prim(g, rho, mx, my, mz, i + oi, j + oj, k + ok, floor_);
                    V4<T> qp2 = prim(g, rho, mx, my, mz, i + 2 * oi, j + 2 * oj, k + 2 * ok, floor_);
                    T cm1 = csq(g, xi, i - oi, j - oj, k - ok, cn2, ci2);
                    T c0 = csq(g, xi, i, j, k, cn2, ci2);
                    T cp1 = csq(g, xi, i + oi, j + oj, k + ok, cn2, ci2);
                    V4<T> fR = face_flux(qm1, q0, qp1, qp2, c0, cp1, e, floor_, hll, lim);
                    V4<T> fL = face_flux(qm2, qm1, q0, qp1, cm1, c0, e, floor_, hll, lim);
                    for (int c = 0; c < 4; ++c) div.c[c] = div.c[c] + (fR.c[c] - fL.c[c]);
                }
                long q = g.idx(i, j, k);
                V4<T> U{{rho[q], mx[q], my[q], mz[q]}};
                V4<T> dU;
                for (int c = 0; c < 4; ++c) dU.c[c] = -div.c[c] / dx;
                V3<T> p{{(T(i) + T(0.5)) * dx, (T(j) + T(0.5)) * dx, (T(k) + T(0.5)) * dx}};
                T x_ion = xi[q];
                if (wind > T(0) && x_ion > T(0.01)) {
                    V3<T> acc{{T(0), T(0), T(0)}};
                    for (int s = 0; s < nstars; ++s) {
                        const T* st = stars + 4 * s;
                        if (st[3] > T(0)) {
                            V3<T> rel{{p.c[0] - st[0], p.c[1] - st[1], p.c[2] - st[2]}};
                            T r2 = dot3(rel, rel) + T(0.0004);
                            T f = st[3] / (r2 * std::sqrt(r2));
                            for (int c = 0; c < 3; ++c) acc.c[c] = acc.c[c] + rel.c[c] * f;
                        }
                    }
                    T wx = wind * x_ion;
                    for (int c = 0; c < 3; ++c) acc.c[c] = acc.c[c] * wx;
                    dU.c[0] = dU.c[0] + T(0);
                    for (int c = 0; c < 3; ++c) dU.c[c + 1] = dU.c[c + 1] + U.c[0] * acc.c[c];
                }
                V3<T> accj{{T(0), T(0), T(0)}};
                for (int s = 0; s < nstars; ++s) {
                    const T* jt = jets + 4 * s;
                    const T* st = stars + 4 * s;
                    if (jt[3] > T(0) && st[3] > T(0)) {
                        V3<T> rel{{p.c[0] - st[0], p.c[1] - st[1], p.c[2] - st[2]}};
                        T r = len3(rel);
                        if (r < jet_r && r > T(1e-6)) {
                            V3<T> ax{{jt[0], jt[1], jt[2]}};
                            T c = dot3(rel, ax) / r;
                            if (std::fabs(c) > jet_cos) {
                                T f = (c > T(0) ? T(1) : T(-1)) * jt[3] * pulse / (r * r + T(0.0004));
                                for (int cc = 0; cc < 3; ++cc) accj.c[cc] = accj.c[cc] + ax.c[cc] * f;
                            }
                        }
                    }
                }
                dU.c[0] = dU.c[0] + T(0);
                for (int c = 0; c < 3; ++c) dU.c[c + 1] = dU.c[c + 1] + U.c[0] * accj.c[c];
                V4<T> Un, out;
                for (int c = 0; c < 4; ++c) Un.c[c] = U.c[c] + dt * dU.c[c];
                V4<T> U0{{r0[q], mx0[q], my0[q], mz0[q]}};
                for (int c = 0; c < 4; ++c) out.c[c] = a * U0.c[c] + b * Un.c[c];
                T r = tmax(out.c[0], floor_);
                V3<T> vel{{out.c[1] / r, out.c[2] / r, out.c[3] / r}};
                T sp = len3(vel);
                if (sp > vmax) {
                    T f = vmax / sp;
                    for (int c = 0; c < 3; ++c) vel.c[c] = vel.c[c] * f;
                }
                o_r[q] = r;
                o_mx[q] = r * vel.c[0];
                o_my[q] = r * vel.c[1];
                o_mz[q] = r * vel.c[2];
            }
}

template <class T>
static T max_speed_t(int nx, int ny, int nz, const T* rho, const T* mx, const T* my, const T* mz, const T* xi,
                     T cn2, T ci2) {
    // nebula3d.py:154-162 max_speed (atomic_max -> an exact max reduction)
    long n = (long)nx * ny * nz;
    T best = T(0);
#pragma omp parallel for reduction(max : best) schedule(static)
    for (long q = 0; q < n; ++q) {
        T r = rho[q];
        T vx = mx[q] / r, vy = my[q] / r, vz = mz[q] / r;
        T c = std::sqrt(cn2 + xi[q] * (ci2 - cn2));
        T v = std::fabs(vx) + std::fabs(vy) + std::fabs(vz) + c;
        if (v > best) best = v;
    }
    return best;
}

template <class T>
static void cast_rays_t(int nx, int ny, int nz, const T* rho, const T* star3, T Q, T dr, int nsteps, T dx, T rcap,
                        const T* bmax3, int nu, int nphi, T* rfront) {
    // nebula3d.py:247-270 cast_rays
    Grid g{nx, ny, nz};
    V3<T> star{{star3[0], star3[1], star3[2]}}, bmax{{bmax3[0], bmax3[1], bmax3[2]}};
#pragma omp parallel for schedule(dynamic, 4)
    for (int iu = 0; iu < nu; ++iu)
        for (int ip = 0; ip < nphi; ++ip) {
            V3<T> d = ray_dir<T>(iu, ip, nu, nphi);
            T col = T(0), rf = rcap, t0, t1;
            box_range(star, d, bmax, t0, t1);
            long n0 = trunc_l(t0 / dr);
            long n1 = std::min((long)nsteps, trunc_l(t1 / dr) + 2);
            for (long n = n0; n < n1; ++n) {
                T r = (T(n) + T(0.5)) * dr;
                V3<T> p{{star.c[0] + d.c[0] * r, star.c[1] + d.c[1] * r, star.c[2] + d.c[2] * r}};
                T nv = sample_n(g, rho, p, dx);
                T inc = nv * nv * r * r * dr;
                if (col + inc > Q) {
                    rf = r - T(0.5) * dr + dr * (Q - col) / tmax(inc, T(1e-20));
                    break;
                }
                col = col + inc;
            }
            rfront[(long)iu * nphi + ip] = rf;
        }
}

template <class T>
static void apply_front_t(int nx, int ny, int nz, const T* rfront, int nu, int nphi, const T* star3, T dx, T width,
                          T* xi, T* dfront) {
    // nebula3d.py:273-307 rf_at + apply_front
    Grid g{nx, ny, nz};
    V3<T> star{{star3[0], star3[1], star3[2]}};
    auto rf_at = [&](int iu, int ip) {
        int ipw = ((ip % nphi) + nphi) % nphi;
        return rfront[(long)iclamp(iu, 0, nu - 1) * nphi + ipw];
    };
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                T r, u, phi;
                cell_dir(i, j, k, dx, star, r, u, phi);
                T fu = (u + T(1)) * T(0.5) * T(nu) - T(0.5);
                T fp = phi / (T(2) * pi_t<T>()) * T(nphi) - T(0.5);
                int iu = (int)std::floor(fu), ip = (int)std::floor(fp);
                T tu = fu - T(iu), tp = fp - T(ip);
                T a = rf_at(iu, ip) * (T(1) - tp) + rf_at(iu, ip + 1) * tp;
                T b = rf_at(iu + 1, ip) * (T(1) - tp) + rf_at(iu + 1, ip + 1) * tp;
                T rf = a * (T(1) - tu) + b * tu;
                T val = tclamp((rf - r) / width + T(0.5), T(0), T(1));
                long q = g.idx(i, j, k);
                if (val > xi[q]) xi[q] = val;
                dfront[q] = tmin(dfront[q], r - rf);
            }
}

template <class T>
static void smooth_xi_t(int nx, int ny, int nz, const T* src, T* dst) {
    // nebula3d.py:310-315 smooth_xi
    Grid g{nx, ny, nz};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                T m = (src[g.idxc(i - 1, j, k)] + src[g.idxc(i + 1, j, k)] + src[g.idxc(i, j - 1, k)] +
                       src[g.idxc(i, j + 1, k)] + src[g.idxc(i, j, k - 1)] + src[g.idxc(i, j, k + 1)]) / T(6);
                long q = g.idx(i, j, k);
                dst[q] = T(0.5) * src[q] + T(0.5) * m;
            }
}

template <class T>
static void cast_fuv_t(int nx, int ny, int nz, const T* rho, const T* xi, const T* star3, T kappa, T dr, int nsteps,
                       T dx, T binr, const T* bmax3, int nr, int nu, int nphi, T* att) {
    // nebula3d.py:320-352 cast_fuv
    Grid g{nx, ny, nz};
    V3<T> star{{star3[0], star3[1], star3[2]}}, bmax{{bmax3[0], bmax3[1], bmax3[2]}};
#pragma omp parallel for schedule(dynamic, 4)
    for (int iu = 0; iu < nu; ++iu)
        for (int ip = 0; ip < nphi; ++ip) {
            V3<T> d = ray_dir<T>(iu, ip, nu, nphi);
            T tau = T(0), t0, t1;
            int ib = 0;
            box_range(star, d, bmax, t0, t1);
            long n0 = trunc_l(t0 / dr);
            long n1 = std::min((long)nsteps, trunc_l(t1 / dr) + 2);
            auto at = [&](int b) -> T& { return att[((long)b * nu + iu) * nphi + ip]; };
            for (long n = n0; n < n1; ++n) {
                T r = (T(n) + T(0.5)) * dr;
                V3<T> q{{star.c[0] + d.c[0] * r, star.c[1] + d.c[1] * r, star.c[2] + d.c[2] * r}};
                T n_tot = sample_n(g, rho, q, dx);
                T x_i = sample_n(g, xi, q, dx);
                tau = tau + kappa * n_tot * (T(1) - T(0.92) * x_i) * dr;
                int nb = (int)trunc_l(r / binr);
                if (nb > ib) {
                    T v = std::exp(-tau);
                    for (int b = ib; b < imin(nb, nr); ++b) at(b) = v;
                    ib = nb;
                }
                if (ib >= nr) break;
            }
            T v = std::exp(-tau);
            for (int b = ib; b < nr; ++b) at(b) = v;
        }
}

template <class T>
static void apply_fuv_t(int nx, int ny, int nz, const T* att, int nr, int nu, int nphi, const T* star3, T lum, T dx,
                        T binr, T* g0) {
    // nebula3d.py:355-388 apply_fuv
    Grid g{nx, ny, nz};
    V3<T> star{{star3[0], star3[1], star3[2]}};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                T r, u, phi;
                cell_dir(i, j, k, dx, star, r, u, phi);
                T fr = r / binr - T(0.5);
                T fu = (u + T(1)) * T(0.5) * T(nu) - T(0.5);
                T fp = phi / (T(2) * pi_t<T>()) * T(nphi) - T(0.5);
                int ir = (int)std::floor(fr), iu = (int)std::floor(fu), ip = (int)std::floor(fp);
                T tr = fr - T(ir), tu = fu - T(iu), tp = fp - T(ip);
                T acc = T(0);
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b)
                        for (int c = 0; c < 2; ++c) {
                            T w = (a == 0 ? T(1) - tr : tr) * (b == 0 ? T(1) - tu : tu) * (c == 0 ? T(1) - tp : tp);
                            int rr = iclamp(ir + a, 0, nr - 1);
                            int uu = iclamp(iu + b, 0, nu - 1);
                            int pp = (((ip + c) % nphi) + nphi) % nphi;
                            acc = acc + w * att[((long)rr * nu + uu) * nphi + pp];
                        }
                T r2 = tmax(r * r, T(0.0004));
                long q = g.idx(i, j, k);
                g0[q] = g0[q] + lum * acc / r2;
            }
}

// Plane-parallel source on the -x face (no reference counterpart; the CUDA path defines it the
// same way): per (j,k) column the column sum n^2 dx along +x, the front interpolated in the
// crossing cell as in nebula3d.py:262-268, rcap when the flux is never used up.
template <class T>
static void plane_front_t(int nx, int ny, int nz, const T* rho, T F, T dx, T rcap, T* xf) {
    const long long plane = (long long)ny * nz;
#pragma omp parallel for schedule(static)
    for (long long col = 0; col < plane; ++col) {
        T sum = T(0), x = rcap;
        for (int i = 0; i < nx; ++i) {
            const T n = rho[i * plane + col];
            const T inc = n * n * dx;
            if (sum + inc > F) {
                x = (T(i) + T(0.5)) * dx - T(0.5) * dx + dx * (F - sum) / tmax(inc, T(1e-20));
                break;
            }
            sum = sum + inc;
        }
        xf[col] = x;
    }
}

// merge of the plane front into xi / dfront with nebula3d.py:303-307's rules
template <class T>
static void apply_plane_t(int nx, int ny, int nz, const T* xf, T dx, T width, T* xi, T* dfront) {
    Grid g{nx, ny, nz};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const T px = (T(i) + T(0.5)) * dx;
                const T x = xf[(long long)j * nz + k];
                const T val = tclamp((x - px) / width + T(0.5), T(0), T(1));
                const long long q = g.idx(i, j, k);
                if (val > xi[q]) xi[q] = val;
                dfront[q] = tmin(dfront[q], px - x);
            }
}

// FUV of the plane source: tau of nebula3d.py:343 summed along +x to each cell centre
template <class T>
static void plane_fuv_t(int nx, int ny, int nz, const T* rho, const T* xi, T kappa, T lum, T dx, T* g) {
    const long long plane = (long long)ny * nz;
#pragma omp parallel for schedule(static)
    for (long long col = 0; col < plane; ++col) {
        T tau = T(0);
        for (int i = 0; i < nx; ++i) {
            const long long q = i * plane + col;
            const T dtau = kappa * rho[q] * (T(1) - T(0.92) * xi[q]) * dx;
            g[q] = lum * std::exp(-(tau + T(0.5) * dtau));
            tau = tau + dtau;
        }
    }
}

// float -> IEEE binary16 bits, round to nearest even (the conversion of sim.py:511-514 to_half)
static inline uint16_t f32_to_f16_rne(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);           // rounds to >= 65520 -> inf
    if (ax < 0x38800000u) {                                              // below 2^-14: subnormal half or 0
        if (ax < 0x33000000u) return (uint16_t)sign;                     // < 2^-25 rounds to 0
        uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        int e = (int)(ax >> 23);                                         // 102..112
        int shift = 126 - e;                                             // 14..24
        uint32_t q = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (q & 1u))) ++q;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (ax >> 23) - 112u;
    uint32_t m = ax & 0x7fffffu;
    uint32_t q = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) ++q;
    return (uint16_t)(sign | q);
}

// nebula3d.py:165-179 drive: m += rho * amp * dt * ((1 - blend) F_A + blend F_B), the forcing
// sampled (sample_n) on the coarse grid gs of spacing dxs at the cell centre (i + 1/2) dx
template <class T>
static void drive_t(int nx, int ny, int nz, const T* rho, T* mx, T* my, T* mz, int sx, int sy, int sz, const T* fa,
                    const T* fb, T blend, T amp, T dt, T dx, T dxs) {
    const Grid gs{sx, sy, sz};
    const long S = (long)sx * sy * sz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const V3<T> p{{(T(i) + T(0.5)) * dx, (T(j) + T(0.5)) * dx, (T(k) + T(0.5)) * dx}};
                T f[3];
                for (int c = 0; c < 3; ++c) {
                    const T a = sample_n(gs, fa + c * S, p, dxs);
                    const T b = sample_n(gs, fb + c * S, p, dxs);
                    f[c] = (T(1) - blend) * a + blend * b;
                }
                const long q = ((long)i * ny + j) * nz + k;
                const T r = rho[q] * amp * dt;
                mx[q] = mx[q] + r * f[0];
                my[q] = my[q] + r * f[1];
                mz[q] = mz[q] + r * f[2];
            }
}

// sim.py:352-363 add_torus
template <class T>
static void add_torus_t(long n, const T* torus, T* rho, T* mx, T* my, T* mz) {
#pragma omp parallel for schedule(static)
    for (long q = 0; q < n; ++q) {
        const T r = rho[q], tq = torus[q];
        const T f = T(1) - tq / (tq + r);
        rho[q] = r + tq;
        mx[q] = mx[q] * f;
        my[q] = my[q] * f;
        mz[q] = mz[q] * f;
    }
}

// float16 bits -> float (exact)
static inline float f16_to_f32(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    float v;
    if (e == 0) {
        v = std::ldexp((float)m, -24);                                   // zero / subnormal
    } else if (e == 31) {
        v = m ? std::numeric_limits<float>::quiet_NaN() : std::numeric_limits<float>::infinity();
    } else {
        v = std::ldexp((float)(m | 0x400u), (int)e - 25);
    }
    uint32_t b;
    std::memcpy(&b, &v, 4);
    b |= sign;
    std::memcpy(&v, &b, 4);
    return v;
}

// nebula3d.py:182-191 shock_field at one cell (render.py:165-174 shock_at): max(0, -div v) rho,
// central differences on clamped neighbours
static inline float shock_at_f(const Grid& g, const float* rho, const float* mx, const float* my, const float* mz,
                               int i, int j, int k, float dx) {
    const float du = mx[g.idxc(i + 1, j, k)] / rho[g.idxc(i + 1, j, k)] - mx[g.idxc(i - 1, j, k)] / rho[g.idxc(i - 1, j, k)];
    const float dv = my[g.idxc(i, j + 1, k)] / rho[g.idxc(i, j + 1, k)] - my[g.idxc(i, j - 1, k)] / rho[g.idxc(i, j - 1, k)];
    const float dw = mz[g.idxc(i, j, k + 1)] / rho[g.idxc(i, j, k + 1)] - mz[g.idxc(i, j, k - 1)] / rho[g.idxc(i, j, k - 1)];
    const float div = (du + dv + dw) / (2.0f * dx);
    return tmax(-div, 0.0f) * rho[g.idx(i, j, k)];
}

// render.py:127-131 sstep, 135-139 fade_axis
static inline float sstep_f(float e0, float e1, float x) {
    const float t = tclamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
static inline float fade_f(float u, float e) { return e <= 0.0f ? 1.0f : sstep_f(0.0f, e, u) * sstep_f(0.0f, e, 1.0f - u); }

// render.py:176-205 pack_volume_lm: one RGBA16F voxel (emission rgb, dust) per cell.
// pp: c_ha[3] c_o3[3] c_s2[3] c_dg[3] c_sh[3] gs ambient edge inv_L[3] dx (render.py:77-88 PackParams)
static void render_pack_f(int nx, int ny, int nz, const float* rho, const float* mx, const float* my, const float* mz,
                          const float* xi, const uint16_t* df16, const uint16_t* g016, const float* pp, int shock_on,
                          uint16_t* out) {
    const Grid g{nx, ny, nz};
    const float *c_ha = pp, *c_o3 = pp + 3, *c_s2 = pp + 6, *c_dg = pp + 9, *c_sh = pp + 12;
    const float gs = pp[15], ambient = pp[16], edge = pp[17], *inv_L = pp + 18, dx = pp[21];
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const long q = g.idx(i, j, k);
                const float r = rho[q];
                const float x = tclamp(xi[q], 0.0f, 1.0f);
                const float df = f16_to_f32(df16[q]);
                const float ni = r * x;
                const float ha = ni * ni;
                const float oiii = ha * sstep_f(-0.03f, -0.12f, df);
                const float sii = ha * sstep_f(-0.05f, -0.005f, df);
                float dust = r * (1.0f - x) + 0.08f * ni;
                const float gv = f16_to_f32(g016[q]);
                const float geff = gv / (1.0f + gv / gs) + ambient;
                const float sh = shock_on ? shock_at_f(g, rho, mx, my, mz, i, j, k, dx) : 0.0f;
                float em[3];
                for (int c = 0; c < 3; ++c)
                    em[c] = ha * c_ha[c] + oiii * c_o3[c] + sii * c_s2[c] + (dust * geff) * c_dg[c] + sh * c_sh[c];
                const float p0 = ((float)i + 0.5f) * dx * inv_L[0];
                const float p1 = ((float)j + 0.5f) * dx * inv_L[1];
                const float p2 = ((float)k + 0.5f) * dx * inv_L[2];
                const float f = fade_f(p0, edge) * fade_f(p1, edge) * fade_f(p2, edge);
                for (int c = 0; c < 3; ++c) em[c] = em[c] * f;
                dust = dust * f;
                const float m = 60000.0f;
                for (int c = 0; c < 3; ++c) out[q * 4 + c] = f32_to_f16_rne(tmin(em[c], m));
                out[q * 4 + 3] = f32_to_f16_rne(tmin(dust, m));
            }
}

// render.py:281-298 smooth_axis: [1 4 1]/6 along one axis, clamped at the faces
static void render_smooth_f(int nx, int ny, int nz, const uint16_t* src, uint16_t* dst, int axis) {
    const Grid g{nx, ny, nz};
    const int oi = axis == 0, oj = axis == 1, ok = axis == 2;
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const long a = g.idx(imax(i - oi, 0), imax(j - oj, 0), imax(k - ok, 0));
                const long b = g.idx(i, j, k);
                const long c = g.idx(imin(i + oi, nx - 1), imin(j + oj, ny - 1), imin(k + ok, nz - 1));
                for (int ch = 0; ch < 4; ++ch) {
                    const float v = (f16_to_f32(src[a * 4 + ch]) + 4.0f * f16_to_f32(src[b * 4 + ch]) +
                                     f16_to_f32(src[c * 4 + ch])) / 6.0f;
                    dst[b * 4 + ch] = f32_to_f16_rne(v);
                }
            }
}

// ==================================================================================== C ABI
#define NB_ORACLE_EXPORT extern "C" __attribute__((visibility("default")))

#define INSTANTIATE(T, SFX)                                                                                         \
    NB_ORACLE_EXPORT void oracle_hydro_stage_##SFX(                                                                   \
        int nx, int ny, int nz, const T* rho, const T* mx, const T* my, const T* mz, const T* xi, const T* r0,        \
        const T* mx0, const T* my0, const T* mz0, T* o_r, T* o_mx, T* o_my, T* o_mz, const T* stars, int nstars,      \
        T wind, const T* jets, T jet_cos, T jet_r, T pulse, T dt, T dx, T a, T b, T floor_, T cn2, T ci2, T vmax,     \
        int solver, int lim) {                                                                                      \
        hydro_stage_t<T>(nx, ny, nz, rho, mx, my, mz, xi, r0, mx0, my0, mz0, o_r, o_mx, o_my, o_mz, stars, nstars,   \
                         wind, jets, jet_cos, jet_r, pulse, dt, dx, a, b, floor_, cn2, ci2, vmax, solver, lim);      \
    }                                                                                                               \
    NB_ORACLE_EXPORT T oracle_max_speed_##SFX(int nx, int ny, int nz, const T* rho, const T* mx, const T* my,        \
                                              const T* mz, const T* xi, T cn2, T ci2) {                             \
        return max_speed_t<T>(nx, ny, nz, rho, mx, my, mz, xi, cn2, ci2);                                           \
    }                                                                                                               \
    NB_ORACLE_EXPORT void oracle_cast_rays_##SFX(int nx, int ny, int nz, const T* rho, const T* star, T Q, T dr,     \
                                                 int nsteps, T dx, T rcap, const T* bmax, int nu, int nphi,         \
                                                 T* rfront) {                                                       \
        cast_rays_t<T>(nx, ny, nz, rho, star, Q, dr, nsteps, dx, rcap, bmax, nu, nphi, rfront);                     \
    }                                                                                                               \
    NB_ORACLE_EXPORT void oracle_apply_front_##SFX(int nx, int ny, int nz, const T* rfront, int nu, int nphi,        \
                                                   const T* star, T dx, T width, T* xi, T* dfront) {                \
        apply_front_t<T>(nx, ny, nz, rfront, nu, nphi, star, dx, width, xi, dfront);                                \
    }                                                                                                               \
    NB_ORACLE_EXPORT void oracle_smooth_xi_##SFX(int nx, int ny, int nz, const T* src, T* dst) {                    \
        smooth_xi_t<T>(nx, ny, nz, src, dst);                                                                       \
    }                                                                                                               \
    NB_ORACLE_EXPORT void oracle_cast_fuv_##SFX(int nx, int ny, int nz, const T* rho, const T* xi, const T* star,    \
                                                T kappa, T dr, int nsteps, T dx, T binr, const T* bmax, int nr,     \
                                                int nu, int nphi, T* att) {                                         \
        cast_fuv_t<T>(nx, ny, nz, rho, xi, star, kappa, dr, nsteps, dx, binr, bmax, nr, nu, nphi, att);             \
    }                                                                                                               \
    NB_ORACLE_EXPORT void oracle_apply_fuv_##SFX(int nx, int ny, int nz, const T* att, int nr, int nu, int nphi,     \
                                                 const T* star, T lum, T dx, T binr, T* g0) {                       \
        apply_fuv_t<T>(nx, ny, nz, att, nr, nu, nphi, star, lum, dx, binr, g0);                                     \
    }

#define INSTANTIATE_PLANE(T, SFX)                                                                           \
    NB_ORACLE_EXPORT void oracle_plane_front_##SFX(int nx, int ny, int nz, const T* rho, T F, T dx, T rcap, T* xf) {  \
        plane_front_t<T>(nx, ny, nz, rho, F, dx, rcap, xf);                                                      \
    }                                                                                                         \
    NB_ORACLE_EXPORT void oracle_apply_plane_##SFX(int nx, int ny, int nz, const T* xf, T dx, T width, T* xi,     \
                                                   T* dfront) {                                               \
        apply_plane_t<T>(nx, ny, nz, xf, dx, width, xi, dfront);                                              \
    }                                                                                                         \
    NB_ORACLE_EXPORT void oracle_plane_fuv_##SFX(int nx, int ny, int nz, const T* rho, const T* xi, T kappa, T lum, \
                                                 T dx, T* g) {                                                \
        plane_fuv_t<T>(nx, ny, nz, rho, xi, kappa, lum, dx, g);                                               \
    }
#define INSTANTIATE_STIR(T, SFX)                                                                              \
    NB_ORACLE_EXPORT void oracle_drive_##SFX(int nx, int ny, int nz, const T* rho, T* mx, T* my, T* mz, int sx,      \
                                             int sy, int sz, const T* fa, const T* fb, T blend, T amp, T dt, T dx,   \
                                             T dxs) {                                                               \
        drive_t<T>(nx, ny, nz, rho, mx, my, mz, sx, sy, sz, fa, fb, blend, amp, dt, dx, dxs);                       \
    }                                                                                                               \
    NB_ORACLE_EXPORT void oracle_add_torus_##SFX(long n, const T* torus, T* rho, T* mx, T* my, T* mz) {             \
        add_torus_t<T>(n, torus, rho, mx, my, mz);                                                                  \
    }
INSTANTIATE_STIR(float, f32)
INSTANTIATE_STIR(double, f64)

INSTANTIATE_PLANE(float, f32)
INSTANTIATE_PLANE(double, f64)

INSTANTIATE(float, f32)
INSTANTIATE(double, f64)

NB_ORACLE_EXPORT void oracle_to_half(const float* src, uint16_t* dst, long n) {
#pragma omp parallel for schedule(static)
    for (long q = 0; q < n; ++q) dst[q] = f32_to_f16_rne(src[q]);
}

NB_ORACLE_EXPORT void oracle_render_pack(int nx, int ny, int nz, const float* rho, const float* mx, const float* my,
                                          const float* mz, const float* xi, const uint16_t* df16,
                                          const uint16_t* g016, const float* pp, int shock_on, uint16_t* out) {
    render_pack_f(nx, ny, nz, rho, mx, my, mz, xi, df16, g016, pp, shock_on, out);
}

NB_ORACLE_EXPORT void oracle_render_smooth(int nx, int ny, int nz, const uint16_t* src, uint16_t* dst, int axis) {
    render_smooth_f(nx, ny, nz, src, dst, axis);
}

NB_ORACLE_EXPORT int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
