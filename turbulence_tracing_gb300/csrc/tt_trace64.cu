// K2a: plain FP64 drop-in tracer and the dndr lookup.
//
// Replaces ElectronCube.solve / dsdt / dndr / ray_at_exit
// (particle_tracking/particle_tracker.py:243-256, 312-380, 398-419).
// One thread integrates one ray with its own explicit Runge-Kutta instance
// that follows scipy.integrate.solve_ivp step for step: RK45 (Dormand-Prince
// 5(4), the reference's default method) built in, and any pair of the shapes
// of scipy's RK23 (3 stages) and DOP853 (12 stages, E5/E3 error norm) from a
// caller's tableau; scipy's initial-step rule, RMS error norm over the ray's
// own components, safety 0.9, step factors in [0.2, 10], exponent
// -1/(error order + 1), step clipped to t_bound, 10-spacing minimum step.
// Lookups reproduce RegularGridInterpolator(method='linear', fill_value=0)
// operation by operation.  The file is compiled with -fmad=false so every
// product and sum is rounded separately, as numpy does.
//
// The reference integrates all rays as one system with one global step; a
// per-ray step is the GPU-natural decomposition and converges to the same
// trajectories (parity is asserted at tight tolerance).
#include <math.h>
#include <string.h>

#include "tt_common.cuh"

namespace {

struct Grid64 {
    const double* g[3];
    int n[3];
    size_t s0, s1;  // element strides of ix and iy
};

struct Vols64 {
    const double* v[4];  // dndx, dndy, dndz, ne_nc
    int nvol;
};

// searchsorted(g, v, 'left') - 1 clipped to [0, n-2], starting from a guess
// made with the mean spacing; falls back to bisection if the guess is far off.
__device__ inline int locate64(const double* __restrict__ g, int n, double g0, double gn, double v)
{
    // first guess in FP32 (the walk below makes it exact)
    const float span = (float)(gn - g0);
    int i = span > 0.f ? (int)floorf((float)(v - g0) * __fdividef((float)(n - 1), span)) : 0;
    if (i < -1) i = -1;
    if (i > n - 1) i = n - 1;
    // want the largest i with g[i] < v (i = -1 if none)
    int it = 0;
    while (i + 1 < n && __ldg(g + i + 1) < v && it < 4) { ++i; ++it; }
    while (i >= 0 && !(__ldg(g + i) < v) && it < 8) { --i; ++it; }
    const bool ok = (i + 1 >= n || !(__ldg(g + i + 1) < v)) && (i < 0 || __ldg(g + i) < v);
    if (!ok) {
        int lo = 0, hi = n;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(g + mid) < v) lo = mid + 1; else hi = mid;
        }
        i = lo - 1;
    }
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    return i;
}

// Trilinear lookup of the first NV volumes at p.  Returns 0 = inside,
// 1 = outside (values 0), 2 = NaN coordinate (values NaN).
template <int NV>
__device__ inline int lookup64(const Grid64& G, const Vols64& V, const double p[3], double out[NV])
{
    int idx[3];
    double d[3];
    int oob = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double v = p[a];
        if (v != v) {
#pragma unroll
            for (int k = 0; k < NV; ++k) out[k] = CUDART_NAN;
            return 2;
        }
        const double lo = __ldg(G.g[a]), hi = __ldg(G.g[a] + G.n[a] - 1);
        if (v < lo || v > hi) oob = 1;
        const int i = locate64(G.g[a], G.n[a], lo, hi, v);
        idx[a] = i;
        const double gi = __ldg(G.g[a] + i);
        d[a] = (v - gi) / (__ldg(G.g[a] + i + 1) - gi);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = 0.0;
    if (oob) return 1;
    const size_t base = (size_t)idx[0] * G.s0 + (size_t)idx[1] * G.s1 + (size_t)idx[2];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int a = c >> 2, b = (c >> 1) & 1, e = c & 1;
        double w = 1.0;
        w = w * (a ? d[0] : 1.0 - d[0]);
        w = w * (b ? d[1] : 1.0 - d[1]);
        w = w * (e ? d[2] : 1.0 - d[2]);
        const size_t off = base + (a ? G.s0 : 0) + (b ? G.s1 : 0) + (size_t)e;
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = out[k] + __ldg(V.v[k] + off) * w;
    }
    return 0;
}

struct Cube64 {
    Grid64 G;
    Vols64 V;
    double k0;
};

// Right-hand side without the trivial rows: the accelerations (dv/dt = the
// interpolated gradients, dsdt at particle_tracker.py:398-419) and, with
// NEQ == 7, the phase rate k0 (n - 1) |v|.  Position rates are the velocity.
template <int NEQ>
__device__ inline void accel64(const Cube64& C, const double* pos, const double* vel, double* a)
{
    double g[NEQ == 7 ? 4 : 3];
    lookup64<NEQ == 7 ? 4 : 3>(C.G, C.V, pos, g);
    a[0] = g[0];
    a[1] = g[1];
    a[2] = g[2];
    if (NEQ == 7) {
        const double q = g[3];
        double r = 1.0 - q;
        if (r < 0.0) r = 0.0;
        const double nm1 = -q / (1.0 + sqrt(r));
        const double sp = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
        a[3] = C.k0 * nm1 * sp;
    }
}

// An explicit Runge-Kutta pair as scipy's RungeKutta classes hold it (A, B,
// C, E or DOP853's E5/E3) and its error order, in the kernel parameter bank.
struct RKDev {
    double a[TT_RK_MAX_STAGES][TT_RK_MAX_STAGES];
    double b[TT_RK_MAX_STAGES];
    double e[TT_RK_MAX_STAGES + 1];   // E, or E5 (DOP853)
    double e3[TT_RK_MAX_STAGES + 1];  // DOP853 only
    double err_exp;   // -1 / (error order + 1)
    double init_exp;  //  1 / (error order + 1)
};

template <int NEQ>
__device__ inline double rms(const double* v)
{
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NEQ; ++i) s += v[i] * v[i];
    return sqrt(s) / sqrt((double)NEQ);
}

// scipy.integrate._ivp.common.select_initial_step (Hairer, Norsett & Wanner,
// Sec. II.4); f0 holds the accelerations (and phase rate) at y0.
template <int NEQ>
__device__ double initial_step64(const Cube64& C, const RKDev& T, const double* y0, const double* f0,
                                 double t_bound, double rtol, double atol)
{
    constexpr int NA = NEQ - 3;
    double sc[NEQ], tmp[NEQ], f[NEQ];
    const double L = fabs(t_bound);
    if (L == 0.0) return 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) f[i] = y0[3 + i];
#pragma unroll
    for (int i = 0; i < NA; ++i) f[3 + i] = f0[i];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) sc[i] = atol + fabs(y0[i]) * rtol;
#pragma unroll
    for (int i = 0; i < NEQ; ++i) tmp[i] = y0[i] / sc[i];
    const double d0 = rms<NEQ>(tmp);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) tmp[i] = f[i] / sc[i];
    const double d1 = rms<NEQ>(tmp);
    double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    if (h0 > L) h0 = L;
    double y1[NEQ], f1[NA];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) y1[i] = y0[i] + h0 * f[i];
    accel64<NEQ>(C, y1, y1 + 3, f1);
#pragma unroll
    for (int i = 0; i < 3; ++i) tmp[i] = (y1[3 + i] - f[i]) / sc[i];
#pragma unroll
    for (int i = 0; i < NA; ++i) tmp[3 + i] = (f1[i] - f[3 + i]) / sc[3 + i];
    const double d2 = rms<NEQ>(tmp) / h0;
    double h1;
    if (d1 <= 1e-15 && d2 <= 1e-15) {
        h1 = h0 * 1e-3;
        if (h1 < 1e-6) h1 = 1e-6;
    } else {
        const double m = d1 > d2 ? d1 : d2;
        h1 = pow(0.01 / m, T.init_exp);
    }
    double h = 100.0 * h0;
    if (h1 < h) h = h1;
    if (L < h) h = L;
    return h;
}

// One ray through scipy's RungeKutta loop (safety 0.9, factors in [0.2, 10],
// RMS norm, step clipped to t_bound, TOO_SMALL below 10 spacings of t), cut
// into single attempts so that a warp's lanes can each carry their own ray:
// attempt() makes one try of a step (scipy's rk_step + _estimate_error_norm +
// the accept/reject decision of _step_impl) and keeps the loop state in Ray64.
// NS stages per step plus the FSAL evaluation at the new point; every stage's
// rates are kept for all NEQ components and combined in scipy's order
// (y + (sum_j K[j] a[s][j]) h).  DOP853 (DOP = true) takes scipy's combined
// E5/E3 error norm.
template <int NS, int NEQ>
struct Ray64 {
    double y[NEQ];
    double K[NS + 1][NEQ];  // K[0]: the rates at y (scipy's self.f)
    double t, h_abs;
    long long natt, nacc;
    bool fresh;     // the next attempt starts a new step (scipy's _step_impl entry)
    bool rejected;  // a try of the current step was rejected
};

enum { kAttemptMore = -1 };

template <int NEQ>
__device__ inline void rhs64(const Cube64& C, const double* y, double* f)
{
#pragma unroll
    for (int i = 0; i < 3; ++i) f[i] = y[3 + i];
    accel64<NEQ>(C, y, y + 3, f + 3);
}

// Start a ray: rates at y0 and scipy's initial step.  Returns false for a
// non-finite start (status NaN).
template <int NS, int NEQ>
__device__ bool start64(const Cube64& C, const RKDev& T, Ray64<NS, NEQ>& R, double t_bound, double rtol, double atol)
{
    R.t = 0.0;
    R.natt = R.nacc = 0;
    R.fresh = true;
    R.rejected = false;
    for (int i = 0; i < NEQ; ++i)
        if (!isfinite(R.y[i])) return false;
    rhs64<NEQ>(C, R.y, R.K[0]);
    R.h_abs = initial_step64<NEQ>(C, T, R.y, R.K[0] + 3, t_bound, rtol, atol);
    return true;
}

// One try of a step.  Returns kAttemptMore while the ray goes on, else its
// final tt_ray_status (TT_RAY_OK once t reaches t_bound).
template <int NS, bool DOP, int NEQ>
__device__ int attempt64(const Cube64& C, const RKDev& T, Ray64<NS, NEQ>& R, double t_bound, double rtol,
                         double atol, long long max_steps)
{
    if (R.t == t_bound) return TT_RAY_OK;
    const double min_step = 10.0 * fabs(nextafter(R.t, CUDART_INF) - R.t);
    if (R.fresh) {
        if (R.h_abs < min_step) R.h_abs = min_step;
        R.rejected = false;
        R.fresh = false;
    }
    if (R.h_abs < min_step) return TT_RAY_STEP_TOO_SMALL;
    if (R.natt >= max_steps) return TT_RAY_MAX_STEPS;
    ++R.natt;
    double h = R.h_abs;
    double t_new = R.t + h;
    if (t_new - t_bound > 0) t_new = t_bound;
    h = t_new - R.t;
    R.h_abs = fabs(h);
    double yn[NEQ];
    // stages 1..NS-1 and the new point (the B row) at s = NS
#pragma unroll 1
    for (int s = 1; s <= NS; ++s) {
        const double* a = s < NS ? T.a[s] : T.b;
        double ys[NEQ];
#pragma unroll
        for (int i = 0; i < NEQ; ++i) {
            double acc = 0.0;
            for (int j = 0; j < s; ++j) acc += R.K[j][i] * a[j];
            ys[i] = R.y[i] + acc * h;
        }
        if (s == NS) {
#pragma unroll
            for (int i = 0; i < NEQ; ++i) yn[i] = ys[i];
        }
        rhs64<NEQ>(C, ys, R.K[s]);
    }
    double e5s = 0.0, e3s = 0.0;
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        const double ay = fabs(R.y[i]), an = fabs(yn[i]);
        const double sc = atol + (ay > an ? ay : an) * rtol;
        double acc = 0.0, acc3 = 0.0;
        for (int j = 0; j <= NS; ++j) {
            acc += R.K[j][i] * T.e[j];
            if (DOP) acc3 += R.K[j][i] * T.e3[j];
        }
        if (DOP) {
            const double x5 = acc / sc, x3 = acc3 / sc;
            e5s += x5 * x5;
            e3s += x3 * x3;
        } else {
            const double e = acc * h / sc;
            e5s += e * e;
        }
    }
    double en;
    if (DOP) {
        if (e5s == 0.0 && e3s == 0.0) en = 0.0;
        else en = fabs(h) * e5s / sqrt((e5s + 0.01 * e3s) * (double)NEQ);
    } else {
        en = sqrt(e5s) / sqrt((double)NEQ);
    }
    if (en < 1.0) {
        double factor;
        if (en == 0.0) factor = 10.0;
        else {
            factor = 0.9 * pow(en, T.err_exp);
            if (!(factor < 10.0)) factor = 10.0;
        }
        if (R.rejected && !(factor < 1.0)) factor = 1.0;
        R.h_abs *= factor;
        ++R.nacc;
        R.t = t_new;
#pragma unroll
        for (int i = 0; i < NEQ; ++i) {
            R.y[i] = yn[i];
            R.K[0][i] = R.K[NS][i];
        }
        R.fresh = true;
        return (R.t - t_bound >= 0) ? TT_RAY_OK : kAttemptMore;
    }
    double factor = 0.9 * pow(en, T.err_exp);
    if (!(factor > 0.2)) factor = 0.2;
    R.h_abs *= factor;
    R.rejected = true;
    return kAttemptMore;
}

// ray_at_exit, particle_tracker.py:333-380
__device__ inline void ray_at_exit64(const double* y, int axis, double extent, double rf[4])
{
    const double x = y[0], yy = y[1], z = y[2], vx = y[3], vy = y[4], vz = y[5];
    if (axis == 0) {
        const double tbp = (x - extent) / vx;
        rf[0] = yy - vy * tbp;
        rf[2] = z - vz * tbp;
        rf[1] = atan(vy / vx);
        rf[3] = atan(vz / vx);
    } else if (axis == 1) {
        const double tbp = (yy - extent) / vy;
        rf[0] = x - vx * tbp;
        rf[2] = z - vz * tbp;
        rf[1] = atan(vx / vy);
        rf[3] = atan(vz / vy);
    } else {
        const double tbp = (z - extent) / vz;
        rf[0] = x - vx * tbp;
        rf[2] = yy - vy * tbp;
        rf[1] = atan(vx / vz);
        rf[3] = atan(vy / vz);
    }
}

// Persistent form: the grid fills the GPU, each warp owns a contiguous range
// of rays, and a lane whose ray is done takes the next ray of its warp's range
// (ballot + popc, no global atomics), so the lanes of a warp stay busy while
// rays with short and long paths mix.  Each loop pass makes one attempt on
// every busy lane.  Registers: 3 blocks of 128 per SM for RK23 / RK45, 2 for
// DOP853.
template <int NS>
struct Occ64 {
    static constexpr int blocks = NS <= 6 ? 3 : 2;
};

template <int NS, int NEQ>
__device__ inline void finish64(const Ray64<NS, NEQ>& R, int code, long long r, long long np, int axis, double extent,
                                double* __restrict__ sf, double* __restrict__ rf, double* __restrict__ phase,
                                int* __restrict__ status, int* __restrict__ nsteps)
{
    if (sf) {
#pragma unroll
        for (int i = 0; i < 6; ++i) sf[(size_t)i * np + r] = R.y[i];
    }
    if (rf) {
        double o[4];
        ray_at_exit64(R.y, axis, extent, o);
#pragma unroll
        for (int i = 0; i < 4; ++i) rf[(size_t)i * np + r] = o[i];
    }
    if (phase) phase[r] = NEQ == 7 ? R.y[NEQ - 1] : 0.0;
    if (status) status[r] = code;
    if (nsteps) nsteps[r] = (int)(R.nacc > 0x7fffffff ? 0x7fffffff : R.nacc);
}

template <int NS, bool DOP, int NEQ>
__global__ void __launch_bounds__(128, Occ64<NS>::blocks)
trace64_kernel(Cube64 C, const __grid_constant__ RKDev T, const double* __restrict__ s0, long long np,
               double t_end, int axis, double extent, double rtol, double atol, long long max_steps,
               double* __restrict__ sf, double* __restrict__ rf, double* __restrict__ phase,
               int* __restrict__ status, int* __restrict__ nsteps)
{
    const unsigned lane = threadIdx.x & 31u;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const long long per = (np + nwarps - 1) / nwarps;
    const long long wbeg = w * per < np ? w * per : np;
    const long long wend = wbeg + per < np ? wbeg + per : np;
    long long next = wbeg;  // warp-uniform cursor into the warp's range
    long long r = -1;
    Ray64<NS, NEQ> R;
    for (;;) {
        const bool need = r < 0;
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        if (mask) {
            const unsigned rank = __popc(mask & ((1u << lane) - 1u));
            if (need && next + rank < wend) {
                r = next + rank;
#pragma unroll
                for (int i = 0; i < 6; ++i) R.y[i] = s0[(size_t)i * np + r];
                if (NEQ == 7) R.y[NEQ - 1] = 0.0;
                if (!start64<NS, NEQ>(C, T, R, t_end, rtol, atol)) {
                    finish64<NS, NEQ>(R, TT_RAY_NAN, r, np, axis, extent, sf, rf, phase, status, nsteps);
                    r = -1;  // refilled on the next pass
                }
            }
            const long long got = next + __popc(mask);
            next = got < wend ? got : wend;
        }
        if (__ballot_sync(0xffffffffu, r >= 0 || next < wend) == 0u) break;
        if (r >= 0) {
            const int code = attempt64<NS, DOP, NEQ>(C, T, R, t_end, rtol, atol, max_steps);
            if (code != kAttemptMore) {
                finish64<NS, NEQ>(R, code, r, np, axis, extent, sf, rf, phase, status, nsteps);
                r = -1;
            }
        }
    }
}

template <int NV>
__global__ void dndr_kernel(Grid64 G, Vols64 V, const double* __restrict__ pts, long long npts,
                            double* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npts;
         i += (long long)gridDim.x * blockDim.x) {
        double p[3] = {pts[i], pts[npts + i], pts[2 * npts + i]};
        double o[NV];
        lookup64<NV>(G, V, p, o);
#pragma unroll
        for (int k = 0; k < NV; ++k) out[(size_t)k * npts + i] = o[k];
    }
}

int make_grid(int nx, int ny, int nz, const double* x, const double* y, const double* z, Grid64* G)
{
    const double* cs[3] = {x, y, z};
    const int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        G->g[a] = cs[a];
        G->n[a] = n[a];
    }
    G->s0 = (size_t)ny * nz;
    G->s1 = (size_t)nz;
    return TT_OK;
}

int grid_size(long long n, int block)
{
    long long g = (n + block - 1) / block;
    const long long cap = (long long)tt::sm_count() * 64;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

extern "C" int tt_dndr(const double* const* vols, int nvol, int nx, int ny, int nz, const double* x,
                       const double* y, const double* z, const double* pts, int64_t npts, double* out,
                       void* stream)
{
    if (!vols || nvol < 1 || nvol > 4) return tt::invalid("dndr: need 1..4 volumes");
    if (nx < 2 || ny < 2 || nz < 2) return tt::invalid("dndr: every axis needs at least 2 points");
    if (!x || !y || !z || (npts > 0 && (!pts || !out))) return tt::invalid("dndr: null pointer");
    if (npts < 0) return tt::invalid("dndr: npts < 0");
    if (npts == 0) return TT_OK;
    Grid64 G;
    TT_TRY(make_grid(nx, ny, nz, x, y, z, &G));
    Vols64 V;
    V.nvol = nvol;
    for (int k = 0; k < 4; ++k) V.v[k] = k < nvol ? vols[k] : nullptr;
    for (int k = 0; k < nvol; ++k)
        if (!V.v[k]) return tt::invalid("dndr: null volume");
    const int g = grid_size(npts, 256);
    cudaStream_t st = tt::as_stream(stream);
    switch (nvol) {
        case 1: dndr_kernel<1><<<g, 256, 0, st>>>(G, V, pts, npts, out); break;
        case 2: dndr_kernel<2><<<g, 256, 0, st>>>(G, V, pts, npts, out); break;
        case 3: dndr_kernel<3><<<g, 256, 0, st>>>(G, V, pts, npts, out); break;
        default: dndr_kernel<4><<<g, 256, 0, st>>>(G, V, pts, npts, out); break;
    }
    return tt::launch_status("dndr kernel");
}

namespace {

// Dormand-Prince 5(4) as scipy's RK45 holds it (Dormand & Prince 1980).
tt_rk_tableau dp54()
{
    tt_rk_tableau t{};
    t.n_stages = 6;
    t.error_order = 4;
    t.error_kind = 0;
    const double C[6] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0};
    const double A[6][5] = {
        {0, 0, 0, 0, 0},
        {1.0 / 5, 0, 0, 0, 0},
        {3.0 / 40, 9.0 / 40, 0, 0, 0},
        {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0},
        {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0},
        {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656}};
    const double B[6] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84};
    const double E[7] = {-71.0 / 57600, 0, 71.0 / 16695, -71.0 / 1920, 17253.0 / 339200, -22.0 / 525, 1.0 / 40};
    for (int s = 0; s < 6; ++s) {
        t.C[s] = C[s];
        t.B[s] = B[s];
        for (int k = 0; k < 5; ++k) t.A[s][k] = A[s][k];
    }
    for (int s = 0; s < 7; ++s) t.E[s] = E[s];
    return t;
}

// Checks a caller's tableau and forms the device copy.
int make_rkdev(const tt_rk_tableau* t, RKDev* D)
{
    const int ns = t->n_stages;
    if (!(ns == 3 || ns == 6 || ns == 12))
        return tt::invalid("trace_f64: n_stages must be 3, 6 or 12 (RK23, RK45, DOP853 forms)");
    if (t->error_kind != 0 && t->error_kind != 1) return tt::invalid("trace_f64: error_kind must be 0 or 1");
    if ((t->error_kind == 1) != (ns == 12))
        return tt::invalid("trace_f64: the E5/E3 error norm (error_kind 1) goes with 12 stages");
    if (t->error_order < 1 || t->error_order > 16) return tt::invalid("trace_f64: error_order must be 1..16");
    for (int s = 0; s < ns; ++s) {
        double rs = 0.0;
        for (int k = 0; k < s; ++k) rs += t->A[s][k];
        for (int k = s; k < TT_RK_MAX_STAGES; ++k)
            if (t->A[s][k] != 0.0) return tt::invalid("trace_f64: A must be strictly lower triangular");
        if (fabs(rs - t->C[s]) > 1e-12) return tt::invalid("trace_f64: row sums of A must equal C");
    }
    double sb = 0.0, se = 0.0, se3 = 0.0;
    for (int s = 0; s < ns; ++s) sb += t->B[s];
    for (int s = 0; s <= ns; ++s) {
        se += t->E[s];
        se3 += t->E3[s];
    }
    if (fabs(sb - 1.0) > 1e-12 || fabs(se) > 1e-12 || (t->error_kind == 1 && fabs(se3) > 1e-12))
        return tt::invalid("trace_f64: B must sum to 1 and E to 0");
    RKDev d;
    memset(&d, 0, sizeof(d));
    for (int s = 0; s < ns; ++s) {
        d.b[s] = t->B[s];
        for (int k = 0; k < ns; ++k) d.a[s][k] = t->A[s][k];
    }
    for (int k = 0; k <= ns; ++k) {
        d.e[k] = t->E[k];
        d.e3[k] = t->error_kind == 1 ? t->E3[k] : 0.0;
    }
    d.err_exp = -1.0 / (t->error_order + 1);
    d.init_exp = 1.0 / (t->error_order + 1);
    *D = d;
    return TT_OK;
}

// Resident blocks of 128 on the whole GPU, capped by the rays (a warp per 32 rays).
template <typename KernelT>
int resident_grid(KernelT kernel, long long np)
{
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 128, 0) != cudaSuccess || b < 1) b = 1;
    long long g = (long long)b * tt::sm_count();
    const long long need = (np + 127) / 128;
    if (g > need) g = need;
    return (int)(g < 1 ? 1 : g);
}

template <int NS, bool DOP>
void launch64(bool phase, const Cube64& C, const RKDev& T, const double* s0, long long np, double t_end, int axis,
              double extent, const tt_trace_opts* o, long long maxs, double* sf, double* rf, double* ph, int* st,
              int* ns, cudaStream_t s)
{
    if (phase)
        trace64_kernel<NS, DOP, 7><<<resident_grid(trace64_kernel<NS, DOP, 7>, np), 128, 0, s>>>(
            C, T, s0, np, t_end, axis, extent, o->rtol, o->atol, maxs, sf, rf, ph, st, ns);
    else
        trace64_kernel<NS, DOP, 6><<<resident_grid(trace64_kernel<NS, DOP, 6>, np), 128, 0, s>>>(
            C, T, s0, np, t_end, axis, extent, o->rtol, o->atol, maxs, sf, rf, ph, st, ns);
}

int trace64(const double* dndx, const double* dndy, const double* dndz, const double* ne_nc, int nx, int ny, int nz,
            const double* x, const double* y, const double* z, double omega, const double* s0, int64_t np,
            double t_end, int probing_axis, double extent, const tt_trace_opts* opts, const tt_rk_tableau* tab,
            double* sf, double* rf, double* phase, int32_t* status, int32_t* nsteps, void* stream)
{
    if (!opts) return tt::invalid("trace_f64: opts is null");
    if (!dndx || !dndy || !dndz || !x || !y || !z) return tt::invalid("trace_f64: null pointer");
    if (opts->with_phase && !ne_nc) return tt::invalid("trace_f64: phase needs ne_nc");
    if (nx < 2 || ny < 2 || nz < 2) return tt::invalid("trace_f64: every axis needs at least 2 points");
    if (probing_axis < 0 || probing_axis > 2) return tt::invalid("trace_f64: probing_axis must be 0, 1 or 2");
    if (np < 0) return tt::invalid("trace_f64: np < 0");
    if (!(opts->rtol > 0.0) || !(opts->atol >= 0.0)) return tt::invalid("trace_f64: need rtol > 0, atol >= 0");
    if (!(t_end >= 0.0)) return tt::invalid("trace_f64: t_end must be >= 0");
    RKDev T;
    TT_TRY(make_rkdev(tab, &T));
    if (np == 0) return TT_OK;
    if (!s0) return tt::invalid("trace_f64: s0 is null");
    Cube64 C;
    TT_TRY(make_grid(nx, ny, nz, x, y, z, &C.G));
    C.V.v[0] = dndx;
    C.V.v[1] = dndy;
    C.V.v[2] = dndz;
    C.V.v[3] = ne_nc;
    C.V.nvol = opts->with_phase ? 4 : 3;
    C.k0 = omega / TT_C_LIGHT;
    const long long maxs = opts->max_steps > 0 ? opts->max_steps : TT_DEFAULT_MAX_STEPS;
    cudaStream_t s = tt::as_stream(stream);
    const bool ph = opts->with_phase != 0;
    if (tab->n_stages == 3)
        launch64<3, false>(ph, C, T, s0, np, t_end, probing_axis, extent, opts, maxs, sf, rf, phase, status, nsteps, s);
    else if (tab->n_stages == 6)
        launch64<6, false>(ph, C, T, s0, np, t_end, probing_axis, extent, opts, maxs, sf, rf, phase, status, nsteps, s);
    else
        launch64<12, true>(ph, C, T, s0, np, t_end, probing_axis, extent, opts, maxs, sf, rf, phase, status, nsteps,
                           s);
    return tt::launch_status("trace_f64 kernel");
}

}  // namespace

extern "C" int tt_trace_f64(const double* dndx, const double* dndy, const double* dndz, const double* ne_nc,
                            int nx, int ny, int nz, const double* x, const double* y, const double* z,
                            double omega, const double* s0, int64_t np, double t_end, int probing_axis,
                            double extent, const tt_trace_opts* opts, double* sf, double* rf,
                            double* phase, int32_t* status, int32_t* nsteps, void* stream)
{
    static const tt_rk_tableau T = dp54();
    return trace64(dndx, dndy, dndz, ne_nc, nx, ny, nz, x, y, z, omega, s0, np, t_end, probing_axis, extent, opts,
                   &T, sf, rf, phase, status, nsteps, stream);
}

extern "C" int tt_trace_f64_rk(const double* dndx, const double* dndy, const double* dndz, const double* ne_nc,
                               int nx, int ny, int nz, const double* x, const double* y, const double* z,
                               double omega, const double* s0, int64_t np, double t_end, int probing_axis,
                               double extent, const tt_trace_opts* opts, const tt_rk_tableau* tableau, double* sf,
                               double* rf, double* phase, int32_t* status, int32_t* nsteps, void* stream)
{
    if (!tableau) return tt::invalid("trace_f64_rk: tableau is null");
    return trace64(dndx, dndy, dndz, ne_nc, nx, ny, nz, x, y, z, omega, s0, np, t_end, probing_axis, extent, opts,
                   tableau, sf, rf, phase, status, nsteps, stream);
}
