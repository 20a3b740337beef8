/*
 * tt_oracle.c -- CPU restatement of the turbulence_tracing ray-integration
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark call this as the checker.  The product
 * (turbulence_tracing_gb300) never links, loads or calls it.
 *
 * Every function cites the reference code it restates (paths are relative to
 * the jdhare/turbulence_tracing repository).  Third-party arithmetic the
 * reference relies on is restated from its published algorithm:
 *   - numpy.gradient (edge_order=1, coordinate arrays) -- numpy 2.x
 *   - scipy.interpolate.RegularGridInterpolator(method='linear',
 *     bounds_error=False, fill_value=0) -- scipy 1.18
 *   - scipy.integrate.solve_ivp(method='RK45'): Dormand-Prince 5(4) with the
 *     step controller of scipy's RungeKutta class (safety 0.9, factor range
 *     [0.2, 10], error exponent -1/5, RMS error norm, Hairer-Norsett-Wanner
 *     initial step selection).
 * Compile with -ffp-contract=off so that results do not depend on whether the
 * host compiler fuses multiply-adds (it does by default on aarch64).
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>

#define TTO_C 299792458.0 /* scipy.constants.c, particle_tracker.py:118 */

/* ------------------------------------------------------------------------ */
/* numpy.gradient along one axis of a C-ordered (n0,n1,n2) array, with a
 * coordinate array, edge_order=1.  Used by calc_dndr, particle_tracker.py:235-237.
 * numpy reduces the coordinate spacing to a scalar when np.diff(coord) is
 * exactly constant, and uses the three-point non-uniform formula otherwise. */
static void grad_axis(const double* f, const int n[3], int axis,
                      const double* coord, double* out)
{
    const int na = n[axis];
    size_t stride = 1;
    for (int a = 2; a > axis; --a) stride *= (size_t)n[a];
    size_t outer = 1;
    for (int a = 0; a < axis; ++a) outer *= (size_t)n[a];
    const size_t inner = stride;

    int uniform = 1;
    const double d0 = coord[1] - coord[0];
    for (int i = 1; i < na - 1; ++i)
        if (coord[i + 1] - coord[i] != d0) { uniform = 0; break; }

    for (size_t o = 0; o < outer; ++o) {
        const size_t base = o * (size_t)na * inner;
        for (size_t r = 0; r < inner; ++r) {
            const double* fl = f + base + r;
            double* ol = out + base + r;
            for (int i = 1; i < na - 1; ++i) {
                const double fm = fl[(size_t)(i - 1) * inner];
                const double f0 = fl[(size_t)i * inner];
                const double fp = fl[(size_t)(i + 1) * inner];
                double v;
                if (uniform) {
                    v = (fp - fm) / (2.0 * d0);
                } else {
                    const double dx1 = coord[i] - coord[i - 1];
                    const double dx2 = coord[i + 1] - coord[i];
                    const double a = -(dx2) / (dx1 * (dx1 + dx2));
                    const double b = (dx2 - dx1) / (dx1 * dx2);
                    const double c = dx1 / (dx2 * (dx1 + dx2));
                    v = a * fm + b * f0 + c * fp;
                }
                ol[(size_t)i * inner] = v;
            }
            const double dfirst = uniform ? d0 : (coord[1] - coord[0]);
            const double dlast = uniform ? d0 : (coord[na - 1] - coord[na - 2]);
            ol[0] = (fl[inner] - fl[0]) / dfirst;
            ol[(size_t)(na - 1) * inner] =
                (fl[(size_t)(na - 1) * inner] - fl[(size_t)(na - 2) * inner]) / dlast;
        }
    }
}

/* ElectronCube.calc_dndr, particle_tracker.py:220-237: omega, critical density,
 * n_e/n_c clipped at ne_max, and dndi = -0.5 c^2 d(ne_nc)/di.
 * Returns omega.  Arrays are C-ordered [ix,iy,iz]. */
double tto_calc_dndr(const double* ne, int nx, int ny, int nz,
                     const double* x, const double* y, const double* z,
                     double lwl, double ne_max,
                     double* ne_nc, double* dndx, double* dndy, double* dndz)
{
    const double omega = (2.0 * M_PI) * (TTO_C / lwl);
    const double nc = 3.14207787e-4 * (omega * omega);
    const size_t nv = (size_t)nx * ny * nz;
    for (size_t i = 0; i < nv; ++i) {
        double q = ne[i] / nc;
        if (q > ne_max) q = ne_max;
        ne_nc[i] = q;
    }
    const int n[3] = {nx, ny, nz};
    const double k = -0.5 * (TTO_C * TTO_C);
    grad_axis(ne_nc, n, 0, x, dndx);
    grad_axis(ne_nc, n, 1, y, dndy);
    grad_axis(ne_nc, n, 2, z, dndz);
    for (size_t i = 0; i < nv; ++i) {
        dndx[i] = k * dndx[i];
        dndy[i] = k * dndy[i];
        dndz[i] = k * dndz[i];
    }
    return omega;
}

/* ------------------------------------------------------------------------ */
/* RegularGridInterpolator(method='linear', bounds_error=False, fill_value=0),
 * built at particle_tracker.py:239-241 and called by dndr (:243-256).
 * Cell search: searchsorted(grid, v, 'left') - 1 clipped to [0, n-2];
 * weights multiplied in axis order and corners summed with the last axis
 * varying fastest (the order of scipy's hypercube loop). */
typedef struct {
    int n[3];
    const double* g[3];
} tto_grid;

static int locate(const double* g, int n, double v)
{
    int lo = 0, hi = n; /* first index with g[idx] >= v */
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (g[mid] < v) lo = mid + 1; else hi = mid;
    }
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    return i;
}

typedef struct {
    size_t off[8];
    double w[8];
    int oob;
    int nan;
} tto_stencil;

static void stencil(const tto_grid* G, const double p[3], tto_stencil* s)
{
    int idx[3];
    double d[3];
    s->oob = 0;
    s->nan = 0;
    for (int a = 0; a < 3; ++a) {
        const double v = p[a];
        if (v != v) { s->nan = 1; return; }
        if (v < G->g[a][0] || v > G->g[a][G->n[a] - 1]) s->oob = 1;
        const int i = locate(G->g[a], G->n[a], v);
        idx[a] = i;
        d[a] = (v - G->g[a][i]) / (G->g[a][i + 1] - G->g[a][i]);
    }
    if (s->oob) return;
    const size_t s1 = (size_t)G->n[2], s0 = (size_t)G->n[1] * G->n[2];
    int c = 0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int e = 0; e < 2; ++e) {
                double w = 1.0;
                w = w * (a ? d[0] : 1.0 - d[0]);
                w = w * (b ? d[1] : 1.0 - d[1]);
                w = w * (e ? d[2] : 1.0 - d[2]);
                s->w[c] = w;
                s->off[c] = (size_t)(idx[0] + a) * s0 + (size_t)(idx[1] + b) * s1 + (size_t)(idx[2] + e);
                ++c;
            }
}

static double apply(const tto_stencil* s, const double* vol)
{
    if (s->nan) return NAN;
    if (s->oob) return 0.0;
    double v = 0.0;
    for (int c = 0; c < 8; ++c) v = v + vol[s->off[c]] * s->w[c];
    return v;
}

/* Interpolate one volume at N points given as pts[3*i+a]. */
void tto_interp(const double* vol, int nx, int ny, int nz,
                const double* x, const double* y, const double* z,
                const double* pts, int64_t npts, double* out)
{
    tto_grid G = {{nx, ny, nz}, {x, y, z}};
    for (int64_t i = 0; i < npts; ++i) {
        tto_stencil s;
        stencil(&G, pts + 3 * i, &s);
        out[i] = apply(&s, vol);
    }
}

/* ------------------------------------------------------------------------ */
/* Ray ODE right-hand side, dsdt (particle_tracker.py:398-419) with dndr
 * (:243-256): x' = v, v' = grad.  The optional 7th component is the phase,
 * dphi/dt = k0 (n - 1) |v| with n - 1 = -q / (1 + sqrt(1 - q)) and q the
 * trilinearly interpolated n_e/n_c (the reference has no phase; this is the
 * restated definition). */
typedef struct {
    tto_grid G;
    const double* dndx;
    const double* dndy;
    const double* dndz;
    const double* ne_nc; /* only with phase */
    double k0;
    int neq;             /* 6, or 7 with phase */
} tto_cube;

static void rhs(const tto_cube* C, const double* y, double* f)
{
    tto_stencil s;
    stencil(&C->G, y, &s);
    f[0] = y[3];
    f[1] = y[4];
    f[2] = y[5];
    f[3] = apply(&s, C->dndx);
    f[4] = apply(&s, C->dndy);
    f[5] = apply(&s, C->dndz);
    if (C->neq == 7) {
        double q = apply(&s, C->ne_nc);
        double r = 1.0 - q;
        if (r < 0.0) r = 0.0;
        const double nm1 = -q / (1.0 + sqrt(r));
        const double sp = sqrt(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
        f[6] = C->k0 * nm1 * sp;
    }
}

/* Dormand-Prince 5(4) tableau (Dormand & Prince 1980), as used by RK45. */
static const double DP_C[6] = {0.0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1.0};
static const double DP_A[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656}};
static const double DP_B[6] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84};
static const double DP_E[7] = {-71.0 / 57600, 0, 71.0 / 16695, -71.0 / 1920, 17253.0 / 339200, -22.0 / 525, 1.0 / 40};

static double rms(const double* v, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += v[i] * v[i];
    return sqrt(s) / sqrt((double)n);
}

/* scipy.integrate._ivp.common.select_initial_step with order 4. */
static double initial_step(const tto_cube* C, const double* y0, const double* f0,
                           double t_bound, double rtol, double atol, int64_t* nfev)
{
    const int n = C->neq;
    double sc[7], tmp[7], y1[7], f1[7];
    const double L = fabs(t_bound);
    if (L == 0.0) return 0.0;
    for (int i = 0; i < n; ++i) sc[i] = atol + fabs(y0[i]) * rtol;
    for (int i = 0; i < n; ++i) tmp[i] = y0[i] / sc[i];
    const double d0 = rms(tmp, n);
    for (int i = 0; i < n; ++i) tmp[i] = f0[i] / sc[i];
    const double d1 = rms(tmp, n);
    double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    if (h0 > L) h0 = L;
    for (int i = 0; i < n; ++i) y1[i] = y0[i] + h0 * f0[i];
    rhs(C, y1, f1);
    ++*nfev;
    for (int i = 0; i < n; ++i) tmp[i] = (f1[i] - f0[i]) / sc[i];
    const double d2 = rms(tmp, n) / h0;
    double h1;
    if (d1 <= 1e-15 && d2 <= 1e-15) {
        h1 = h0 * 1e-3;
        if (h1 < 1e-6) h1 = 1e-6;
    } else {
        const double m = d1 > d2 ? d1 : d2;
        h1 = pow(0.01 / m, 1.0 / 5.0);
    }
    double h = 100.0 * h0;
    if (h1 < h) h = h1;
    if (L < h) h = L;
    return h;
}

enum { TTO_OK = 0, TTO_TOO_SMALL = 1, TTO_MAXSTEPS = 2 };

/* One ray through solve_ivp(RK45) from t=0 to t_bound (particle_tracker.py:312-331),
 * with each ray carrying its own step size and RMS norm over its own components. */
static int integrate_ray(const tto_cube* C, double* y, double t_bound,
                         double rtol, double atol, int64_t max_steps,
                         int64_t* nacc, int64_t* nrej, int64_t* nfev)
{
    const int n = C->neq;
    double f[7], K[7][7], yn[7], ys[7], sc[7], e[7];
    rhs(C, y, f);
    *nfev = 1;
    *nacc = 0;
    *nrej = 0;
    double h_abs = initial_step(C, y, f, t_bound, rtol, atol, nfev);
    double t = 0.0;
    if (t == t_bound) return TTO_OK;
    for (;;) {
        const double min_step = 10.0 * fabs(nextafter(t, INFINITY) - t);
        if (h_abs < min_step) h_abs = min_step;
        int rejected = 0;
        double t_new, h;
        for (;;) {
            if (h_abs < min_step) return TTO_TOO_SMALL;
            if (*nacc + *nrej >= max_steps) return TTO_MAXSTEPS;
            h = h_abs;
            t_new = t + h;
            if (t_new - t_bound > 0) t_new = t_bound;
            h = t_new - t;
            h_abs = fabs(h);
            /* rk_step */
            for (int i = 0; i < n; ++i) K[0][i] = f[i];
            for (int s = 1; s < 6; ++s) {
                for (int i = 0; i < n; ++i) {
                    double acc = 0.0;
                    for (int j = 0; j < s; ++j) acc += K[j][i] * DP_A[s][j];
                    ys[i] = y[i] + acc * h;
                }
                rhs(C, ys, K[s]);
            }
            for (int i = 0; i < n; ++i) {
                double acc = 0.0;
                for (int j = 0; j < 6; ++j) acc += K[j][i] * DP_B[j];
                yn[i] = y[i] + h * acc;
            }
            rhs(C, yn, K[6]);
            *nfev += 6;
            for (int i = 0; i < n; ++i) {
                const double ay = fabs(y[i]), an = fabs(yn[i]);
                sc[i] = atol + (ay > an ? ay : an) * rtol;
                double acc = 0.0;
                for (int j = 0; j < 7; ++j) acc += K[j][i] * DP_E[j];
                e[i] = acc * h / sc[i];
            }
            const double en = rms(e, n);
            /* Python's min/max keep the constant when the other operand is NaN */
            if (en < 1.0) {
                double factor;
                if (en == 0.0) factor = 10.0;
                else {
                    factor = 0.9 * pow(en, -0.2);
                    if (!(factor < 10.0)) factor = 10.0;
                }
                if (rejected && !(factor < 1.0)) factor = 1.0;
                h_abs *= factor;
                break;
            } else {
                double factor = 0.9 * pow(en, -0.2);
                if (!(factor > 0.2)) factor = 0.2;
                h_abs *= factor;
                rejected = 1;
                ++*nrej;
            }
        }
        ++*nacc;
        t = t_new;
        for (int i = 0; i < n; ++i) { y[i] = yn[i]; f[i] = K[6][i]; }
        if (t - t_bound >= 0) return TTO_OK;
    }
}

/* Trace rays [0, nrays) of s0 (6 x np_total, SoA rows x,y,z,vx,vy,vz) from
 * t=0 to t_end.  Writes sf (same layout), phase (may be NULL), per-ray
 * accepted/rejected step and RHS-evaluation counts and a status code.
 * first/count select a slice so callers can split work across threads. */
int tto_trace(const double* dndx, const double* dndy, const double* dndz,
              const double* ne_nc, int nx, int ny, int nz,
              const double* x, const double* y, const double* z,
              double omega, const double* s0, int64_t np_total,
              int64_t first, int64_t count, double t_end,
              double rtol, double atol, int with_phase, int64_t max_steps,
              double* sf, double* phase, int64_t* nacc, int64_t* nrej,
              int64_t* nfev, int32_t* status)
{
    tto_cube C;
    C.G.n[0] = nx; C.G.n[1] = ny; C.G.n[2] = nz;
    C.G.g[0] = x; C.G.g[1] = y; C.G.g[2] = z;
    C.dndx = dndx; C.dndy = dndy; C.dndz = dndz; C.ne_nc = ne_nc;
    C.k0 = omega / TTO_C;
    C.neq = with_phase ? 7 : 6;
    for (int64_t r = first; r < first + count; ++r) {
        double st[7];
        for (int i = 0; i < 6; ++i) st[i] = s0[(size_t)i * np_total + r];
        st[6] = 0.0;
        int64_t a = 0, b = 0, c = 0;
        const int code = integrate_ray(&C, st, t_end, rtol, atol, max_steps, &a, &b, &c);
        for (int i = 0; i < 6; ++i) sf[(size_t)i * np_total + r] = st[i];
        if (phase) phase[r] = with_phase ? st[6] : 0.0;
        if (nacc) nacc[r] = a;
        if (nrej) nrej[r] = b;
        if (nfev) nfev[r] = c;
        if (status) status[r] = code;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Any explicit Runge-Kutta pair of scipy.integrate's RungeKutta family
 * (solve_ivp's method='RK23', 'RK45', 'DOP853'; particle_tracker.py:312, 323
 * passes `method` through): scipy's rk_step (stages K[s] = f(y + h sum_j
 * a[s][j] K[j]), y_new = y + h sum_j B[j] K[j], FSAL K[ns] = f(y_new)),
 * _estimate_error_norm (RMS of h K^T E / scale; DOP853: |h| |e5|^2 /
 * sqrt((|e5|^2 + 0.01 |e3|^2) n) with e = K^T E / scale), the step loop of
 * _step_impl (factor 0.9 err^(-1/(q+1)) in [0.2, 10], min(1, .) after a
 * rejection, TOO_SMALL below 10 spacings of t) and select_initial_step with
 * the error order q.  Per ray, as integrate_ray. */
typedef struct {
    int ns, kind, order;
    const double* A; /* ns x ns, row-major */
    const double* B; /* ns */
    const double* E; /* ns + 1 (E, or E5) */
    const double* E3;/* ns + 1, kind 1 */
} tto_rk;

#define TTO_RK_MAX 16

static double initial_step_q(const tto_cube* C, const double* y0, const double* f0,
                             double t_bound, double rtol, double atol, int order, int64_t* nfev)
{
    const int n = C->neq;
    double sc[7], tmp[7], y1[7], f1[7];
    const double L = fabs(t_bound);
    if (L == 0.0) return 0.0;
    for (int i = 0; i < n; ++i) sc[i] = atol + fabs(y0[i]) * rtol;
    for (int i = 0; i < n; ++i) tmp[i] = y0[i] / sc[i];
    const double d0 = rms(tmp, n);
    for (int i = 0; i < n; ++i) tmp[i] = f0[i] / sc[i];
    const double d1 = rms(tmp, n);
    double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
    if (h0 > L) h0 = L;
    for (int i = 0; i < n; ++i) y1[i] = y0[i] + h0 * f0[i];
    rhs(C, y1, f1);
    ++*nfev;
    for (int i = 0; i < n; ++i) tmp[i] = (f1[i] - f0[i]) / sc[i];
    const double d2 = rms(tmp, n) / h0;
    double h1;
    if (d1 <= 1e-15 && d2 <= 1e-15) {
        h1 = h0 * 1e-3;
        if (h1 < 1e-6) h1 = 1e-6;
    } else {
        const double m = d1 > d2 ? d1 : d2;
        h1 = pow(0.01 / m, 1.0 / (order + 1));
    }
    double h = 100.0 * h0;
    if (h1 < h) h = h1;
    if (L < h) h = L;
    return h;
}

static int integrate_ray_rk(const tto_cube* C, const tto_rk* T, double* y, double t_bound,
                            double rtol, double atol, int64_t max_steps,
                            int64_t* nacc, int64_t* nrej, int64_t* nfev)
{
    const int n = C->neq, ns = T->ns;
    const double ex = -1.0 / (T->order + 1);
    double f[7], K[TTO_RK_MAX + 1][7], yn[7], ys[7];
    rhs(C, y, f);
    *nfev = 1;
    *nacc = 0;
    *nrej = 0;
    double h_abs = initial_step_q(C, y, f, t_bound, rtol, atol, T->order, nfev);
    double t = 0.0;
    if (t == t_bound) return TTO_OK;
    for (;;) {
        const double min_step = 10.0 * fabs(nextafter(t, INFINITY) - t);
        if (h_abs < min_step) h_abs = min_step;
        int rejected = 0;
        double t_new, h;
        for (;;) {
            if (h_abs < min_step) return TTO_TOO_SMALL;
            if (*nacc + *nrej >= max_steps) return TTO_MAXSTEPS;
            h = h_abs;
            t_new = t + h;
            if (t_new - t_bound > 0) t_new = t_bound;
            h = t_new - t;
            h_abs = fabs(h);
            for (int i = 0; i < n; ++i) K[0][i] = f[i];
            for (int s = 1; s < ns; ++s) {
                for (int i = 0; i < n; ++i) {
                    double acc = 0.0;
                    for (int j = 0; j < s; ++j) acc += K[j][i] * T->A[s * ns + j];
                    ys[i] = y[i] + acc * h;
                }
                rhs(C, ys, K[s]);
            }
            for (int i = 0; i < n; ++i) {
                double acc = 0.0;
                for (int j = 0; j < ns; ++j) acc += K[j][i] * T->B[j];
                yn[i] = y[i] + h * acc;
            }
            rhs(C, yn, K[ns]);
            *nfev += ns;
            double e5 = 0.0, e3 = 0.0;
            for (int i = 0; i < n; ++i) {
                const double ay = fabs(y[i]), an = fabs(yn[i]);
                const double sc = atol + (ay > an ? ay : an) * rtol;
                double a5 = 0.0, a3 = 0.0;
                for (int j = 0; j <= ns; ++j) {
                    a5 += K[j][i] * T->E[j];
                    if (T->kind == 1) a3 += K[j][i] * T->E3[j];
                }
                if (T->kind == 1) {
                    e5 += (a5 / sc) * (a5 / sc);
                    e3 += (a3 / sc) * (a3 / sc);
                } else {
                    const double e = a5 * h / sc;
                    e5 += e * e;
                }
            }
            double en;
            if (T->kind == 1)
                en = (e5 == 0.0 && e3 == 0.0) ? 0.0 : fabs(h) * e5 / sqrt((e5 + 0.01 * e3) * n);
            else
                en = sqrt(e5) / sqrt((double)n);
            if (en < 1.0) {
                double factor;
                if (en == 0.0) factor = 10.0;
                else {
                    factor = 0.9 * pow(en, ex);
                    if (!(factor < 10.0)) factor = 10.0;
                }
                if (rejected && !(factor < 1.0)) factor = 1.0;
                h_abs *= factor;
                break;
            } else {
                double factor = 0.9 * pow(en, ex);
                if (!(factor > 0.2)) factor = 0.2;
                h_abs *= factor;
                rejected = 1;
                ++*nrej;
            }
        }
        ++*nacc;
        t = t_new;
        for (int i = 0; i < n; ++i) { y[i] = yn[i]; f[i] = K[ns][i]; }
        if (t - t_bound >= 0) return TTO_OK;
    }
}

/* tto_trace with the method's tableau (ns <= 16 stages). */
int tto_trace_rk(const double* dndx, const double* dndy, const double* dndz,
                 const double* ne_nc, int nx, int ny, int nz,
                 const double* x, const double* y, const double* z,
                 double omega, const double* s0, int64_t np_total,
                 int64_t first, int64_t count, double t_end,
                 double rtol, double atol, int with_phase, int64_t max_steps,
                 int ns, int kind, int order, const double* A, const double* B,
                 const double* E, const double* E3,
                 double* sf, double* phase, int64_t* nacc, int64_t* nrej,
                 int64_t* nfev, int32_t* status)
{
    if (ns < 1 || ns > TTO_RK_MAX) return -1;
    tto_cube C;
    C.G.n[0] = nx; C.G.n[1] = ny; C.G.n[2] = nz;
    C.G.g[0] = x; C.G.g[1] = y; C.G.g[2] = z;
    C.dndx = dndx; C.dndy = dndy; C.dndz = dndz; C.ne_nc = ne_nc;
    C.k0 = omega / TTO_C;
    C.neq = with_phase ? 7 : 6;
    tto_rk T = {ns, kind, order, A, B, E, E3};
    for (int64_t r = first; r < first + count; ++r) {
        double st[7];
        for (int i = 0; i < 6; ++i) st[i] = s0[(size_t)i * np_total + r];
        st[6] = 0.0;
        int64_t a = 0, b = 0, c = 0;
        const int code = integrate_ray_rk(&C, &T, st, t_end, rtol, atol, max_steps, &a, &b, &c);
        for (int i = 0; i < 6; ++i) sf[(size_t)i * np_total + r] = st[i];
        if (phase) phase[r] = with_phase ? st[6] : 0.0;
        if (nacc) nacc[r] = a;
        if (nrej) nrej[r] = b;
        if (nfev) nfev[r] = c;
        if (status) status[r] = code;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* numpy.histogram2d(x, y, bins=[nbx, nby], range=[[x0,x1],[y0,y1]]) followed by
 * the transpose at ray_transfer_matrix.py:188-191.  NaN samples are skipped
 * (the reference drops them at :185-186), samples outside the range are
 * dropped, the last bin of each axis is closed on the right.  Bin index is
 * found from the linspace edges (numpy computes edges with linspace and
 * corrects the fast index computation against them).  Output H is (nby, nbx)
 * counts, row-major; weights may be NULL (counts) or give weighted sums. */
void tto_histogram2d(const double* xs, const double* ys, const double* wts, int64_t n,
                     int nbx, int nby, double x0, double x1, double y0, double y1,
                     const double* xedges, const double* yedges, double* H)
{
    memset(H, 0, sizeof(double) * (size_t)nbx * nby);
    for (int64_t i = 0; i < n; ++i) {
        const double xv = xs[i], yv = ys[i];
        if (xv != xv || yv != yv) continue;
        if (xv < x0 || xv > x1 || yv < y0 || yv > y1) continue;
        /* searchsorted(edges, v, 'right') - 1, then the right edge maps to the last bin */
        int lo = 0, hi = nbx + 1;
        while (lo < hi) { int m = (lo + hi) >> 1; if (xedges[m] <= xv) lo = m + 1; else hi = m; }
        int bx = lo - 1;
        if (bx == nbx) bx = nbx - 1;
        lo = 0; hi = nby + 1;
        while (lo < hi) { int m = (lo + hi) >> 1; if (yedges[m] <= yv) lo = m + 1; else hi = m; }
        int by = lo - 1;
        if (by == nby) by = nby - 1;
        if (bx < 0 || by < 0) continue;
        H[(size_t)by * nbx + bx] += wts ? wts[i] : 1.0;
    }
}
