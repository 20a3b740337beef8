// K2b: persistent FP32 tracer over brick-tiled node volumes (one, or a batch).
//
// Same ODE as ElectronCube.solve/dsdt/dndr (particle_tracking/particle_tracker.py:
// 243-256, 312-331, 398-419) in normalised variables:
//   P  = position in cells along (a, b, c), kept as integer cell + fraction,
//   u  = v / c,  sigma = c t / spacing_c (path parameter in cells of the probing axis),
//   dP/dsigma = r u   (r = spacing_c / spacing_axis),
//   du/dsigma = H(P)  (H = -0.5 d(ne_nc)/dx * spacing_c, trilinear in the cell),
//   dphi/dsigma = kappa (n - 1) |u|, n - 1 = -q / (1 + sqrt(1 - q)), kappa = k0 spacing_c.
// Each Dormand-Prince 5(4) step is aimed at the cell's next face (predicted
// from position, velocity and acceleration), so all seven stages evaluate one
// cell's trilinear polynomial (8 float4 nodes loaded once) and the kinks of
// the interpolant sit at step ends.  A stage that leaves the cell is looked up
// exactly (neighbour cell, or the fill value 0 beyond the box, as
// RegularGridInterpolator's fill_value=0), and a step that runs too far past
// a face is redone ending at the crossing.  Outside the box the ray is a
// straight line, finished analytically.  Error control per ray (scipy's
// controller constants) on position (cells), direction and phase.  Path
// length and phase are compensated sums (the phase optionally an FP64 sum:
// one double add per accepted step, the stage arithmetic staying FP32).  The interpolant and the stage
// combinations of the two transverse components run as packed FP32x2 FMAs
// (__ffma2_rn: per lane the same rounding as fmaf, so results are unchanged).
//
// Work distribution: rays are bucketed by (instance, the 4x4-cell tile they
// start in) -- the volume's own tile order -- then a persistent grid of
// resident blocks pulls them through one global work counter; each warp
// refills its finished lanes with one warp-aggregated atomic (ballot / popc),
// so lanes stay busy while rays with long and short paths mix.  In the batched
// forms each lane finds its ray's instance once per ray: volumes of one shape
// share the single-volume kernel's constant geometry and differ only in node
// buffer and ray block; volumes of mixed shapes read per-lane geometry.
#include <math.h>
#include <stddef.h>

#include <atomic>

#include "tt_common.cuh"

namespace {

__device__ __host__ inline uint32_t spread3(uint32_t v)
{
    return (v & 1u) | ((v & 2u) << 1) | ((v & 4u) << 2);
}

// Dormand-Prince 5(4) (Dormand & Prince 1980; scipy's RK45 tableau) as
// compile-time functions: after the stage loops unroll every coefficient is an
// immediate operand (kernel-parameter constants cost the packed FP32x2 FMAs a
// register move each; immediates measured 7% faster).  Row 6 of A is B.  The
// step loop also uses the products AA = A A (stage positions from the stored
// accelerations) and EA = E A (the position error), formed here in double and
// rounded to float once, as the scalar tableau would be.
//
// The step loop skips the terms whose weight is zero in exact arithmetic:
// b[1] = e[1] = 0 (stage 1's rates enter neither the new state nor the error
// estimate, so its phase rate is not formed), AA[s][k] = 0 for k >= s - 1 (A
// is strictly lower triangular: a stage's position waits only for the
// accelerations up to two stages back), AA[6][1] = (B A)[1] = 0 and EA[1] = 0.
__host__ __device__ constexpr double dp_a(int s, int k)
{
    return s == 1 ? (k == 0 ? 1.0 / 5 : 0.0)
         : s == 2 ? (k == 0 ? 3.0 / 40 : k == 1 ? 9.0 / 40 : 0.0)
         : s == 3 ? (k == 0 ? 44.0 / 45 : k == 1 ? -56.0 / 15 : k == 2 ? 32.0 / 9 : 0.0)
         : s == 4 ? (k == 0 ? 19372.0 / 6561 : k == 1 ? -25360.0 / 2187 : k == 2 ? 64448.0 / 6561
                   : k == 3 ? -212.0 / 729 : 0.0)
         : s == 5 ? (k == 0 ? 9017.0 / 3168 : k == 1 ? -355.0 / 33 : k == 2 ? 46732.0 / 5247
                   : k == 3 ? 49.0 / 176 : k == 4 ? -5103.0 / 18656 : 0.0)
         : s == 6 ? (k == 0 ? 35.0 / 384 : k == 2 ? 500.0 / 1113 : k == 3 ? 125.0 / 192
                   : k == 4 ? -2187.0 / 6784 : k == 5 ? 11.0 / 84 : 0.0)
         : 0.0;
}

__host__ __device__ constexpr double dp_e(int k)
{
    return k == 0 ? -71.0 / 57600 : k == 2 ? 71.0 / 16695 : k == 3 ? -71.0 / 1920
         : k == 4 ? 17253.0 / 339200 : k == 5 ? -22.0 / 525 : k == 6 ? 1.0 / 40 : 0.0;
}

__host__ __device__ constexpr double dp_c(int s)
{
    return s == 0 ? 0.0 : s == 1 ? 1.0 / 5 : s == 2 ? 3.0 / 10 : s == 3 ? 4.0 / 5 : s == 4 ? 8.0 / 9 : 1.0;
}

__host__ __device__ constexpr double dp_aa(int s, int k)
{
    double acc = 0.0;
    for (int j = 0; j < 6; ++j) acc += dp_a(s, j) * dp_a(j, k);
    return acc;
}

__host__ __device__ constexpr double dp_ea(int k)
{
    double acc = 0.0;
    for (int j = 0; j < 7; ++j) acc += dp_e(j) * dp_a(j, k);
    return acc;
}

// the float coefficients the step loop uses
__host__ __device__ constexpr float fa(int s, int k) { return (float)dp_a(s, k); }
__host__ __device__ constexpr float faa(int s, int k) { return (float)dp_aa(s, k); }
__host__ __device__ constexpr float fc(int s) { return (float)dp_c(s); }
__host__ __device__ constexpr float fe(int k) { return (float)dp_e(k); }
__host__ __device__ constexpr float fea(int k) { return (float)dp_ea(k); }

// exactly zero for k >= s - 1; AA[6][1] and EA[1] are zero in exact arithmetic
// and within a few ulps of zero in double (the skipped FMA adds below 1e-15 of an
// acceleration, far under FP32's rounding)
static_assert(dp_aa(3, 2) == 0.0 && dp_aa(6, 5) == 0.0, "A A is zero for k >= s - 1");
static_assert(dp_aa(6, 1) < 1e-15 && dp_aa(6, 1) > -1e-15 && dp_ea(1) < 1e-15 && dp_ea(1) > -1e-15,
              "A A [6][1] and E A [1] vanish");

// Resident tracer threads per SM the register budget is sized for (the
// launch bounds give each thread 65536 / kThreadsPerSM registers).
#ifndef TT_TRACE32_THREADS_PER_SM
#define TT_TRACE32_THREADS_PER_SM 512
#endif
constexpr int kThreadsPerSM = TT_TRACE32_THREADS_PER_SM;

// Geometry of one volume instance.
struct Geo {
    const float4* nodes;
    long long tile_f4;    // float4 per tile column
    long long ray_begin;  // first ray of this instance (its arrays are the blocks starting there)
    long long nrays;      // rays of this instance
    double origin[3];
    double spacing[3];
    double inv_spacing[3];
    double sig_end;
    double extent;
    int n[3];
    int axis[3];
    int st_b;
    int bd;               // nodes per brick along c
    int bd_shift;
    int brick_f4;         // float4 per brick (25 bd)
    int bin_base;         // first bucket of this instance
    float r[3];
    float kappa;
    float sig_end_f;      // sig_end in FP32 for the step loop (no FP64 in the hot loop)
};

// Controls shared by every instance.
struct Ctl {
    float rtol, inv_rtol, inv_atol_cells, atol_phase;
    int with_phase;
    int phase_f64;  // accumulate the phase in FP64 (else a Neumaier-compensated FP32 pair)
    int chunk;  // rays a warp takes from the work counter at a time (>= 32)
    int refill;  // a warp takes new rays once at least this many lanes are idle (1..32)
    long long max_steps;
};

// Instance table, passed by value as a kernel parameter (so the launch can be
// captured in a CUDA graph without any host-to-device copy).
struct GeoTable {
    int n;
    Geo g[TT_MAX_INSTANCES];
};
static_assert(sizeof(GeoTable) < 30000, "instance table must fit in the kernel parameter space");

__device__ __forceinline__ long long tile_base(const Geo& G, int ta, int tb)
{
    const int sa = ta >> 3, sb = tb >> 3;
    const uint32_t m = spread3((uint32_t)(ta & 7)) | (spread3((uint32_t)(tb & 7)) << 1);
    return ((long long)(sa * G.st_b + sb) * 64 + m) * G.tile_f4;
}

__device__ __forceinline__ int tile_key(const Geo& G, int ta, int tb)
{
    const int sa = ta >> 3, sb = tb >> 3;
    const uint32_t m = spread3((uint32_t)(ta & 7)) | (spread3((uint32_t)(tb & 7)) << 1);
    return (sa * G.st_b + sb) * 64 + (int)m;
}

// The trilinear polynomial of two components at once (packed FP32x2):
//   c0 + fc c3 + fb (c2 + fc c6) + fa ((c1 + fc c5) + fb (c4 + fc c7)).
__device__ __forceinline__ float2 tri2(const float2* c, float fa, float fb, float fc)
{
    const float2 A = make_float2(fa, fa), Bv = make_float2(fb, fb), Cv = make_float2(fc, fc);
    const float2 t1 = __ffma2_rn(c[7], Cv, c[4]);
    const float2 t2 = __ffma2_rn(c[5], Cv, c[1]);
    const float2 t3 = __ffma2_rn(Bv, t1, t2);
    const float2 t4 = __ffma2_rn(c[6], Cv, c[2]);
    const float2 t5 = __ffma2_rn(c[3], Cv, c[0]);
    const float2 t6 = __ffma2_rn(Bv, t4, t5);
    return __ffma2_rn(A, t3, t6);
}

// a - b lane-wise, rounded as the scalar subtraction (fma(b, -1, a) is exact up to its one rounding)
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}

// Polynomial coefficients of the trilinear interpolant of two components at
// once (packed FP32x2; lane-wise the scalar differences
//   c0 = v000, c1 = v100 - v000, c2 = v010 - v000, c3 = v001 - v000,
//   c4 = (v110 - v100) - c2, c5 = (v101 - v100) - c3, c6 = (v011 - v010) - c3,
//   c7 = ((v111 - v110) - (v101 - v100)) - c6).
__device__ __forceinline__ void poly2(float2 v000, float2 v001, float2 v010, float2 v011, float2 v100, float2 v101,
                                      float2 v110, float2 v111, float2* c)
{
    c[0] = v000;
    c[1] = sub2(v100, v000);
    c[2] = sub2(v010, v000);
    c[3] = sub2(v001, v000);
    const float2 d101 = sub2(v101, v100);
    c[4] = sub2(sub2(v110, v100), c[2]);
    c[5] = sub2(d101, c[3]);
    c[6] = sub2(sub2(v011, v010), c[3]);
    c[7] = sub2(sub2(sub2(v111, v110), d101), c[6]);
}

__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// One component's polynomial, as one lane of poly2 / tri2 (the same rounding).
__device__ __forceinline__ void poly1(float v000, float v001, float v010, float v011, float v100, float v101,
                                      float v110, float v111, float* c)
{
    c[0] = v000;
    c[1] = __fsub_rn(v100, v000);
    c[2] = __fsub_rn(v010, v000);
    c[3] = __fsub_rn(v001, v000);
    const float d101 = __fsub_rn(v101, v100);
    c[4] = __fsub_rn(__fsub_rn(v110, v100), c[2]);
    c[5] = __fsub_rn(d101, c[3]);
    c[6] = __fsub_rn(__fsub_rn(v011, v010), c[3]);
    c[7] = __fsub_rn(__fsub_rn(__fsub_rn(v111, v110), d101), c[6]);
}
__device__ __forceinline__ float tri1(const float* c, float fa, float fb, float fc)
{
    const float t1 = fmaf(c[7], fc, c[4]);
    const float t2 = fmaf(c[5], fc, c[1]);
    const float t3 = fmaf(fb, t1, t2);
    const float t4 = fmaf(c[6], fc, c[2]);
    const float t5 = fmaf(c[3], fc, c[0]);
    const float t6 = fmaf(fb, t4, t5);
    return fmaf(fa, t3, t6);
}

// The cell's trilinear polynomials: (H_a, H_b) packed, and (H_c, q) packed
// when the phase is integrated; without the phase H_c alone (8 registers fewer).
template <int PHASE>
struct CellPoly {
    float2 ab[8];
    float2 cq[8];
};
template <>
struct CellPoly<0> {
    float2 ab[8];
    float c[8];
};

template <int PHASE>
__device__ __forceinline__ void cell_eval(const CellPoly<PHASE>& cp, float fa, float fb, float fc, float H[3],
                                          float& q)
{
    const float2 hab = tri2(cp.ab, fa, fb, fc);
    H[0] = hab.x;
    H[1] = hab.y;
    if constexpr (PHASE == 0) {
        H[2] = tri1(cp.c, fa, fb, fc);
        q = 0.f;
    } else {
        const float2 hcq = tri2(cp.cq, fa, fb, fc);
        H[2] = hcq.x;
        q = hcq.y;
    }
}

template <int PHASE>
__device__ __forceinline__ void load_cell(const Geo& G, const float4* __restrict__ nodes, long long tbase, int ca,
                                          int cb, int cc, CellPoly<PHASE>& cp)
{
    const int cl = cc & (G.bd - 1);
    const int dc = (cl == G.bd - 1) ? G.brick_f4 - (G.bd - 1) : 1;
    const long long base = tbase + (long long)(cc >> G.bd_shift) * G.brick_f4 + ((ca & 3) * 5 + (cb & 3)) * G.bd + cl;
    const float4* p = nodes + base;
    const int db = G.bd, da = 5 * G.bd;
    const float4 n000 = __ldg(p), n001 = __ldg(p + dc);
    const float4 n010 = __ldg(p + db), n011 = __ldg(p + db + dc);
    const float4 n100 = __ldg(p + da), n101 = __ldg(p + da + dc);
    const float4 n110 = __ldg(p + da + db), n111 = __ldg(p + da + db + dc);
    poly2(lo2(n000), lo2(n001), lo2(n010), lo2(n011), lo2(n100), lo2(n101), lo2(n110), lo2(n111), cp.ab);
    if constexpr (PHASE == 0)
        poly1(n000.z, n001.z, n010.z, n011.z, n100.z, n101.z, n110.z, n111.z, cp.c);
    else
        poly2(hi2(n000), hi2(n001), hi2(n010), hi2(n011), hi2(n100), hi2(n101), hi2(n110), hi2(n111), cp.cq);
}

// Square roots and reciprocals of the phase rate and the face prediction as the
// hardware's approximate instructions (sqrt.approx, rcp.approx: about 2^-22
// relative, the same class as rsqrtf and __fdividef, with fewer instructions
// around them; 8% faster together).
__device__ __forceinline__ float sqrt_apx(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_apx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float nm1f(float q)
{
    const float r = 1.0f - q;
    return -q * rcp_apx(1.0f + sqrt_apx(r > 0.0f ? r : 0.0f));
}

// Smallest h > 0 with v h + acc h^2 / 2 = d (d >= 0, moving from 0 toward d).
__device__ __forceinline__ float first_hit(float v, float acc, float d)
{
    if (!(d > 0.f)) return 3.0e38f;
    const float disc = fmaf(v, v, 2.f * acc * d);
    if (disc < 0.f) return 3.0e38f;
    const float den = v + sqrt_apx(disc);  // predictor only: approximate is fine
    return den > 0.f ? 2.f * d * rcp_apx(den) : 3.0e38f;
}

// Neumaier summation s + x with running compensation c (no contraction).
__device__ __forceinline__ void neumaier(float& s, float& c, float x)
{
    const float t = __fadd_rn(s, x);
    if (fabsf(s) >= fabsf(x)) c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, t), x));
    else c = __fadd_rn(c, __fadd_rn(__fsub_rn(x, t), s));
    s = t;
}

struct Ray {
    int ci[3];
    float fr[3];
    float u[3];
    float sig, sigc;
    float uc[3];     // compensation of u (Kahan)
    float ph, phc;   // phase: Neumaier pair, or (FP64 accumulation) the two words of one double
    float hctrl;
    float hcap;    // one-shot cap on the next attempt after a face-crossing rejection
    int natt, nacc;
    int state;     // 0 = stepping, 1 = exited box, 2 = reached sigma_end, 3 = failed
    int code;
    bool rejected;
    bool cell_dirty;
    int ta, tb;
    long long tbase;
};

// The FP64 phase accumulator kept in the registers of the (ph, phc) pair.
__device__ __forceinline__ double ph_get(const Ray& R)
{
    return __hiloint2double(__float_as_int(R.ph), __float_as_int(R.phc));
}

__device__ __forceinline__ void ph_set(Ray& R, double v)
{
    R.ph = __int_as_float(__double2hiint(v));
    R.phc = __int_as_float(__double2loint(v));
}

// Interior faces: a stage may use the current cell's polynomial up to kTolE
// cells past a face, and a step may run at most kFacePath (path, in cells) past
// the face it crosses; so a kink of the interpolant always sits within
// kFacePath of a step end.  Box faces (where the field jumps to the fill value
// 0): no extrapolation and at most kBoxPath of path past the face.
constexpr float kTolE = 1e-3f;
constexpr float kFacePath = 1e-3f;
constexpr float kBoxPath = 1e-6f;


// Exact lookup (RegularGridInterpolator semantics, fill 0 outside) at cell
// ci + floor(P), used when a stage leaves the current cell.  Scalars in,
// float4 {H_a, H_b, H_c, q} out, so the caller's stage arrays stay in registers.
__device__ __noinline__ float4 eval_exact(const float4* __restrict__ nodes, int n0, int n1, int n2, int st_b,
                                          long long tile_f4, int bd, int bd_shift, int brick_f4, int c0, int c1,
                                          int c2, float p0, float p1, float p2)
{
    const int n[3] = {n0, n1, n2};
    int c[3] = {c0, c1, c2};
    const float P[3] = {p0, p1, p2};
    float f[3];
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float fl = floorf(P[a]);
        c[a] += (int)fl;
        f[a] = P[a] - fl;
        if (c[a] == n[a] - 1 && f[a] == 0.f) {
            c[a] = n[a] - 2;
            f[a] = 1.f;
        }
        out = out || c[a] < 0 || c[a] > n[a] - 2;
    }
    if (out) return make_float4(0.f, 0.f, 0.f, 0.f);
    const int ta = c[0] >> 2, tb = c[1] >> 2;
    const uint32_t m = spread3((uint32_t)(ta & 7)) | (spread3((uint32_t)(tb & 7)) << 1);
    const long long tbase = ((long long)((ta >> 3) * st_b + (tb >> 3)) * 64 + m) * tile_f4;
    const int cl = c[2] & (bd - 1);
    const int dc = (cl == bd - 1) ? brick_f4 - (bd - 1) : 1;
    const long long base = tbase + (long long)(c[2] >> bd_shift) * brick_f4 + ((c[0] & 3) * 5 + (c[1] & 3)) * bd + cl;
    const float4* p = nodes + base;
    const int db = bd, da = 5 * bd;
    const float4 n000 = __ldg(p), n001 = __ldg(p + dc);
    const float4 n010 = __ldg(p + db), n011 = __ldg(p + db + dc);
    const float4 n100 = __ldg(p + da), n101 = __ldg(p + da + dc);
    const float4 n110 = __ldg(p + da + db), n111 = __ldg(p + da + db + dc);
    const float fa = f[0], fb = f[1], fc = f[2];
#define TT_LERP3(C)                                                                                  \
    fmaf(fa, fmaf(fb, fmaf(fc, n111.C - n110.C, n110.C) - fmaf(fc, n101.C - n100.C, n100.C),         \
                  fmaf(fc, n101.C - n100.C, n100.C)) -                                                \
             fmaf(fb, fmaf(fc, n011.C - n010.C, n010.C) - fmaf(fc, n001.C - n000.C, n000.C),          \
                  fmaf(fc, n001.C - n000.C, n000.C)),                                                 \
         fmaf(fb, fmaf(fc, n011.C - n010.C, n010.C) - fmaf(fc, n001.C - n000.C, n000.C),              \
              fmaf(fc, n001.C - n000.C, n000.C)))
    const float4 r = make_float4(TT_LERP3(x), TT_LERP3(y), TT_LERP3(z), TT_LERP3(w));
#undef TT_LERP3
    return r;
}

// Normalise after an accepted step: P = ci + fr, fr in [0, 1), a ray within
// kTolE of an interior face and moving through it is assigned to the cell it
// enters; the upper box face belongs to the last cell.  Returns true when the
// ray is outside the box.
__device__ __forceinline__ bool renormalise(const Geo& G, Ray& R)
{
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float fl = floorf(R.fr[a]);
        int c = R.ci[a] + (int)fl;
        float f = R.fr[a] - fl;
        if (c == G.n[a] - 1 && f == 0.f) {
            c = G.n[a] - 2;
            f = 1.f;
        }
        // pre-assign only when the face is within kFacePath of path ahead, so a
        // slow (grazing) ray never runs far on the next cell's polynomial
        const float vel = G.r[a] * R.u[a];
        if (vel > 0.f && 1.f - f < fminf(kTolE, kFacePath * vel) && c < G.n[a] - 2) {
            c += 1;
            f -= 1.f;
        } else if (vel < 0.f && f < fminf(kTolE, -kFacePath * vel) && c > 0) {
            c -= 1;
            f += 1.f;
        }
        if (c != R.ci[a]) R.cell_dirty = true;
        R.ci[a] = c;
        R.fr[a] = f;
        out = out || c < 0 || c > G.n[a] - 2;
    }
    return out;
}

// Initialise from s0 (SI units, physical axes).  Returns false when the ray
// never enters the box before t_end (straight line throughout).
// The rays of one volume: node buffer and its block of the instance-blocked arrays.
struct Src {
    const float4* nodes;
    long long begin, count;
};

__device__ __forceinline__ bool init_ray(const Geo& G, const Src& src, const double* __restrict__ s0, long long np,
                                         long long r, Ray& R, double P[3], double uu[3])
{
    // instance-blocked arrays: this instance's s0 is (6, nrays) at 6 * ray_begin
    const double* s = s0 + 6 * src.begin;
    const long long lr = r - src.begin, ln = src.count;
    double x[3], v[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        x[i] = s[(size_t)i * ln + lr];
        v[i] = s[(size_t)(3 + i) * ln + lr];
    }
    bool finite = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        P[a] = (x[G.axis[a]] - G.origin[a]) * G.inv_spacing[a];  // FP64 multiply, no divide
        // a start on a box face (up to the rounding of this transform) is on it,
        // as RegularGridInterpolator counts the end coordinates as inside
        const double hi = (double)(G.n[a] - 1);
        if (fabs(P[a]) < 1e-9) P[a] = 0.0;
        if (fabs(P[a] - hi) < 1e-9 * hi) P[a] = hi;
        uu[a] = v[G.axis[a]] * (1.0 / TT_C_LIGHT);
        finite = finite && isfinite(P[a]) && isfinite(uu[a]);
    }
    R.natt = R.nacc = 0;
    R.sig = R.sigc = 0.f;
    R.ph = R.phc = 0.f;
    R.uc[0] = R.uc[1] = R.uc[2] = 0.f;
    R.hctrl = 1.0f;
    R.hcap = 3.0e38f;
    R.rejected = false;
    R.code = TT_RAY_OK;
    if (!finite) {
        R.code = TT_RAY_NAN;
        R.state = 3;
        return false;
    }
    // slab test in sigma units (dP/dsigma = r u), FP32: rays that start inside
    // get tin = 0 exactly; for the others it places the entry point
    float tin = 0.f, tout = G.sig_end_f;
    int enter_axis = -1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float vel = G.r[a] * (float)uu[a];
        const float hi = (float)(G.n[a] - 1);
        const float pa = (float)P[a];
        if (vel == 0.f) {
            if (P[a] < 0.0 || P[a] > (double)(G.n[a] - 1)) tout = -1.f;
        } else {
            const float iv = 1.f / vel;
            float t1 = (0.f - pa) * iv, t2 = (hi - pa) * iv;
            if (t1 > t2) { const float t = t1; t1 = t2; t2 = t; }
            if (t1 > tin) { tin = t1; enter_axis = a; }
            if (t2 < tout) tout = t2;
        }
    }
    if (!(tin <= tout) || tin >= G.sig_end_f) {
        R.state = 1;  // never inside: straight line
        R.sig = 0.f;
        return false;
    }
    double Pe[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) Pe[a] = fma((double)G.r[a] * uu[a], (double)tin, P[a]);
    if (enter_axis >= 0) Pe[enter_axis] = uu[enter_axis] > 0.0 ? 0.0 : (double)(G.n[enter_axis] - 1);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double c = floor(Pe[a]);
        if (c > G.n[a] - 2) c = G.n[a] - 2;
        if (c < 0) c = 0;
        R.ci[a] = (int)c;
        R.fr[a] = (float)(Pe[a] - c);
        R.u[a] = (float)uu[a];
    }
    R.sig = tin;
    R.sigc = 0.f;
    R.state = 0;
    R.cell_dirty = true;
    R.ta = -1;
    R.tb = -1;
    return true;
}

// ENTERED: the ray stepped inside the box (its state is in R); otherwise it
// never met the box and P0, u0 hold its start (a separate instantiation, so a
// stepping ray keeps no start state live across the step loop).
template <bool ENTERED>
__device__ __forceinline__ void finish_ray(const Geo& G, const Src& src, const Ray& R, const double* P0,
                                           const double* u0, long long r, long long np, double* __restrict__ sf,
                                           double* __restrict__ rf, double* __restrict__ phase,
                                           int* __restrict__ status, int* __restrict__ nsteps, bool ph64)
{
    // Position/velocity where stepping stopped, then the straight-line flight to
    // t_end for rays outside the box (zero field there): rays that left the box,
    // and rays that never meet it (whole interval).
    double P[3], u[3], ds = 0.0;
    if (ENTERED) {
        const double sig = (double)R.sig + (double)R.sigc;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            P[a] = (double)R.ci[a] + (double)R.fr[a];
            u[a] = (double)R.u[a] - (double)R.uc[a];
        }
        if (R.state == 1 && R.code == TT_RAY_OK) ds = G.sig_end - sig > 0.0 ? G.sig_end - sig : 0.0;
    } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            P[a] = P0[a];
            u[a] = u0[a];
        }
        if (R.code == TT_RAY_OK) ds = G.sig_end;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) P[a] += (double)G.r[a] * u[a] * ds;
    double y[6];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        y[G.axis[a]] = G.origin[a] + P[a] * G.spacing[a];
        y[3 + G.axis[a]] = u[a] * TT_C_LIGHT;
    }
    const long long lr = r - src.begin, ln = src.count;
    if (sf) {
        double* o = sf + 6 * src.begin;
#pragma unroll
        for (int i = 0; i < 6; ++i) o[(size_t)i * ln + lr] = y[i];
    }
    if (rf) {
        double* o = rf + 4 * src.begin;
        const int ax = G.axis[2];
        const int p0 = ax == 0 ? 1 : 0, p1 = ax == 2 ? 1 : 2;
        const double tbp = (y[ax] - G.extent) / y[3 + ax];
        o[lr] = y[p0] - y[3 + p0] * tbp;
        o[(size_t)2 * ln + lr] = y[p1] - y[3 + p1] * tbp;
        // angles from the FP32 direction the ray carries (relative error ~1e-7 of the angle)
        const float uc = (float)u[2];
        o[(size_t)ln + lr] = (double)atanf((float)y[3 + p0] * (1.f / 299792458.f) / uc);
        o[(size_t)3 * ln + lr] = (double)atanf((float)y[3 + p1] * (1.f / 299792458.f) / uc);
    }
    if (phase) phase[r] = ph64 ? ph_get(R) : (double)R.ph + (double)R.phc;
    if (status) status[r] = R.code;
    if (nsteps) nsteps[r] = R.nacc;
}

// Right-hand side at stage position Ps (fractions in the current cell):
// the current cell's polynomial while Ps stays within kTolE of it (never past
// a box face), the exact lookup otherwise.
template <int PHASE>
__device__ __forceinline__ void stage_eval(const Geo& G, const float4* __restrict__ nodes, const Ctl& K, const Ray& R,
                                           const CellPoly<PHASE>& cp, const float Ps[3], float H[3], float& q,
                                           const float* lo, const float* hi)
{
    bool home = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) home = home && Ps[a] >= lo[a] && Ps[a] <= hi[a];
    // the polynomial first, on every path: the rare branch to the exact
    // lookup then only overrides it, and the common path is one block
    cell_eval<PHASE>(cp, Ps[0], Ps[1], Ps[2], H, q);
    if (!home) {
        const float4 r = eval_exact(nodes, G.n[0], G.n[1], G.n[2], G.st_b, G.tile_f4, G.bd, G.bd_shift,
                                    G.brick_f4, R.ci[0], R.ci[1], R.ci[2], Ps[0], Ps[1], Ps[2]);
        H[0] = r.x;
        H[1] = r.y;
        H[2] = r.z;
        q = r.w;
    }
}

// One attempted step.  Returns with R updated.  PHASE is a template parameter:
// 0 no phase, 1 the phase integrated as a seventh equation and summed in a
// compensated FP32 pair, 2 the same summed in FP64.  As run-time flags they
// put branches in every stage and step, which split the unrolled stage loop
// into blocks the compiler schedules separately (5.7% and 2.1% slower).
template <int PHASE>
__device__ __forceinline__ void step(const Geo& G, const float4* __restrict__ nodes, const Ctl& K, Ray& R,
                                     CellPoly<PHASE>& coef)
{
    if (R.cell_dirty) {
        const int ta = R.ci[0] >> 2, tb = R.ci[1] >> 2;
        if (ta != R.ta || tb != R.tb) {
            R.ta = ta;
            R.tb = tb;
            R.tbase = tile_base(G, ta, tb);
        }
        load_cell(G, nodes, R.tbase, R.ci[0], R.ci[1], R.ci[2], coef);
        R.cell_dirty = false;
    }
    const float rem = (G.sig_end_f - R.sig) - R.sigc;
    if (!(rem > 0.f) || R.natt >= K.max_steps) {  // at t_end, or out of attempts
        if (rem > 0.f) R.code = TT_RAY_MAX_STEPS;
        R.state = rem > 0.f ? 3 : 2;
        return;
    }
    float Hs[7][3];
    float q0;
    {  // stage 0 is at the ray's own position, always inside the current cell's range
        cell_eval<PHASE>(coef, R.fr[0], R.fr[1], R.fr[2], Hs[0], q0);
    }
    // Predict the first face crossing of the cell from position, velocity and
    // acceleration; aim the step end at it.  Leaving through a box face within
    // kBoxPath: the ray has left (the field beyond is the fill value 0).
    float hf = 3.0e38f;
    bool leave = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float vel = G.r[a] * R.u[a];
        const float acc = G.r[a] * Hs[0][a];
        // the face ahead is reached first if the ray gets there before it
        // turns back; otherwise the face behind (the same root as the
        // smaller of the two face times)
        const bool up = vel >= 0.f;
        float v1 = up ? vel : -vel, a1 = up ? acc : -acc;
        float d1 = up ? 1.f - R.fr[a] : R.fr[a];
        if (!(d1 > 0.f) || fmaf(v1, v1, 2.f * a1 * d1) < 0.f) {
            v1 = -v1;
            a1 = -a1;
            d1 = up ? R.fr[a] : 1.f - R.fr[a];
        }
        const float hfa = first_hit(v1, a1, d1);
        const bool box_up = R.ci[a] == G.n[a] - 2, box_lo = R.ci[a] == 0;
        leave = leave || (box_up && vel > 0.f && (1.f - R.fr[a]) <= kBoxPath * vel) ||
                (box_lo && vel < 0.f && R.fr[a] <= -kBoxPath * vel);
        hf = fminf(hf, hfa);
    }
    if (leave) {  // within kBoxPath of a box face it is moving through: it has left
        R.state = 1;
        return;
    }
    ++R.natt;
    bool last = false;
    float h = fminf(fminf(R.hctrl, R.hcap), hf);
    R.hcap = 3.0e38f;
    if (h >= rem) {
        h = rem;
        last = true;
    }
    float phb = 0.f, phe = 0.f;
    float Pn[3], un[3], inc6[3];
    if (PHASE) {
        const float u2 = fmaf(R.u[0], R.u[0], fmaf(R.u[1], R.u[1], R.u[2] * R.u[2]));
        const float sp = sqrt_apx(u2);
        const float dph = G.kappa * nm1f(q0) * sp;
        phb = fa(6, 0) * dph;
        phe = fe(0) * dph;
    }
    // The cell's in-cell bounds for the stage tests (no tolerance at a box
    // face), formed once per step: left to stage_eval, the compare-and-select
    // was rebuilt in every stage (5% of the step's time).
    float blo[3], bhi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        blo[a] = R.ci[a] == 0 ? 0.f : -kTolE;
        bhi[a] = R.ci[a] == G.n[a] - 2 ? 1.f : 1.f + kTolE;
    }
    const float2 h2 = make_float2(h, h);
    const float2 hr2 = make_float2(h * G.r[0], h * G.r[1]);
    const float2 u2v = make_float2(R.u[0], R.u[1]);
    const float2 fr2 = make_float2(R.fr[0], R.fr[1]);
#pragma unroll
    for (int s = 1; s < 7; ++s) {
        float Ps[3], us[3];
        {  // transverse pair (components 0, 1): packed FP32x2, lane-wise the scalar arithmetic below
            float2 sa = make_float2(0.f, 0.f), saa = make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < s && k < 6; ++k) {
                const float2 hk = make_float2(Hs[k][0], Hs[k][1]);
                if (!(s == 6 && k == 1)) sa = __ffma2_rn(make_float2(fa(s, k), fa(s, k)), hk, sa);
                if (k + 1 < s && !(s == 6 && k == 1)) saa = __ffma2_rn(make_float2(faa(s, k), faa(s, k)), hk, saa);
            }
            const float2 uu = __ffma2_rn(h2, sa, u2v);
            const float2 pp = __ffma2_rn(hr2, __ffma2_rn(make_float2(fc(s), fc(s)), u2v, __fmul2_rn(h2, saa)), fr2);
            us[0] = uu.x;
            us[1] = uu.y;
            if (s == 6) {
                inc6[0] = sa.x;
                inc6[1] = sa.y;
            }
            Ps[0] = pp.x;
            Ps[1] = pp.y;
        }
        {
            const int c = 2;
            float sa = 0.f, saa = 0.f;
#pragma unroll
            for (int k = 0; k < s && k < 6; ++k) {
                if (!(s == 6 && k == 1)) sa = fmaf(fa(s, k), Hs[k][c], sa);
                if (k + 1 < s && !(s == 6 && k == 1)) saa = fmaf(faa(s, k), Hs[k][c], saa);
            }
            us[c] = fmaf(h, sa, R.u[c]);
            if (s == 6) inc6[c] = sa;
            Ps[c] = fmaf(h * G.r[c], fmaf(fc(s), R.u[c], h * saa), R.fr[c]);
        }
        float q;
        stage_eval<PHASE>(G, nodes, K, R, coef, Ps, Hs[s], q, blo, bhi);
        // Dormand-Prince's b and e weights of stage 1 are zero: its phase rate
        // is not needed (the sums are unchanged: an FMA with weight 0 adds an exact 0)
        if (PHASE && s != 1) {
            const float u2 = fmaf(us[0], us[0], fmaf(us[1], us[1], us[2] * us[2]));
            const float sp = sqrt_apx(u2);
            const float dph = G.kappa * nm1f(q) * sp;
            if (s < 6) phb = fmaf(fa(6, s), dph, phb);
            phe = fmaf(fe(s), dph, phe);
        }
        if (s == 6) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                Pn[c] = Ps[c];
                un[c] = us[c];
            }
        }
    }
    // error estimate; velocity scale is rtol times the speed (|u| ~ 1), so the
    // velocity tolerance is an angle
    const float q0u = fmaf(R.u[0], R.u[0], fmaf(R.u[1], R.u[1], R.u[2] * R.u[2]));
    const float q1u = fmaf(un[0], un[0], fmaf(un[1], un[1], un[2] * un[2]));
    const float inv_scu = rsqrtf(fmaxf(q0u, q1u)) * K.inv_rtol;  // 1 / (rtol |u|)
    float eus[3], eps[3];
    {  // the error sums of the transverse pair packed (lane-wise the scalar FMAs)
        float2 eu2 = make_float2(0.f, 0.f), ep2 = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 7; ++k)
            if (k != 1) eu2 = __ffma2_rn(make_float2(fe(k), fe(k)), make_float2(Hs[k][0], Hs[k][1]), eu2);
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (k != 1) ep2 = __ffma2_rn(make_float2(fea(k), fea(k)), make_float2(Hs[k][0], Hs[k][1]), ep2);
        eus[0] = eu2.x; eus[1] = eu2.y; eps[0] = ep2.x; eps[1] = ep2.y;
        float eu = 0.f, ep = 0.f;
#pragma unroll
        for (int k = 0; k < 7; ++k)
            if (k != 1) eu = fmaf(fe(k), Hs[k][2], eu);
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (k != 1) ep = fmaf(fea(k), Hs[k][2], ep);
        eus[2] = eu; eps[2] = ep;
    }
    float es = 0.f;
    const float hs = h * inv_scu, hp = h * h * K.inv_atol_cells;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float x1 = eus[c] * hs;
        const float x2 = eps[c] * (hp * G.r[c]);
        es = fmaf(x1, x1, fmaf(x2, x2, es));
    }
    int neq = 6;
    float dphi = 0.f;
    if (PHASE) {
        dphi = h * phb;
        const float phv = (PHASE == 2) ? (float)ph_get(R) : R.ph;
        const float phn = phv + dphi;
        const float scp = K.atol_phase + K.rtol * fmaxf(fabsf(phv), fabsf(phn));
        const float x = __fdividef(h * phe, scp);
        es = fmaf(x, x, es);
        neq = 7;
    }
    // the squared RMS error norm: the controller's en^-1/5 is (en^2)^-1/10
    const float en2 = es * (neq == 7 ? (1.f / 7.f) : (1.f / 6.f));
    // Where did the step cross a face?  If it ran too far past one, redo it
    // ending at the crossing (estimated backwards from the end point).
    float hre = 3.0e38f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float vend = G.r[a] * un[a];
        // path past the crossed face, without branches
        const bool xu = Pn[a] > 1.f && R.fr[a] <= 1.f;
        const bool xl = !xu && Pn[a] < 0.f && R.fr[a] >= 0.f;
        const float num = xu ? Pn[a] - 1.f : -Pn[a];
        const float den = fmaxf(xu ? vend : -vend, 1e-6f);
        const float over = (xu || xl) ? __fdividef(num, den) : 0.f;
        const bool box = xu ? R.ci[a] == G.n[a] - 2 : (xl && R.ci[a] == 0);
        float hn = h - 1.01f * over;
        if (!(hn > 0.1f * h)) hn = 0.5f * h;
        hre = over > (box ? kBoxPath : kFacePath) ? fminf(hre, hn) : hre;
    }
    // one branch off the accepted path: a NaN, then a rejected error, then a
    // face-crossing retry, in that order
    if (!(en2 < 1.0f) || hre < 3.0e38f) {
        if (!(en2 == en2)) {
            R.code = TT_RAY_NAN;
            R.state = 3;
        } else if (en2 >= 1.0f) {
            const float factor = fmaxf(0.2f, 0.9f * __powf(en2, -0.1f));
            R.hctrl = h * factor;
            R.rejected = true;
            if (R.hctrl < 1e-7f) {
                R.code = TT_RAY_STEP_TOO_SMALL;
                R.state = 3;
            }
        } else {
            R.hcap = hre;  // controller state untouched: this was a geometric retry
        }
        return;
    }
    float factor = en2 == 0.f ? 10.f : fminf(10.f, 0.9f * __powf(en2, -0.1f));
    if (R.rejected) factor = fminf(1.f, factor);
    R.rejected = false;
    R.hctrl = h * factor;
    ++R.nacc;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        R.fr[c] = Pn[c];
        // u is a compensated sum of the accepted increments h (b . H): FP32
        // rounding of u itself, ~6e-8 per step, would otherwise random-walk
        // to ~1e-6 rad over a few hundred strongly deflecting steps
        const float y = fmaf(h, inc6[c], -R.uc[c]);
        const float t = __fadd_rn(R.u[c], y);
        R.uc[c] = __fsub_rn(__fsub_rn(t, R.u[c]), y);
        R.u[c] = t;
    }
    {  // Kahan on sigma
        const float y = __fsub_rn(h, R.sigc);
        const float t = __fadd_rn(R.sig, y);
        R.sigc = __fsub_rn(__fsub_rn(t, R.sig), y);
        R.sig = t;
    }
    if (PHASE) {
        if (PHASE == 2) ph_set(R, ph_get(R) + (double)dphi);
        else neumaier(R.ph, R.phc, dphi);
    }
    if (renormalise(G, R)) R.state = 1;
    else if (last) R.state = 2;
}

// Instance of ray r: the last instance whose ray_begin <= r.
__device__ __forceinline__ int instance_of(const Geo* g, int n, long long r)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g[mid].ray_begin <= r) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The persistent loop, shared by the single-volume and batched kernels.
// GeoOf(r) returns the geometry of ray r's instance.
// The persistent loop, shared by the single-volume and batched kernels.  The
// policy gives, for ray r: the geometry of its volume (geo), and its ray
// block (src: node buffer and the block of the instance-blocked arrays).  It
// is asked once per fetched ray; the node pointer is kept for the ray's steps
// unless the policy has it as a constant (pol.nodes).
template <int PHASE, typename Policy>
__device__ __forceinline__ void persistent_loop(Policy pol, const Ctl& K, const double* __restrict__ s0,
                                                long long np, const unsigned* __restrict__ perm,
                                                unsigned long long* __restrict__ counter, double* __restrict__ sf,
                                                double* __restrict__ rf, double* __restrict__ phase,
                                                int* __restrict__ status, int* __restrict__ nsteps)
{
    // perm positions and ray indices fit in 32 bits (the host keeps np <= 2^32 - 2^16)
    const unsigned lane = threadIdx.x & 31u;
    const unsigned n32 = (unsigned)np;
    bool busy = false;        // this lane holds a ray
    unsigned ray = 0;
    bool drained = false;
    unsigned wnext = 0, wend = 0;  // the warp's chunk of perm positions (warp-uniform)
    const float4* nodes = nullptr;
    Ray R;
    CellPoly<PHASE> coef;
    R.state = 1;
    for (;;) {
        const bool need = !busy && !drained;
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        // refill once K.refill lanes are idle (or none is busy): with 32, a
        // warp's lanes trace 32 neighbouring rays together to the end
        if (mask && (K.refill <= 1 || __popc(mask) >= K.refill || __ballot_sync(0xffffffffu, busy) == 0u)) {
            // lanes are refilled from the warp's chunk of consecutive bucketed
            // rays; a new chunk comes from the shared work counter.  (Larger
            // chunks, and per-block segments with stealing, both measured slower.)
            const unsigned cnt = __popc(mask);
            const unsigned avail = wend - wnext;
            unsigned nb = 0, ne = 0;
            if (avail < cnt) {
                const int leader = __ffs(mask) - 1;
                if ((int)lane == leader) {
                    nb = ne = n32;
                    const unsigned long long got = atomicAdd(counter, (unsigned long long)K.chunk);
                    if (got < n32) {
                        nb = (unsigned)got;
                        ne = (unsigned)(got + K.chunk < n32 ? got + K.chunk : n32);
                    }
                }
                nb = __shfl_sync(0xffffffffu, nb, leader);
                ne = __shfl_sync(0xffffffffu, ne, leader);
            }
            if (need) {
                const unsigned rank = __popc(mask & ((1u << lane) - 1u));
                bool got = rank < avail;
                unsigned my = wnext + rank;
                if (!got) {
                    my = nb + (rank - avail);
                    got = my < ne;
                }
                if (got) {
                    ray = perm ? perm[my] : my;
                    busy = true;
                    const Src src = pol.src(ray);
                    nodes = src.nodes;
                    double P0[3], u0[3];
                    if (!init_ray(pol.geo(ray), src, s0, np, ray, R, P0, u0)) {
                        finish_ray<false>(pol.geo(ray), src, R, P0, u0, ray, np, sf, rf, phase, status, nsteps,
                                          PHASE == 2);
                        busy = false;  // picked up again on the next pass
                    }
                } else if (nb == ne) {
                    drained = true;  // no ray left anywhere
                }
            }
            if (avail < cnt) {
                const unsigned take = cnt - avail < ne - nb ? cnt - avail : ne - nb;
                wnext = nb + take;
                wend = ne;
            } else {
                wnext += cnt;
            }
            // only a refill can leave the warp with nothing to do: every lane
            // is then busy or drained (a lane whose ray missed the box is
            // neither, and takes another on the next pass)
            if (__ballot_sync(0xffffffffu, busy || (!drained)) == 0u) break;
        }
        if (busy) {
            step<PHASE>(pol.geo(ray), pol.nodes(nodes), K, R, coef);
            if (R.state != 0) {
                finish_ray<true>(pol.geo(ray), pol.src(ray), R, nullptr, nullptr, ray, np, sf, rf, phase, status,
                                 nsteps, PHASE == 2);
                busy = false;
            }
        }
    }
}

struct SinglePolicy {
    const Geo* g;
    __device__ __forceinline__ const Geo& geo(long long) const { return *g; }
    __device__ __forceinline__ Src src(long long) const { return Src{g->nodes, g->ray_begin, g->nrays}; }
    __device__ __forceinline__ const float4* nodes(const float4*) const { return g->nodes; }
};

template <int BLOCK, int PHASE>
__global__ void __launch_bounds__(BLOCK, kThreadsPerSM / BLOCK)
trace32_kernel(const Geo G, Ctl K, const double* __restrict__ s0, long long np,
               const unsigned* __restrict__ perm, unsigned long long* __restrict__ counter,
               double* __restrict__ sf, double* __restrict__ rf, double* __restrict__ phase,
               int* __restrict__ status, int* __restrict__ nsteps)
{
    persistent_loop<PHASE>(SinglePolicy{&G}, K, s0, np, perm, counter, sf, rf, phase, status, nsteps);
}

// Volumes of different shapes: each lane reads its ray's instance entry from
// the table, which stays in the parameter bank (__grid_constant__); the lane
// keeps a pointer to the entry of its current ray.  (A shared-memory copy of
// the table measured 3-8% slower.)
struct MixedPolicy {
    const Geo* g;
    int n;
    mutable const Geo* cur;
    // The lane's entry: src() is asked first for every ray the lane picks up
    // and moves cur to that ray's instance, so geo() needs no test.
    __device__ __forceinline__ const Geo& geo(long long) const { return *cur; }
    __device__ __forceinline__ Src src(long long r) const
    {
        // rays reach a lane in bucket order, which is instance-major, so the
        // lane's previous instance nearly always owns the next ray too
        if (r < cur->ray_begin || r - cur->ray_begin >= cur->nrays) cur = g + instance_of(g, n, r);
        return Src{cur->nodes, cur->ray_begin, cur->nrays};
    }
    __device__ __forceinline__ const float4* nodes(const float4* kept) const { return kept; }
};

template <int BLOCK, int PHASE>
__global__ void __launch_bounds__(BLOCK, kThreadsPerSM / BLOCK)
trace32_batched_kernel(const __grid_constant__ GeoTable table, Ctl K, const double* __restrict__ s0, long long np,
                       const unsigned* __restrict__ perm, unsigned long long* __restrict__ counter,
                       double* __restrict__ sf, double* __restrict__ rf, double* __restrict__ phase,
                       int* __restrict__ status, int* __restrict__ nsteps)
{
    persistent_loop<PHASE>(MixedPolicy{table.g, table.n, table.g}, K, s0, np, perm, counter, sf, rf, phase, status,
                           nsteps);
}

// Volumes of one shape (grid, spacing, brick depth, t_end): the geometry is
// the first entry, read from the constant bank like the single-volume kernel;
// only the node buffer and the ray block differ per instance.
struct UniformPolicy {
    const Geo* g;
    int n;
    __device__ __forceinline__ const Geo& geo(long long) const { return g[0]; }
    // asked twice per ray (start, finish): a search of the table, so that no
    // per-lane instance state stays live across the step loop
    __device__ __forceinline__ Src src(long long r) const
    {
        const Geo& e = g[instance_of(g, n, r)];
        return Src{e.nodes, e.ray_begin, e.nrays};
    }
    __device__ __forceinline__ const float4* nodes(const float4* kept) const { return kept; }
};

template <int BLOCK, int PHASE>
__global__ void __launch_bounds__(BLOCK, kThreadsPerSM / BLOCK)
trace32_uniform_kernel(const __grid_constant__ GeoTable table, Ctl K, const double* __restrict__ s0,
                       long long np, const unsigned* __restrict__ perm, unsigned long long* __restrict__ counter,
                       double* __restrict__ sf, double* __restrict__ rf, double* __restrict__ phase,
                       int* __restrict__ status, int* __restrict__ nsteps)
{
    persistent_loop<PHASE>(UniformPolicy{table.g, table.n}, K, s0, np, perm, counter, sf, rf, phase, status, nsteps);
}

// --- ray bucketing by (instance, entry tile) ----------------------------------
__device__ __forceinline__ int ray_key(const Geo& G, const double* __restrict__ s0, long long np, long long r)
{
    const double* s = s0 + 6 * G.ray_begin;
    const long long lr = r - G.ray_begin, ln = G.nrays;
    const double xa = s[(size_t)G.axis[0] * ln + lr];
    const double xb = s[(size_t)G.axis[1] * ln + lr];
    double pa = (xa - G.origin[0]) * G.inv_spacing[0];
    double pb = (xb - G.origin[1]) * G.inv_spacing[1];
    if (!(pa >= 0.0)) pa = 0.0;  // NaN too
    if (!(pb >= 0.0)) pb = 0.0;
    int ca = pa > (double)(G.n[0] - 2) ? G.n[0] - 2 : (int)pa;
    int cb = pb > (double)(G.n[1] - 2) ? G.n[1] - 2 : (int)pb;
    return G.bin_base + tile_key(G, ca >> 2, cb >> 2);
}

__global__ void bin_count_kernel(const GeoTable table, const double* __restrict__ s0, long long np,
                                 unsigned* __restrict__ cnt)
{
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < np;
         r += (long long)gridDim.x * blockDim.x) {
        const int key = ray_key(table.g[instance_of(table.g, table.n, r)], s0, np, r);
        const unsigned peers = __match_any_sync(__activemask(), key);
        const int leader = __ffs(peers) - 1;
        if ((int)(threadIdx.x & 31u) == leader) atomicAdd(cnt + key, (unsigned)__popc(peers));
    }
}

// exclusive scan of n counters by one block (n up to a few hundred thousand)
__global__ void bin_scan_kernel(unsigned* __restrict__ cnt, int n)
{
    __shared__ unsigned part[1024];
    const int t = threadIdx.x;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int lo = t * per, hi = min(n, lo + per);
    unsigned s = 0;
    for (int i = lo; i < hi; ++i) s += cnt[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        const unsigned v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned run = part[t] - s;
    for (int i = lo; i < hi; ++i) {
        const unsigned c = cnt[i];
        cnt[i] = run;
        run += c;
    }
}

__global__ void bin_scatter_kernel(const GeoTable table, const double* __restrict__ s0, long long np,
                                   unsigned* __restrict__ cursor, unsigned* __restrict__ perm)
{
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < np;
         r += (long long)gridDim.x * blockDim.x) {
        const int key = ray_key(table.g[instance_of(table.g, table.n, r)], s0, np, r);
        const unsigned peers = __match_any_sync(__activemask(), key);
        const int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if ((int)(threadIdx.x & 31u) == leader) base = atomicAdd(cursor + key, (unsigned)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        const unsigned rank = __popc(peers & ((1u << (threadIdx.x & 31u)) - 1u));
        perm[base + rank] = (unsigned)r;
    }
}

// ---------------------------------------------------------------------------
// Host side
int make_geo(const tt_volume* vol, double t_end, double extent, long long ray_begin, long long nrays, int bin_base,
             Geo* out)
{
    if (!vol->nodes) return tt::invalid("trace_f32: volume has no node buffer");
    for (int i = 0; i < 3; ++i)
        if (vol->n[i] < 2) return tt::invalid("trace_f32: volume axis with < 2 nodes");
    const int bd = vol->brick_depth;
    if (bd < 4 || bd > 32 || (bd & (bd - 1)) != 0) return tt::invalid("trace_f32: bad brick_depth");
    if (!(t_end >= 0.0)) return tt::invalid("trace_f32: t_end must be >= 0");
    Geo G;
    G.nodes = static_cast<const float4*>(vol->nodes);
    for (int i = 0; i < 3; ++i) {
        G.n[i] = vol->n[i];
        G.origin[i] = vol->origin[i];
        G.spacing[i] = vol->spacing[i];
        G.inv_spacing[i] = 1.0 / vol->spacing[i];
        G.axis[i] = vol->axis[i];
        G.r[i] = (float)(vol->spacing[2] / vol->spacing[i]);
    }
    G.st_b = vol->supertiles[1];
    G.bd = bd;
    G.bd_shift = __builtin_ctz((unsigned)bd);
    G.brick_f4 = 25 * bd;
    G.tile_f4 = (long long)vol->bricks_c * G.brick_f4;
    if ((long long)vol->supertiles[0] * vol->supertiles[1] * 64 * G.tile_f4 != vol->n_float4)
        return tt::invalid("trace_f32: volume descriptor is inconsistent (use tt_volume_plan)");
    G.kappa = (float)(vol->omega / TT_C_LIGHT * vol->spacing[2]);
    G.sig_end = t_end * TT_C_LIGHT / vol->spacing[2];
    G.sig_end_f = (float)G.sig_end;
    G.extent = extent;
    G.ray_begin = ray_begin;
    G.nrays = nrays;
    G.bin_base = bin_base;
    *out = G;
    return TT_OK;
}

int make_ctl(const tt_trace_opts* opts, Ctl* K)
{
    if (!(opts->rtol > 0.0) || !(opts->atol > 0.0))
        return tt::invalid("trace_f32: need rtol > 0 and atol > 0 (cells)");
    if (opts->with_phase && !(opts->atol_phase > 0.0)) return tt::invalid("trace_f32: need atol_phase > 0");
    const int bs = opts->block_size;
    if (bs != 0 && bs != 64 && bs != 128 && bs != 256)
        return tt::invalid("trace_f32: block_size must be 64, 128 or 256");
    K->rtol = (float)opts->rtol;
    K->inv_rtol = (float)(1.0 / opts->rtol);
    K->inv_atol_cells = (float)(1.0 / opts->atol);
    K->atol_phase = (float)(opts->with_phase ? opts->atol_phase : 1.0);
    K->with_phase = opts->with_phase ? 1 : 0;
    K->phase_f64 = (opts->with_phase && opts->phase_f64) ? 1 : 0;
    K->max_steps = opts->max_steps > 0 ? opts->max_steps : TT_DEFAULT_MAX_STEPS;
    const int ch = opts->ray_chunk;
    if (ch != 0 && (ch < 32 || ch > 1024 || ch % 32))
        return tt::invalid("trace_f32: ray_chunk must be 0 or 32..1024, a multiple of 32");
    K->chunk = ch ? ch : 32;  // 32 measured fastest
    const int rl = opts->refill_lanes;
    if (rl < 0 || rl > 32) return tt::invalid("trace_f32: refill_lanes must be 0..32");
    K->refill = rl ? rl : 2;  // 2 measured fastest for single traces (0.8% at 512^3 over 1)
    return TT_OK;
}

int vol_bins(const tt_volume* vol) { return vol->supertiles[0] * vol->supertiles[1] * 64; }

struct WsLayout {
    size_t counter_off, cnt_off, perm_off, total;
    int nbins;
};

WsLayout ws_layout(int nbins, long long np)
{
    WsLayout L;
    L.nbins = nbins;
    L.counter_off = 0;
    L.cnt_off = 256;
    L.perm_off = tt::align_up(L.cnt_off + sizeof(unsigned) * (size_t)nbins, 256);
    L.total = tt::align_up(L.perm_off + sizeof(unsigned) * (size_t)np, 256);
    return L;
}

template <typename KernelT>
int occupancy_grid(KernelT kernel, int block, int slot)
{
    // per-(kernel, device) cache; threads may race to fill an entry, all with the same value
    static std::atomic<int> cache[27][64];
    int dev = 0;
    cudaGetDevice(&dev);
    int b = (dev >= 0 && dev < 64) ? cache[slot][dev].load(std::memory_order_relaxed) : 0;
    if (b <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, block, 0) != cudaSuccess || b < 1) b = 1;
        if (dev >= 0 && dev < 64) cache[slot][dev].store(b, std::memory_order_relaxed);
    }
    return b * tt::sm_count();
}


int bin_grid(long long np)
{
    long long g = (np + 255) / 256;
    const long long cap = (long long)tt::sm_count() * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// True when every instance has instance 0's shape: the fields the uniform
// batched kernel reads from entry 0 agree exactly.
bool same_shape(const GeoTable& t)
{
    const Geo& a = t.g[0];
    for (int i = 1; i < t.n; ++i) {
        const Geo& b = t.g[i];
        bool eq = a.tile_f4 == b.tile_f4 && a.sig_end == b.sig_end && a.extent == b.extent && a.st_b == b.st_b &&
                  a.bd == b.bd && a.bd_shift == b.bd_shift && a.brick_f4 == b.brick_f4 && a.kappa == b.kappa &&
                  a.sig_end_f == b.sig_end_f;
        for (int k = 0; k < 3; ++k)
            eq = eq && a.origin[k] == b.origin[k] && a.spacing[k] == b.spacing[k] &&
                 a.inv_spacing[k] == b.inv_spacing[k] && a.n[k] == b.n[k] && a.axis[k] == b.axis[k] && a.r[k] == b.r[k];
        if (!eq) return false;
    }
    return true;
}

// Bucket, then trace.  table.n == 1 runs the single-volume kernel, a batch of
// one shape the uniform kernel, a batch of mixed shapes the mixed kernel.
int run(const GeoTable& table, int nbins, const Ctl& K, int block, const double* s0, long long np, double* sf,
        double* rf, double* phase, int* status, int* nsteps, void* workspace, size_t workspace_bytes,
        cudaStream_t s, const char* who)
{
    const WsLayout L = ws_layout(nbins, np);
    if (!workspace || workspace_bytes < L.total) {
        tt::set_detail("%s: workspace needs %zu bytes", who, L.total);
        return TT_ERR_WORKSPACE_TOO_SMALL;
    }
    char* ws = static_cast<char*>(workspace);
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(ws + L.counter_off);
    unsigned* cnt = reinterpret_cast<unsigned*>(ws + L.cnt_off);
    unsigned* perm = reinterpret_cast<unsigned*>(ws + L.perm_off);
    TT_TRY(tt::cuda_status(cudaMemsetAsync(ws, 0, L.perm_off, s), "trace_f32 workspace clear"));
    bin_count_kernel<<<bin_grid(np), 256, 0, s>>>(table, s0, np, cnt);
    bin_scan_kernel<<<1, 1024, 0, s>>>(cnt, nbins);
    bin_scatter_kernel<<<bin_grid(np), 256, 0, s>>>(table, s0, np, cnt, perm);
    TT_TRY(tt::launch_status("trace_f32 ray binning"));
    const Ctl& Kc = K;
#define TT_LAUNCH_ONE(KERNEL, ARGS, BS, SLOT)                                                         \
    do {                                                                                              \
        if (Kc.with_phase && Kc.phase_f64)                                                            \
            KERNEL<BS, 2><<<occupancy_grid(KERNEL<BS, 2>, BS, (SLOT) + 18), BS, 0, s>>> ARGS;         \
        else if (Kc.with_phase)                                                                       \
            KERNEL<BS, 1><<<occupancy_grid(KERNEL<BS, 1>, BS, (SLOT) + 9), BS, 0, s>>> ARGS;          \
        else                                                                                          \
            KERNEL<BS, 0><<<occupancy_grid(KERNEL<BS, 0>, BS, SLOT), BS, 0, s>>> ARGS;                \
    } while (0)
#define TT_LAUNCH_SINGLE(BS, SLOT) \
    TT_LAUNCH_ONE(trace32_kernel, (table.g[0], Kc, s0, np, perm, counter, sf, rf, phase, status, nsteps), BS, SLOT)
#define TT_LAUNCH_BATCH(BS, SLOT)                                                                         \
    TT_LAUNCH_ONE(trace32_batched_kernel, (table, Kc, s0, np, perm, counter, sf, rf, phase, status, nsteps), BS, \
                  SLOT)
#define TT_LAUNCH_UNIFORM(BS, SLOT)                                                                       \
    TT_LAUNCH_ONE(trace32_uniform_kernel, (table, Kc, s0, np, perm, counter, sf, rf, phase, status, nsteps), BS, \
                  SLOT)
    // block 0 = 256 (measured fastest on the 256^3 and 512^3 workloads)
    if (table.n == 1) {
        if (block == 64) TT_LAUNCH_SINGLE(64, 0);
        else if (block == 128) TT_LAUNCH_SINGLE(128, 1);
        else TT_LAUNCH_SINGLE(256, 2);
    } else if (same_shape(table)) {
        if (block == 64) TT_LAUNCH_UNIFORM(64, 6);
        else if (block == 128) TT_LAUNCH_UNIFORM(128, 7);
        else TT_LAUNCH_UNIFORM(256, 8);
    } else {
        if (block == 64) TT_LAUNCH_BATCH(64, 3);
        else if (block == 128) TT_LAUNCH_BATCH(128, 4);
        else TT_LAUNCH_BATCH(256, 5);
    }
#undef TT_LAUNCH_SINGLE
#undef TT_LAUNCH_BATCH
#undef TT_LAUNCH_UNIFORM
#undef TT_LAUNCH_ONE
    return tt::launch_status("trace_f32 kernel");
}

GeoTable& host_table()
{
    static thread_local GeoTable t;
    return t;
}

}  // namespace

extern "C" size_t tt_trace_f32_workspace_bytes(const tt_volume* vol, int64_t np)
{
    if (!vol || np < 0) return 0;
    return ws_layout(vol_bins(vol), np).total;
}

extern "C" int tt_trace_f32(const tt_volume* vol, const double* s0, int64_t np, double t_end, double extent,
                            const tt_trace_opts* opts, double* sf, double* rf, double* phase, int32_t* status,
                            int32_t* nsteps, void* workspace, size_t workspace_bytes, void* stream)
{
    if (!vol || !opts) return tt::invalid("trace_f32: null volume or opts");
    if (np < 0) return tt::invalid("trace_f32: np < 0");
    if (np > 0xffff0000LL) return tt::invalid("trace_f32: at most 2^32 - 2^16 rays per call");
    GeoTable& H = host_table();
    H.n = 1;
    TT_TRY(make_geo(vol, t_end, extent, 0, np, 0, &H.g[0]));
    Ctl K;
    TT_TRY(make_ctl(opts, &K));
    if (np == 0) return TT_OK;
    if (!s0) return tt::invalid("trace_f32: s0 is null");
    return run(H, vol_bins(vol), K, opts->block_size, s0, np, sf, rf, phase, status, nsteps, workspace,
               workspace_bytes, tt::as_stream(stream), "trace_f32");
}

extern "C" size_t tt_trace_f32_batched_workspace_bytes(const tt_volume* vols, int ninst, int64_t ntot)
{
    if (!vols || ninst < 1 || ninst > TT_MAX_INSTANCES || ntot < 0) return 0;
    int nb = 0;
    for (int i = 0; i < ninst; ++i) nb += vol_bins(&vols[i]);
    return ws_layout(nb, ntot).total;
}

extern "C" int tt_trace_f32_batched(const tt_volume* vols, int ninst, const int64_t* ray_offsets,
                                    const double* t_end, const double* extent, const double* s0,
                                    const tt_trace_opts* opts, double* sf, double* rf, double* phase,
                                    int32_t* status, int32_t* nsteps, void* workspace, size_t workspace_bytes,
                                    void* stream)
{
    if (!vols || !opts || !ray_offsets || !t_end || !extent) return tt::invalid("trace_f32_batched: null argument");
    if (ninst < 1 || ninst > TT_MAX_INSTANCES) return tt::invalid("trace_f32_batched: 1..TT_MAX_INSTANCES instances");
    if (ray_offsets[0] != 0) return tt::invalid("trace_f32_batched: ray_offsets[0] must be 0");
    for (int i = 0; i < ninst; ++i)
        if (ray_offsets[i + 1] < ray_offsets[i]) return tt::invalid("trace_f32_batched: ray_offsets must not decrease");
    const long long np = ray_offsets[ninst];
    if (np > 0xffff0000LL) return tt::invalid("trace_f32_batched: at most 2^32 - 2^16 rays per call");
    Ctl K;
    TT_TRY(make_ctl(opts, &K));
    GeoTable& H = host_table();
    H.n = ninst;
    int nb = 0;
    for (int i = 0; i < ninst; ++i) {
        TT_TRY(make_geo(&vols[i], t_end[i], extent[i], ray_offsets[i], ray_offsets[i + 1] - ray_offsets[i], nb,
                        &H.g[i]));
        nb += vol_bins(&vols[i]);
    }
    if (np == 0) return TT_OK;
    if (!s0) return tt::invalid("trace_f32_batched: s0 is null");
    // an empty instance owns no ray: instance_of() picks the last instance
    // starting at or before a ray, which is never an empty one
    return run(H, nb, K, opts->block_size, s0, np, sf, rf, phase, status, nsteps, workspace, workspace_bytes,
               tt::as_stream(stream), "trace_f32_batched");
}
