// Straight-line (unperturbed-ray) path integrals through a density grid: the
// inputs of the learned surrogate and the first-order (straight-line)
// deflection and phase that it corrects.
//
// For a ray entering at pixel centre (x_p, y_p) of a P x P grid over the box
// face and crossing the box along +z without bending:
//   out[0] = -1/2 * integral dq/dx dz      (paraxial deflection angle, rad)
//   out[1] = -1/2 * integral dq/dy dz
//   out[2] = k0 * integral (sqrt(1 - q) - 1) dz   (phase, rad; k0 = omega / c)
//   out[3] = -1/2 * integral (z - z0) / Lz dq/dx dz  (first moments along the path:
//   out[4] = -1/2 * integral (z - z0) / Lz dq/dy dz   where along z the deflection builds up)
// with q = min(ne / n_c, ne_max) and its gradient taken with numpy.gradient's
// rule on the node grid (central inside, one-sided at the faces), both
// interpolated trilinearly -- the same fields the tracer integrates.  The
// gradient integrals are exact for the trilinear interpolant (trapezoid on
// nodes); the phase uses 4-point Gauss-Legendre in every z cell.
#include "tt_common.cuh"

namespace {

template <typename T>
__device__ __forceinline__ float qval(const T* __restrict__ ne, int i, int j, int k, int ny, int nz, float inv_nc,
                                      float ne_max)
{
    const float q = (float)ne[((size_t)i * ny + j) * nz + k] * inv_nc;
    return q < ne_max ? q : ne_max;
}

// numpy.gradient along one axis at index i of n, unit spacing (the caller divides by h).
template <typename F>
__device__ __forceinline__ float grad1(F f, int i, int n)
{
    if (i == 0) return f(1) - f(0);
    if (i == n - 1) return f(n - 1) - f(n - 2);
    return 0.5f * (f(i + 1) - f(i - 1));
}

template <typename T>
__global__ void maps_kernel(const T* __restrict__ ne, int nx, int ny, int nz, double x0, double hx, double y0,
                            double hy, double hz, float inv_nc, float ne_max, double k0, int P, int nout,
                            float* __restrict__ out)
{
    const int n = P * P;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= n) return;
    const int pi = pix / P, pj = pix % P;
    const double xs = ((pi + 0.5) / P) * (hx * (nx - 1));
    const double ys = ((pj + 0.5) / P) * (hy * (ny - 1));
    int ix = (int)floor(xs / hx), iy = (int)floor(ys / hy);
    ix = ix < 0 ? 0 : (ix > nx - 2 ? nx - 2 : ix);
    iy = iy < 0 ? 0 : (iy > ny - 2 ? ny - 2 : iy);
    const float fx = (float)(xs / hx - ix), fy = (float)(ys / hy - iy);
    const float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w01 = (1.f - fx) * fy, w11 = fx * fy;
    double sx = 0.0, sy = 0.0, sp = 0.0, mx = 0.0, my = 0.0;
    float qprev = 0.f;
    const float gw[4] = {0.0694318442029737f, 0.3300094782075719f, 0.6699905217924281f, 0.9305681557970263f};
    const float gwt[4] = {0.1739274225687269f, 0.3260725774312731f, 0.3260725774312731f, 0.1739274225687269f};
    for (int k = 0; k < nz; ++k) {
        auto q = [&](int i, int j) { return qval(ne, i, j, k, ny, nz, inv_nc, ne_max); };
        const float gx0 = grad1([&](int i) { return q(i, iy); }, ix, nx);
        const float gx1 = grad1([&](int i) { return q(i, iy); }, ix + 1, nx);
        const float gx2 = grad1([&](int i) { return q(i, iy + 1); }, ix, nx);
        const float gx3 = grad1([&](int i) { return q(i, iy + 1); }, ix + 1, nx);
        const float gy0 = grad1([&](int j) { return q(ix, j); }, iy, ny);
        const float gy1 = grad1([&](int j) { return q(ix + 1, j); }, iy, ny);
        const float gy2 = grad1([&](int j) { return q(ix, j); }, iy + 1, ny);
        const float gy3 = grad1([&](int j) { return q(ix + 1, j); }, iy + 1, ny);
        const float gxk = w00 * gx0 + w10 * gx1 + w01 * gx2 + w11 * gx3;
        const float gyk = w00 * gy0 + w10 * gy1 + w01 * gy2 + w11 * gy3;
        const float qk = w00 * q(ix, iy) + w10 * q(ix + 1, iy) + w01 * q(ix, iy + 1) + w11 * q(ix + 1, iy + 1);
        const double wz = (k == 0 || k == nz - 1) ? 0.5 : 1.0;
        sx += wz * gxk;
        sy += wz * gyk;
        // first moment, trapezoid rule on the nodes
        const double zr = (double)k / (double)(nz - 1);
        mx += wz * zr * gxk;
        my += wz * zr * gyk;
        if (k > 0) {
            float cell = 0.f;
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const float qq = qprev + gw[g] * (qk - qprev);
                const float r = 1.f - qq;
                cell += gwt[g] * (sqrtf(r > 0.f ? r : 0.f) - 1.f);
            }
            sp += cell;
        }
        qprev = qk;
    }
    out[pix] = (float)(-0.5 * sx * hz / hx);
    out[n + pix] = (float)(-0.5 * sy * hz / hy);
    out[2 * n + pix] = (float)(k0 * sp * hz);
    if (nout > 3) {
        out[3 * n + pix] = (float)(-0.5 * mx * hz / hx);
        out[4 * n + pix] = (float)(-0.5 * my * hz / hy);
    }
}

}  // namespace

extern "C" int tt_straight_line_maps(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x,
                                     const double* y, const double* z, double lwl, double ne_max, int P, int nout,
                                     float* out, void* stream)
{
    if (nout != 3 && nout != 5) return tt::invalid("straight_line_maps: nout must be 3 or 5");
    if (!ne || !x || !y || !z || !out) return tt::invalid("straight_line_maps: NULL pointer");
    if (nx < 2 || ny < 2 || nz < 2 || P < 1) return tt::invalid("straight_line_maps: bad sizes");
    if (ne_dtype != TT_F32 && ne_dtype != TT_F64) return tt::invalid("straight_line_maps: ne_dtype");
    const double hx = (x[nx - 1] - x[0]) / (nx - 1), hy = (y[ny - 1] - y[0]) / (ny - 1),
                 hz = (z[nz - 1] - z[0]) / (nz - 1);
    if (!(hx > 0) || !(hy > 0) || !(hz > 0)) return tt::invalid("straight_line_maps: coordinates must increase");
    const double omega = 2.0 * CUDART_PI * (TT_C_LIGHT / lwl);
    const double nc = 3.14207787e-4 * omega * omega;
    const double k0 = omega / TT_C_LIGHT;
    const int n = P * P;
    const int grid = (n + 127) / 128;
    cudaStream_t s = tt::as_stream(stream);
    if (ne_dtype == TT_F32)
        maps_kernel<float><<<grid, 128, 0, s>>>((const float*)ne, nx, ny, nz, x[0], hx, y[0], hy, hz,
                                                (float)(1.0 / nc), (float)ne_max, k0, P, nout, out);
    else
        maps_kernel<double><<<grid, 128, 0, s>>>((const double*)ne, nx, ny, nz, x[0], hx, y[0], hy, hz,
                                                 (float)(1.0 / nc), (float)ne_max, k0, P, nout, out);
    return tt::launch_status("straight_line_maps");
}

// Geometric-optics shadowgram of a deflection map: rays leaving pixel centres
// of a P x P grid (pitch h) with angles theta = (tx, ty) land D further on at
// x + D theta; the intensity relative to the uniform beam is 1 / |det J| with
// J = I + D grad(theta) (central differences inside, one-sided at the edges),
// floored at |det J| >= 1e-3 near caustics.  div = dtx/dx + dty/dy.
namespace {

__device__ __forceinline__ float dmap(const float* __restrict__ f, int i, int j, int P, int axis)
{
    if (axis == 0) {
        if (i == 0) return f[P + j] - f[j];
        if (i == P - 1) return f[(size_t)(P - 1) * P + j] - f[(size_t)(P - 2) * P + j];
        return 0.5f * (f[(size_t)(i + 1) * P + j] - f[(size_t)(i - 1) * P + j]);
    }
    const float* r = f + (size_t)i * P;
    if (j == 0) return r[1] - r[0];
    if (j == P - 1) return r[P - 1] - r[P - 2];
    return 0.5f * (r[j + 1] - r[j - 1]);
}

__global__ void shadow_kernel(const float* __restrict__ theta, int P, float inv_h, float D, float* __restrict__ I,
                              float* __restrict__ div)
{
    const int n = P * P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int i = p / P, j = p % P;
    const float* tx = theta;
    const float* ty = theta + n;
    const float axx = dmap(tx, i, j, P, 0) * inv_h, axy = dmap(tx, i, j, P, 1) * inv_h;
    const float ayx = dmap(ty, i, j, P, 0) * inv_h, ayy = dmap(ty, i, j, P, 1) * inv_h;
    if (div) div[p] = axx + ayy;
    if (I) {
        const float det = (1.f + D * axx) * (1.f + D * ayy) - D * D * axy * ayx;
        const float a = fabsf(det);
        I[p] = 1.f / (a > 1e-3f ? a : 1e-3f);
    }
}

}  // namespace

extern "C" int tt_shadowgram(const float* theta, int P, double pitch, double D, float* intensity, float* div,
                             void* stream)
{
    if (!theta || P < 2 || !(pitch > 0)) return tt::invalid("shadowgram: bad arguments");
    if (!intensity && !div) return TT_OK;
    const int n = P * P;
    shadow_kernel<<<(n + 255) / 256, 256, 0, tt::as_stream(stream)>>>(theta, P, (float)(1.0 / pitch), (float)D,
                                                                       intensity, div);
    return tt::launch_status("shadowgram");
}
