// Straight-line (unperturbed-ray) path integrals through a density grid: the
// inputs of the learned surrogate and the first-order (straight-line)
// deflection and phase that it corrects.
//
// For a ray entering at pixel centre (x_p, y_p) of a P x P grid over the box
// face and crossing the box along +z without bending:
//   out[0] = -1/2 * integral dq/dx dz      (paraxial deflection angle, rad)
//   out[1] = -1/2 * integral dq/dy dz
//   out[2] = k0 * integral (sqrt(1 - q) - 1) dz   (phase, rad; k0 = omega / c)
//   out[3 + 2s], out[4 + 2s] = the two deflection integrals over slab s of nslab
//   equal slabs of cells along z (where along the path the deflection builds up)
// with q = min(ne / n_c, ne_max) and its gradient taken with numpy.gradient's
// rule on the node grid (central inside, one-sided at the faces), both
// interpolated trilinearly -- the same fields the tracer integrates.  The
// gradient integrals are exact for the trilinear interpolant (trapezoid on
// nodes); the phase uses 4-point Gauss-Legendre in every z cell.
#include "tt_common.cuh"

namespace {

constexpr int kMaxSlab = 8;

// One warp per pixel: lane l handles nodes k = l, l + 32, ... along z, so
// the column reads (z is the fastest axis of the density) are coalesced; the
// per-lane sums are combined with shuffles.
template <typename T>
__global__ void maps_kernel(const T* __restrict__ ne, int nx, int ny, int nz, double hx, double hy, double hz,
                            float inv_nc, float ne_max, double k0, int P, int nslab, float* __restrict__ out)
{
    const int n = P * P;
    const int warp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int pi = warp / P, pj = warp % P;
    const double xs = ((pi + 0.5) / P) * (hx * (nx - 1));
    const double ys = ((pj + 0.5) / P) * (hy * (ny - 1));
    int ix = (int)floor(xs / hx), iy = (int)floor(ys / hy);
    ix = ix < 0 ? 0 : (ix > nx - 2 ? nx - 2 : ix);
    iy = iy < 0 ? 0 : (iy > ny - 2 ? ny - 2 : iy);
    const float fx = (float)(xs / hx - ix), fy = (float)(ys / hy - iy);
    const float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w01 = (1.f - fx) * fy, w11 = fx * fy;
    const float gw[4] = {0.0694318442029737f, 0.3300094782075719f, 0.6699905217924281f, 0.9305681557970263f};
    const float gwt[4] = {0.1739274225687269f, 0.3260725774312731f, 0.3260725774312731f, 0.1739274225687269f};
    // columns: x neighbours ix-1..ix+2 at rows iy, iy+1; y neighbours iy-1..iy+2 at columns ix, ix+1
    const int xm = ix > 0 ? ix - 1 : ix, xp = ix + 2 < nx ? ix + 2 : ix + 1;
    const int ym = iy > 0 ? iy - 1 : iy, yp = iy + 2 < ny ? iy + 2 : iy + 1;
    auto col = [&](int i, int j) { return ne + ((size_t)i * ny + j) * nz; };
    const T *c00 = col(ix, iy), *c10 = col(ix + 1, iy), *c01 = col(ix, iy + 1), *c11 = col(ix + 1, iy + 1);
    const T *cxm0 = col(xm, iy), *cxp0 = col(xp, iy), *cxm1 = col(xm, iy + 1), *cxp1 = col(xp, iy + 1);
    const T *cym0 = col(ix, ym), *cyp0 = col(ix, yp), *cym1 = col(ix + 1, ym), *cyp1 = col(ix + 1, yp);
    // numpy.gradient (unit spacing): central inside, one-sided at the faces
    const float dx0 = ix > 0 ? 0.5f : 1.f, dx1 = ix + 2 < nx ? 0.5f : 1.f;
    const float dy0 = iy > 0 ? 0.5f : 1.f, dy1 = iy + 2 < ny ? 0.5f : 1.f;
    auto q = [&](const T* c, int k) {
        const float v = (float)c[k] * inv_nc;
        return v < ne_max ? v : ne_max;
    };
    float sx = 0.f, sy = 0.f, sp = 0.f;
    float slx[kMaxSlab], sly[kMaxSlab];
#pragma unroll
    for (int q = 0; q < kMaxSlab; ++q) slx[q] = sly[q] = 0.f;
    for (int k = lane; k < nz; k += 32) {
        const float q00 = q(c00, k), q10 = q(c10, k), q01 = q(c01, k), q11 = q(c11, k);
        // d/dx at (ix, .) uses (ix+1) - (ix-1) (or the one-sided pair), at (ix+1, .) uses (ix+2) - ix
        const float gx0 = dx0 * (q10 - q(cxm0, k)), gx1 = dx1 * (q(cxp0, k) - q00);
        const float gx2 = dx0 * (q11 - q(cxm1, k)), gx3 = dx1 * (q(cxp1, k) - q01);
        const float gy0 = dy0 * (q01 - q(cym0, k)), gy2 = dy1 * (q(cyp0, k) - q00);
        const float gy1 = dy0 * (q11 - q(cym1, k)), gy3 = dy1 * (q(cyp1, k) - q10);
        const float gxk = w00 * gx0 + w10 * gx1 + w01 * gx2 + w11 * gx3;
        const float gyk = w00 * gy0 + w10 * gy1 + w01 * gy2 + w11 * gy3;
        const float wz = (k == 0 || k == nz - 1) ? 0.5f : 1.f;
        sx = fmaf(wz, gxk, sx);
        sy = fmaf(wz, gyk, sy);
        // node k's trapezoid weight is half from cell k-1 and half from cell k,
        // each credited to that cell's slab
        if (nslab > 0) {
#pragma unroll
            for (int q = 0; q < kMaxSlab; ++q) {
                const float wl = (k > 0 && (int)((long long)(k - 1) * nslab / (nz - 1)) == q) ? 0.5f : 0.f;
                const float wr = (k < nz - 1 && (int)((long long)k * nslab / (nz - 1)) == q) ? 0.5f : 0.f;
                slx[q] = fmaf(wl + wr, gxk, slx[q]);
                sly[q] = fmaf(wl + wr, gyk, sly[q]);
            }
        }
        if (k + 1 < nz) {  // the cell [k, k+1]: 4-point Gauss-Legendre on the linear q(z)
            const float qk = w00 * q00 + w10 * q10 + w01 * q01 + w11 * q11;
            const float qn = w00 * q(c00, k + 1) + w10 * q(c10, k + 1) + w01 * q(c01, k + 1) + w11 * q(c11, k + 1);
            float cell = 0.f;
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const float r = 1.f - (qk + gw[g] * (qn - qk));
                cell += gwt[g] * (sqrtf(r > 0.f ? r : 0.f) - 1.f);
            }
            sp += cell;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
#pragma unroll
        for (int q = 0; q < kMaxSlab; ++q) {
            if (q < nslab) {
                slx[q] += __shfl_xor_sync(0xffffffffu, slx[q], off);
                sly[q] += __shfl_xor_sync(0xffffffffu, sly[q], off);
            }
        }
        sp += __shfl_xor_sync(0xffffffffu, sp, off);
    }
    if (lane == 0) {
        out[warp] = (float)(-0.5 * (double)sx * hz / hx);
        out[n + warp] = (float)(-0.5 * (double)sy * hz / hy);
        out[2 * n + warp] = (float)(k0 * (double)sp * hz);
#pragma unroll
        for (int q = 0; q < kMaxSlab; ++q) {
            if (q < nslab) {
                out[(3 + 2 * q) * n + warp] = (float)(-0.5 * (double)slx[q] * hz / hx);
                out[(4 + 2 * q) * n + warp] = (float)(-0.5 * (double)sly[q] * hz / hy);
            }
        }
    }
}

}  // namespace

extern "C" int tt_straight_line_maps(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x,
                                     const double* y, const double* z, double lwl, double ne_max, int P, int nslab,
                                     float* out, void* stream)
{
    if (nslab < 0 || nslab > kMaxSlab) return tt::invalid("straight_line_maps: nslab must be 0..8");
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
    const long long threads = (long long)n * 32;
    const int grid = (int)((threads + 255) / 256);
    cudaStream_t s = tt::as_stream(stream);
    if (ne_dtype == TT_F32)
        maps_kernel<float><<<grid, 256, 0, s>>>((const float*)ne, nx, ny, nz, hx, hy, hz, (float)(1.0 / nc),
                                                (float)ne_max, k0, P, nslab, out);
    else
        maps_kernel<double><<<grid, 256, 0, s>>>((const double*)ne, nx, ny, nz, hx, hy, hz, (float)(1.0 / nc),
                                                 (float)ne_max, k0, P, nslab, out);
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
