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
// nodes); the phase uses 2-point Gauss-Legendre in every z cell.
#include "tt_common.cuh"

namespace {

constexpr int kMaxSlab = 8;

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float sqrt_approx(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// n - 1 = sqrt(1 - q) - 1 in the form without cancellation for small q
__device__ __forceinline__ float index_minus_one(float q)
{
    const float r = 1.f - q;
    return -q * rcp_approx(1.f + sqrt_approx(r > 0.f ? r : 0.f));
}


// One warp per pixel: lane l handles nodes k = l, l + 32, ... along z, so
// the column reads (z is the fastest axis of the density) are coalesced; the
// per-lane sums are combined with shuffles.
template <typename T, bool SLAB>
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
        if (SLAB) {
#pragma unroll
            for (int q = 0; q < kMaxSlab; ++q) {
                const float wl = (k > 0 && (int)((long long)(k - 1) * nslab / (nz - 1)) == q) ? 0.5f : 0.f;
                const float wr = (k < nz - 1 && (int)((long long)k * nslab / (nz - 1)) == q) ? 0.5f : 0.f;
                slx[q] = fmaf(wl + wr, gxk, slx[q]);
                sly[q] = fmaf(wl + wr, gyk, sly[q]);
            }
        }
        if (k + 1 < nz) {  // the cell [k, k+1]: 2-point Gauss-Legendre on the linear q(z)
            const float qk = w00 * q00 + w10 * q10 + w01 * q01 + w11 * q11;
            const float qn = w00 * q(c00, k + 1) + w10 * q(c10, k + 1) + w01 * q(c01, k + 1) + w11 * q(c11, k + 1);
            const float g = 0.2113248654051871f;  // 1/2 - 1/(2 sqrt 3)
            sp += 0.5f * (index_minus_one(fmaf(g, qn - qk, qk)) + index_minus_one(fmaf(g, qk - qn, qn)));
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
        if (SLAB) {
#pragma unroll
            for (int q = 0; q < kMaxSlab; ++q) {
                if (q < nslab) {
                    slx[q] += __shfl_xor_sync(0xffffffffu, slx[q], off);
                    sly[q] += __shfl_xor_sync(0xffffffffu, sly[q], off);
                }
            }
        }
        sp += __shfl_xor_sync(0xffffffffu, sp, off);
    }
    if (lane == 0) {
        out[warp] = (float)(-0.5 * (double)sx * hz / hx);
        out[n + warp] = (float)(-0.5 * (double)sy * hz / hy);
        out[2 * n + warp] = (float)(k0 * (double)sp * hz);
        if (SLAB) {
#pragma unroll
            for (int q = 0; q < kMaxSlab; ++q) {
                if (q < nslab) {
                    out[(3 + 2 * q) * n + warp] = (float)(-0.5 * (double)slx[q] * hz / hx);
                    out[(4 + 2 * q) * n + warp] = (float)(-0.5 * (double)sly[q] * hz / hy);
                }
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
    const float inv_nc = (float)(1.0 / nc), qmax = (float)ne_max;
    if (ne_dtype == TT_F32) {
        if (nslab > 0)
            maps_kernel<float, true><<<grid, 256, 0, s>>>((const float*)ne, nx, ny, nz, hx, hy, hz, inv_nc, qmax, k0,
                                                          P, nslab, out);
        else
            maps_kernel<float, false><<<grid, 256, 0, s>>>((const float*)ne, nx, ny, nz, hx, hy, hz, inv_nc, qmax, k0,
                                                           P, nslab, out);
    } else {
        if (nslab > 0)
            maps_kernel<double, true><<<grid, 256, 0, s>>>((const double*)ne, nx, ny, nz, hx, hy, hz, inv_nc, qmax,
                                                           k0, P, nslab, out);
        else
            maps_kernel<double, false><<<grid, 256, 0, s>>>((const double*)ne, nx, ny, nz, hx, hy, hz, inv_nc, qmax,
                                                            k0, P, nslab, out);
    }
    return tt::launch_status("straight_line_maps");
}

// Marched pixel-centre rays: the ray equation with z as the parameter and
// t = (dx/dz, dy/dz) the ray's slopes,
//   dt/dz   = -1/2 (1 + |t|^2) / (1 + q0 - q) * (grad_perp q - t dq/dz)
//   dphi/dz = k0 (sqrt(1 - q) - 1) sqrt(1 + |t|^2)
// (from dx/dt = v, dv/dt = -c^2/2 grad q and |v|^2 = c^2 (1 + q0 - q), q0 the
// value at the entry point), stepped from node plane to node plane (step hz)
// by kick-drift-kick, the closing kick's slope-dependent term evaluated at the
// slope predicted from the previous step's acceleration (second order), the
// phase summed in FP32 with Kahan compensation (every term has the sign of
// n - 1 <= 0).  Every plane is visited: skipping planes aliases the grid-scale gradient (the
// trapezoid rule on a field with power at the node spacing).  On a plane the
// fields are bilinear in x, y of the node values -- q and its numpy.gradient
// derivatives, zero outside the grid, i.e. the tracer's trilinear fields
// restricted to the node planes.
//
// Layout.  q = min(ne / n_c, ne_max) is first written plane-major into the
// workspace, [z][x + 1][y + 4] with a one-node ghost border around each plane
// holding the linear extrapolation 2 q(edge) - q(edge -+ 1): the central
// difference across the border then equals numpy.gradient's one-sided
// difference at the face, so every in-grid sample uses one branch-free
// stencil.  Rows are padded to a multiple of 4 floats so that y = 0 and every
// staged chunk start on 16 bytes.  The same pass sums q along z per column with
// trapezoid weights; the straight (unbent) ray's deflection is linear in q, so
// a small 2-D kernel turns those sums into the straight-line maps (the same
// definition as tt_straight_line_maps: exact for the trilinear field).
//
// The march: one thread per ray; tiles of kMarchRows x 32 rays (a warp = one
// row of 32 rays, so the staged reads are free of bank conflicts) stage the
// node rows and columns their rays can reach (the tile plus kMarchHalo cells),
// plane by plane, into a ring of kMarchRing planes in shared memory with
// cp.async, kMarchRing - 2 planes ahead of the march.  A ray whose stencil
// leaves the staged window (a drift of more than about kMarchHalo - 2 cells)
// reads that sample from global memory; the results are the same either way.
// Pixel grids coarser than the node grid take the unstaged kernel.
namespace {

constexpr int kPadY = 4;  // padded column of y = 0

__host__ __device__ inline int padded_ny(int ny) { return (ny + kPadY + 1 + 3) & ~3; }
__host__ __device__ inline size_t padded_plane(int nx, int ny) { return (size_t)(nx + 2) * padded_ny(ny); }

struct MarchFields {
    const void* ne[TT_MAX_MARCH_FIELDS];
};

// Per-field workspace (floats): the padded planes, then the column sums.
inline size_t field_ws_floats(int nx, int ny, int nz)
{
    const size_t f = (size_t)nz * padded_plane(nx, ny) + (size_t)nx * ny;
    return (f + 63) & ~(size_t)63;  // 256-byte aligned per field
}

// Four consecutive z values of column (a, y) from z on, zero past nz; VEC:
// 16-byte aligned vector loads (nz % 4 == 0 and an aligned base).
template <bool VEC>
__device__ __forceinline__ void load4(const float* __restrict__ col, int z, int nz, float (&v)[4])
{
    if (VEC && z + 3 < nz) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(col + z));
        v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = z + j < nz ? __ldg(col + z + j) : 0.f;
    }
}

template <bool VEC>
__device__ __forceinline__ void load4(const double* __restrict__ col, int z, int nz, float (&v)[4])
{
    if (VEC && z + 3 < nz) {
        const double2 t0 = __ldg(reinterpret_cast<const double2*>(col + z));
        const double2 t1 = __ldg(reinterpret_cast<const double2*>(col + z + 2));
        v[0] = (float)t0.x, v[1] = (float)t0.y, v[2] = (float)t1.x, v[3] = (float)t1.y;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = z + j < nz ? (float)__ldg(col + z + j) : 0.f;
    }
}

// q -> padded plane-major, and the trapezoid column sums Sum_k w_k q(x, y, k).
// Block: one x, 32 columns y of field blockIdx.z; z in chunks of 128 through
// shared memory (read along z, four values a lane, 16 in flight a thread;
// write along y).  The column sums are per-thread partials over the lane's z
// values, reduced across the warp at the end (a fixed order).
template <typename T, bool VEC>
__global__ void __launch_bounds__(256) plane_q_kernel(const __grid_constant__ MarchFields fields, int nx, int ny,
                                                     int nz, float inv_nc, float ne_max, float* __restrict__ ws,
                                                     size_t ws_field)
{
    __shared__ float tile[32][129];
    const T* __restrict__ ne = static_cast<const T*>(fields.ne[blockIdx.z]);
    float* __restrict__ qt = ws + blockIdx.z * ws_field;
    const size_t plane = padded_plane(nx, ny);
    float* __restrict__ colsum = qt + (size_t)nz * plane;
    const int nyp = padded_ny(ny);
    const int a = blockIdx.y;
    const int y0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float part[4] = {0.f, 0.f, 0.f, 0.f};
    for (int z0 = 0; z0 < nz; z0 += 128) {
        float v[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int y = y0 + w + 8 * i;
            if (y < ny) {
                load4<VEC>(ne + ((size_t)a * ny + y) * nz, z0 + 4 * lane, nz, v[i]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) v[i][j] = 0.f;
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int z = z0 + 4 * lane + j;
                float q = v[i][j] * inv_nc;
                q = q < ne_max ? q : ne_max;
                tile[w + 8 * i][4 * lane + j] = q;
                part[i] = fmaf((z == 0 || z == nz - 1) ? 0.5f : (z < nz ? 1.f : 0.f), q, part[i]);
            }
        }
        __syncthreads();
        const int y = y0 + lane;
        for (int zz = w; zz < 128; zz += 8) {
            const int z = z0 + zz;
            if (z < nz && y < ny) qt[(size_t)z * plane + (size_t)(a + 1) * nyp + y + kPadY] = tile[lane][zz];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) part[i] += __shfl_xor_sync(0xffffffffu, part[i], off);
        const int y = y0 + w + 8 * i;
        if (lane == 0 && y < ny) colsum[(size_t)a * ny + y] = part[i];
    }
}

// Ghost border of every plane: rows x = -1, nx (over y in [0, ny)) and columns
// y = -1, ny (over x in [0, nx)) as 2 q(edge) - q(next).  The four corner
// ghosts are never read by the stencil and are left as they are.
__global__ void plane_ghost_kernel(int nfields, int nx, int ny, int nz, float* __restrict__ ws, size_t ws_field)
{
    const int nyp = padded_ny(ny);
    const size_t plane = padded_plane(nx, ny);
    const long long per = 2LL * ny + 2LL * nx;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= per * nz * nfields) return;
    const int f = (int)(t / (per * nz));
    const long long tf = t - (long long)f * per * nz;
    const int z = (int)(tf / per);
    int e = (int)(tf - (long long)z * per);
    float* pl = ws + f * ws_field + (size_t)z * plane;
    auto at = [&](int x, int y) -> float& { return pl[(size_t)(x + 1) * nyp + y + kPadY]; };
    if (e < ny) {
        at(-1, e) = 2.f * at(0, e) - at(1, e);
    } else if ((e -= ny) < ny) {
        at(nx, e) = 2.f * at(nx - 1, e) - at(nx - 2, e);
    } else if ((e -= ny) < nx) {
        at(e, -1) = 2.f * at(e, 0) - at(e, 1);
    } else {
        e -= nx;
        at(e, ny) = 2.f * at(e, ny - 1) - at(e, ny - 2);
    }
}

// Straight-line deflection at the pixel centres from the column sums:
// -1/2 hz d/dx of the trapezoid sum (numpy.gradient rule), bilinear.
__global__ void straight_from_colsum_kernel(const float* __restrict__ ws, size_t ws_field, int nx, int ny, int nz,
                                            float cx, float cy, int P, float* __restrict__ out)
{
    const int n = P * P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int f = blockIdx.y;
    const float* __restrict__ colsum = ws + f * ws_field + (size_t)nz * padded_plane(nx, ny);
    float* __restrict__ ox = out + ((size_t)f * 5 + 3) * n;
    float* __restrict__ oy = ox + n;
    const int pi = p / P, pj = p % P;
    const double us = ((pi + 0.5) / P) * (nx - 1), vs = ((pj + 0.5) / P) * (ny - 1);
    const int i = min((int)us, nx - 2), j = min((int)vs, ny - 2);
    const float fx = (float)(us - i), fy = (float)(vs - j);
    auto C = [&](int a, int b) { return colsum[(size_t)a * ny + b]; };
    auto gx = [&](int a, int b) {
        if (a == 0) return C(1, b) - C(0, b);
        if (a == nx - 1) return C(nx - 1, b) - C(nx - 2, b);
        return 0.5f * (C(a + 1, b) - C(a - 1, b));
    };
    auto gy = [&](int a, int b) {
        if (b == 0) return C(a, 1) - C(a, 0);
        if (b == ny - 1) return C(a, ny - 1) - C(a, ny - 2);
        return 0.5f * (C(a, b + 1) - C(a, b - 1));
    };
    const float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w01 = (1.f - fx) * fy, w11 = fx * fy;
    ox[p] = cx * (w00 * gx(i, j) + w10 * gx(i + 1, j) + w01 * gx(i, j + 1) + w11 * gx(i + 1, j + 1));
    oy[p] = cy * (w00 * gy(i, j) + w10 * gy(i + 1, j) + w01 * gy(i, j + 1) + w11 * gy(i + 1, j + 1));
}

struct PlaneSample {
    float q, gx, gy, gz;  // q and its derivatives per index unit
};

// The cell of (u, v) (index units) on a node plane; false outside the grid,
// where every field is zero.
__device__ __forceinline__ bool locate(float u, float v, int nx, int ny, int& i, int& j, float& fx, float& fy)
{
    if (!(u >= 0.f && u <= (float)(nx - 1) && v >= 0.f && v <= (float)(ny - 1))) return false;
    i = min((int)u, nx - 2);
    j = min((int)v, ny - 2);
    fx = u - (float)i;
    fy = v - (float)j;
    return true;
}

// q and its derivatives at (i + fx, j + fy): c points at node (i, j) of the
// plane, m and p at that node of the planes used for d/dz (dz = 1/2 inside,
// 1 at the first and last plane, where they are the plane itself and its
// neighbour); ry is the row stride.  Central differences throughout: the ghost
// border supplies the one-sided rule at the faces.
template <typename Stride>
__device__ __forceinline__ PlaneSample sample_node(const float* c, const float* m, const float* p, Stride ry, float dz,
                                                   float fx, float fy)
{
    // corners as (value, d/dz) and (d/dx, d/dy) pairs; packed FP32x2 arithmetic
    const float q00 = c[0], q10 = c[ry], q01 = c[1], q11 = c[ry + 1];
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 Z00 = __ffma2_rn(make_float2(m[0], m[ry]), m1, make_float2(p[0], p[ry]));
    const float2 Z01 = __ffma2_rn(make_float2(m[1], m[ry + 1]), m1, make_float2(p[1], p[ry + 1]));
    const float2 G00 = __ffma2_rn(make_float2(c[-ry], c[-1]), m1, make_float2(q10, q01));
    const float2 G10 = __ffma2_rn(make_float2(q00, c[ry - 1]), m1, make_float2(c[2 * ry], q11));
    const float2 G01 = __ffma2_rn(make_float2(c[1 - ry], q00), m1, make_float2(q11, c[2]));
    const float2 G11 = __ffma2_rn(make_float2(q01, q10), m1, make_float2(c[2 * ry + 1], c[ry + 2]));
    const float2 X = make_float2(fx, fx), Y = make_float2(fy, fy);
    // bilinear as nested linear interpolation: along x at y = j and j + 1, then along y
    auto lerp2 = [&](float2 a, float2 b, float2 t) { return __ffma2_rn(t, __ffma2_rn(a, m1, b), a); };
    const float2 G = lerp2(lerp2(G00, G10, X), lerp2(G01, G11, X), Y);
    const float2 Q = lerp2(lerp2(make_float2(q00, Z00.x), make_float2(q10, Z00.y), X),
                           lerp2(make_float2(q01, Z01.x), make_float2(q11, Z01.y), X), Y);
    PlaneSample s;
    s.q = Q.x;
    s.gx = 0.5f * G.x;
    s.gy = 0.5f * G.y;
    s.gz = dz * Q.y;
    return s;
}

template <int RY>
struct Imm {  // a row stride known at compile time (immediate offsets)
    __device__ __forceinline__ constexpr operator int() const { return RY; }
};

__device__ __noinline__ PlaneSample sample_global(const float* __restrict__ qt, int nx, int ny, int nz, int i, int j,
                                                  float fx, float fy, int k)
{
    const int nyp = padded_ny(ny);
    const size_t plane = padded_plane(nx, ny);
    const int km = k > 0 ? k - 1 : k, kp = k + 1 < nz ? k + 1 : k;
    const float dz = (k > 0 && k + 1 < nz) ? 0.5f : 1.f;
    const size_t node = (size_t)(i + 1) * nyp + j + kPadY;
    return sample_node(qt + (size_t)k * plane + node, qt + (size_t)km * plane + node, qt + (size_t)kp * plane + node,
                       nyp, dz, fx, fy);
}

struct MarchConsts {
    float ihx, ihy, ihz, hz;
};

struct MarchRay {
    float u, v, tx, ty, ax, ay, e_prev, q0;
    float phi, phi_c;  // Kahan-compensated phase sum (per m)
};

__device__ __forceinline__ void march_accel(const PlaneSample& f, float sx, float sy, float q0, const MarchConsts& mc,
                                            float& ax, float& ay)
{
    const float vv = 1.f + q0 - f.q;  // |v|^2 / c^2; the ray turns back where it reaches 0
    const float c = -0.5f * (1.f + sx * sx + sy * sy) * rcp_approx(vv > 1e-6f ? vv : 1e-6f);
    const float gz = f.gz * mc.ihz;
    ax = c * (f.gx * mc.ihx - sx * gz);
    ay = c * (f.gy * mc.ihy - sy * gz);
}

__device__ __forceinline__ float march_dphase(const PlaneSample& f, float sx, float sy)
{
    return index_minus_one(f.q) * sqrt_approx(1.f + sx * sx + sy * sy);
}

__device__ __forceinline__ void march_start(MarchRay& r, const PlaneSample& s, const MarchConsts& mc)
{
    r.q0 = s.q;
    r.tx = r.ty = 0.f;
    march_accel(s, 0.f, 0.f, r.q0, mc, r.ax, r.ay);
    r.e_prev = march_dphase(s, 0.f, 0.f);
    r.phi = r.phi_c = 0.f;
}

// First half of a step of h (m): half kick, then the drift to the next plane.
__device__ __forceinline__ void march_kick_drift(MarchRay& r, float h, const MarchConsts& mc)
{
    const float hh = 0.5f * h;
    r.tx = fmaf(hh, r.ax, r.tx);
    r.ty = fmaf(hh, r.ay, r.ty);
    r.u = fmaf(h * mc.ihx, r.tx, r.u);
    r.v = fmaf(h * mc.ihy, r.ty, r.v);
}

// Second half: the closing half kick with the fields s on the new plane (its
// slope-dependent term at the slope predicted with the previous step's
// acceleration), and the trapezoid phase of the step.
__device__ __forceinline__ void march_kick(MarchRay& r, float h, const PlaneSample& s, const MarchConsts& mc)
{
    const float hh = 0.5f * h;
    march_accel(s, fmaf(hh, r.ax, r.tx), fmaf(hh, r.ay, r.ty), r.q0, mc, r.ax, r.ay);
    r.tx = fmaf(hh, r.ax, r.tx);
    r.ty = fmaf(hh, r.ay, r.ty);
    const float e = march_dphase(s, r.tx, r.ty);
    const float y = hh * (r.e_prev + e) - r.phi_c;
    const float t = r.phi + y;
    r.phi_c = (t - r.phi) - y;
    r.phi = t;
    r.e_prev = e;
}

__device__ __forceinline__ void march_write(const MarchRay& r, double k0, int n, int p, float* __restrict__ out)
{
    out[p] = atanf(r.tx);
    out[n + p] = atanf(r.ty);
    out[2 * n + p] = (float)(k0 * ((double)r.phi - (double)r.phi_c));
}

// Any pixel grid: one thread per ray, fields read from the padded q through L1/L2.
__global__ void __launch_bounds__(128) march_kernel(const float* __restrict__ ws, size_t ws_field, int nx, int ny,
                                                    int nz, MarchConsts mc, double k0, int P, int stride,
                                                    float* __restrict__ out)
{
    const int n = P * P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* __restrict__ qt = ws + blockIdx.y * ws_field;
    out += (size_t)blockIdx.y * 5 * n;
    const int pi = p / P, pj = p % P;
    MarchRay r;
    r.u = (float)(((pi + 0.5) / P) * (nx - 1));
    r.v = (float)(((pj + 0.5) / P) * (ny - 1));
    for (int k = 0, kp = 0; k < nz; kp = k, k = (k + stride < nz || k == nz - 1) ? k + stride : nz - 1) {
        const float h = (float)(k - kp) * mc.hz;
        if (k > 0) march_kick_drift(r, h, mc);
        int i, j;
        float fx, fy;
        PlaneSample s{0.f, 0.f, 0.f, 0.f};
        if (locate(r.u, r.v, nx, ny, i, j, fx, fy)) s = sample_global(qt, nx, ny, nz, i, j, fx, fy, k);
        if (k == 0)
            march_start(r, s, mc);
        else
            march_kick(r, h, s, mc);
    }
    march_write(r, k0, n, p, out);
}

constexpr int kMarchCols = 32;  // rays per tile row (one warp)
constexpr int kMarchRows = 8;   // tile rows (warps per block)
constexpr int kMarchHalo = 8;
constexpr int kMarchRing = 8;
constexpr int kMarchRX = kMarchRows + 2 * kMarchHalo + 4;  // staged rows: tile span + halo + the 4-node stencil
constexpr int kMarchRY = kMarchCols + 2 * kMarchHalo + 8;  // staged columns, incl. the 16-byte alignment slack
constexpr int kMarchPlane = kMarchRX * kMarchRY;
constexpr int kMarchChunks = kMarchPlane / 4;  // 16-byte chunks per staged plane
constexpr int kMarchThreads = kMarchCols * kMarchRows;
constexpr int kMarchChunksPerThread = (kMarchChunks + kMarchThreads - 1) / kMarchThreads;
static_assert(kMarchRY % 4 == 0, "staged rows must be whole 16-byte chunks");

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}

template <int V>
struct Slot {  // a ring slot known at compile time
    static constexpr int value = V;
};

// The march's out-of-line sampler: the first and last planes from the ring
// (d/dz one-sided there) and rays whose stencil has left the staged window
// (from the padded volume in global memory).
__device__ __noinline__ PlaneSample sample_slow(const float* ring, bool staged, int b, const float* __restrict__ qt,
                                                int nx, int ny, int nz, int i, int j, float fx, float fy, int k)
{
    if (!staged) return sample_global(qt, nx, ny, nz, i, j, fx, fy, k);
    const int km = k > 0 ? k - 1 : k, kp = k + 1 < nz ? k + 1 : k;
    const float dz = (k > 0 && k + 1 < nz) ? 0.5f : 1.f;
    return sample_node(ring + (k & (kMarchRing - 1)) * kMarchPlane + b, ring + (km & (kMarchRing - 1)) * kMarchPlane + b,
                       ring + (kp & (kMarchRing - 1)) * kMarchPlane + b, Imm<kMarchRY>{}, dz, fx, fy);
}

// Pixel grids at least as fine as the node grid (a tile spans at most
// kMarchRows x kMarchCols node cells).  Window coordinates are padded ones:
// row R = x + 1, column C = y + kPadY.
template <int STRIDE>
__global__ void __launch_bounds__(kMarchThreads) march_staged_kernel(const float* __restrict__ ws, size_t ws_field,
                                                                     int nx, int ny, int nz, MarchConsts mc, double k0,
                                                                     int P, float* __restrict__ out)
{
    extern __shared__ __align__(16) float ring[];
    const float* __restrict__ qt = ws + blockIdx.z * ws_field;
    out += (size_t)blockIdx.z * 5 * P * P;
    const int ti = threadIdx.x / kMarchCols, tj = threadIdx.x % kMarchCols;
    const int pi = blockIdx.y * kMarchRows + ti, pj = blockIdx.x * kMarchCols + tj;
    const bool active = pi < P && pj < P;
    const int nyp = padded_ny(ny);
    const size_t plane = padded_plane(nx, ny);
    const double sxp = (double)(nx - 1) / P, syp = (double)(ny - 1) / P;
    const int R0 = (int)floor((blockIdx.y * kMarchRows + 0.5) * sxp) + 1 - kMarchHalo;
    const int C0 = ((int)floor((blockIdx.x * kMarchCols + 0.5) * syp) + kPadY - kMarchHalo) & ~3;
    // staged rows/columns that exist in the padded plane
    const int vR0 = max(R0, 0), vR1 = min(R0 + kMarchRX, nx + 2);
    const int vC0 = max(C0, 0), vC1 = min(C0 + kMarchRY, nyp);
    int soff[kMarchChunksPerThread];
    long long goff[kMarchChunksPerThread];
#pragma unroll
    for (int q = 0; q < kMarchChunksPerThread; ++q) {
        const int c = threadIdx.x + q * kMarchThreads;
        soff[q] = -1;
        goff[q] = 0;
        if (c < kMarchChunks) {
            const int r = c / (kMarchRY / 4), cc = (c % (kMarchRY / 4)) * 4;
            const int R = R0 + r, C = C0 + cc;
            if (R >= 0 && R < nx + 2 && C >= 0 && C + 4 <= nyp) {
                soff[q] = r * kMarchRY + cc;
                goff[q] = (long long)R * nyp + C;
            }
        }
    }
    // planes a..b (those below nz) as one cp.async group
    auto issue = [&](int a, int b) {
        for (int pl = a; pl <= b && pl < nz; ++pl) {
            float* dst = ring + (pl & (kMarchRing - 1)) * kMarchPlane;
            const float* src = qt + (size_t)pl * plane;
#pragma unroll
            for (int q = 0; q < kMarchChunksPerThread; ++q)
                if (soff[q] >= 0) cp_async16(dst + soff[q], src + goff[q]);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    // The ray's cell (i, j) and fractions (fx, fy) in [0, 1) are kept as they
    // are; the cell, its in-grid flag and its place in the staged window are
    // recomputed only when the ray crosses a cell face.
    MarchRay r;
    int i = 0, j = 0, b = 0;
    bool in = false, st = false;
    float fx = (float)(((pi + 0.5) / P) * (nx - 1)), fy = (float)(((pj + 0.5) / P) * (ny - 1));
    auto relocate = [&]() {
        const float flx = floorf(fx), fly = floorf(fy);
        i += (int)flx;
        fx -= flx;
        j += (int)fly;
        fy -= fly;
        if (fx >= 1.f) fx -= 1.f, ++i;  // a tiny negative fraction rounds up to 1
        if (fy >= 1.f) fy -= 1.f, ++j;
        if (i == nx - 1 && fx == 0.f) i = nx - 2, fx = 1.f;  // the grid's upper faces belong to the last cell
        if (j == ny - 1 && fy == 0.f) j = ny - 2, fy = 1.f;
        in = i >= 0 && i <= nx - 2 && j >= 0 && j <= ny - 2;
        // stencil rows x = i-1..i+2 -> R = i..i+3, columns y = j-1..j+2 -> C = j+kPadY-1..j+kPadY+2
        const int R = i + 1, C = j + kPadY;
        st = in && R - 1 >= vR0 && R + 2 < vR1 && C - 1 >= vC0 && C + 2 < vC1;
        b = (R - R0) * kMarchRY + (C - C0);
    };
    relocate();
    // one plane per step, or (STRIDE 2) every second plane and the last one
    const float hh = 0.5f * mc.hz, dxi = mc.hz * mc.ihx, dyi = mc.hz * mc.ihy;
    const float h2 = 2.f * mc.hz, hh2 = 0.5f * h2, dxi2 = h2 * mc.ihx, dyi2 = h2 * mc.ihy;
    // Step to plane k, whose ring slot K = k mod kMarchRing is a compile-time
    // constant: inside the volume the stencil's three planes sit at fixed
    // offsets from the ray's window base, so its shared loads need no address
    // arithmetic.  The first and last planes (one-sided d/dz) and rays outside
    // the staged window take the out-of-line sampler.
    auto step = [&](int k, auto slot, bool wide) {
        constexpr int K = decltype(slot)::value;
        const bool first = K == 0 && k == 0;
        if (!first) {  // half kick, drift to plane k
            r.tx = fmaf(wide ? hh2 : hh, r.ax, r.tx);
            r.ty = fmaf(wide ? hh2 : hh, r.ay, r.ty);
            fx = fmaf(wide ? dxi2 : dxi, r.tx, fx);
            fy = fmaf(wide ? dyi2 : dyi, r.ty, fy);
            if (!(fx >= 0.f && fx < 1.f && fy >= 0.f && fy < 1.f)) relocate();
        }
        PlaneSample s{0.f, 0.f, 0.f, 0.f};
        if (in) {
            if (st && !first && k + 1 < nz) {
                const float* c = ring + b;
                s = sample_node(c + K * kMarchPlane, c + ((K + kMarchRing - 1) % kMarchRing) * kMarchPlane,
                                c + ((K + 1) % kMarchRing) * kMarchPlane, Imm<kMarchRY>{}, 0.5f, fx, fy);
            } else {
                s = sample_slow(ring, st, b, qt, nx, ny, nz, i, j, fx, fy, k);
            }
        }
        if (first)
            march_start(r, s, mc);
        else
            march_kick(r, wide ? h2 : mc.hz, s, mc);
    };
    // planes pl and pl + 1 (those below nz) into ring slots S and S + 1, one group
    auto issue2 = [&](int pl, auto slot) {
        constexpr int S = decltype(slot)::value;
        if (pl < nz) {
            const float* src = qt + (size_t)pl * plane;
#pragma unroll
            for (int q = 0; q < kMarchChunksPerThread; ++q)
                if (soff[q] >= 0) cp_async16(ring + S * kMarchPlane + soff[q], src + goff[q]);
        }
        if (pl + 1 < nz) {
            const float* src = qt + (size_t)(pl + 1) * plane;
#pragma unroll
            for (int q = 0; q < kMarchChunksPerThread; ++q)
                if (soff[q] >= 0) cp_async16(ring + ((S + 1) % kMarchRing) * kMarchPlane + soff[q], src + goff[q]);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // Two planes per barrier.  Groups: {0}, {1, 2}, {3, 4} ahead, then {k+5, k+6}
    // at step pair k into the slots of planes k-3 and k-2; at pair k the ring
    // holds planes k-3..k+4 and the pair reads k-1..k+2.
    auto pair = [&](int k, auto slot) {
        constexpr int K = decltype(slot)::value;
        asm volatile("cp.async.wait_group 1;" ::: "memory");  // all but {k+3, k+4}: planes <= k+2 are in
        __syncthreads();
        issue2(k + 5, Slot<(K + 5) % kMarchRing>{});
        if (active) {
            if (STRIDE == 1) {
                step(k, slot, false);
                if (k + 1 < nz) step(k + 1, Slot<K + 1>{}, false);
            } else {  // k is even: a double step to plane k, a single one to a last odd plane
                step(k, slot, k > 0);
                if (k + 1 == nz - 1) step(k + 1, Slot<K + 1>{}, false);
            }
        }
    };
    static_assert(kMarchRing == 8, "ring schedule below assumes 8 planes");
    issue(0, 0);
    issue(1, 2);
    issue(3, 4);
    // four pairs per pass, so every ring slot is a constant
    for (int k = 0; k < nz; k += kMarchRing) {
        pair(k, Slot<0>{});
        if (k + 2 >= nz) break;
        pair(k + 2, Slot<2>{});
        if (k + 4 >= nz) break;
        pair(k + 4, Slot<4>{});
        if (k + 6 >= nz) break;
        pair(k + 6, Slot<6>{});
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (active) march_write(r, k0, P * P, pi * P + pj, out);
}

}  // namespace

extern "C" size_t tt_march_maps_batched_workspace_bytes(int nfields, int nx, int ny, int nz)
{
    if (nfields < 1 || nx < 2 || ny < 2 || nz < 2) return 0;
    return (size_t)nfields * field_ws_floats(nx, ny, nz) * sizeof(float);
}

extern "C" size_t tt_march_maps_workspace_bytes(int nx, int ny, int nz)
{
    return tt_march_maps_batched_workspace_bytes(1, nx, ny, nz);
}

extern "C" int tt_march_maps_batched_stride(const void* const* ne, int nfields, int ne_dtype, int nx, int ny, int nz,
                                            const double* x, const double* y, const double* z, double lwl,
                                            double ne_max, int P, int plane_stride, float* out, void* workspace,
                                            size_t workspace_bytes, void* stream)
{
    if (plane_stride != 1 && plane_stride != 2) return tt::invalid("march_maps: plane_stride must be 1 or 2");
    if (!ne || !x || !y || !z || !out || !workspace) return tt::invalid("march_maps: NULL pointer");
    if (nfields < 1 || nfields > TT_MAX_MARCH_FIELDS) return tt::invalid("march_maps: 1..TT_MAX_MARCH_FIELDS fields");
    if (nx < 2 || ny < 2 || nz < 2 || P < 1 || (long long)P * P > 0x7fffffffLL / 5 || nx > 65535 || ny > 65535 * 32)
        return tt::invalid("march_maps: bad sizes");
    const size_t need = tt_march_maps_batched_workspace_bytes(nfields, nx, ny, nz);
    if (workspace_bytes < need) {
        tt::set_detail("march_maps: workspace needs %zu bytes", need);
        return TT_ERR_WORKSPACE_TOO_SMALL;
    }
    if (ne_dtype != TT_F32 && ne_dtype != TT_F64) return tt::invalid("march_maps: ne_dtype");
    if ((reinterpret_cast<uintptr_t>(workspace) & 15) != 0) return tt::invalid("march_maps: workspace not 16-byte aligned");
    MarchFields fields{};
    for (int f = 0; f < nfields; ++f) {
        if (!ne[f]) return tt::invalid("march_maps: NULL field");
        fields.ne[f] = ne[f];
    }
    const double hx = (x[nx - 1] - x[0]) / (nx - 1), hy = (y[ny - 1] - y[0]) / (ny - 1),
                 hz = (z[nz - 1] - z[0]) / (nz - 1);
    if (!(hx > 0) || !(hy > 0) || !(hz > 0)) return tt::invalid("march_maps: coordinates must increase");
    const double omega = 2.0 * CUDART_PI * (TT_C_LIGHT / lwl);
    const double nc = 3.14207787e-4 * omega * omega;
    const double k0 = omega / TT_C_LIGHT;
    cudaStream_t s = tt::as_stream(stream);
    float* ws = static_cast<float*>(workspace);
    const size_t wsf = field_ws_floats(nx, ny, nz);
    const dim3 tg((ny + 31) / 32, nx, nfields);
    bool vec = nz % 4 == 0;
    for (int f = 0; f < nfields; ++f) vec = vec && (reinterpret_cast<uintptr_t>(ne[f]) & 15) == 0;
    const float inv_nc = (float)(1.0 / nc), qmax = (float)ne_max;
    if (ne_dtype == TT_F32) {
        if (vec)
            plane_q_kernel<float, true><<<tg, 256, 0, s>>>(fields, nx, ny, nz, inv_nc, qmax, ws, wsf);
        else
            plane_q_kernel<float, false><<<tg, 256, 0, s>>>(fields, nx, ny, nz, inv_nc, qmax, ws, wsf);
    } else {
        if (vec)
            plane_q_kernel<double, true><<<tg, 256, 0, s>>>(fields, nx, ny, nz, inv_nc, qmax, ws, wsf);
        else
            plane_q_kernel<double, false><<<tg, 256, 0, s>>>(fields, nx, ny, nz, inv_nc, qmax, ws, wsf);
    }
    TT_TRY(tt::launch_status("march_maps plane_q"));
    const long long nghost = (2LL * nx + 2LL * ny) * nz * nfields;
    plane_ghost_kernel<<<(unsigned)((nghost + 255) / 256), 256, 0, s>>>(nfields, nx, ny, nz, ws, wsf);
    TT_TRY(tt::launch_status("march_maps ghost"));
    const int n = P * P;
    straight_from_colsum_kernel<<<dim3((n + 255) / 256, nfields), 256, 0, s>>>(
        ws, wsf, nx, ny, nz, (float)(-0.5 * hz / hx), (float)(-0.5 * hz / hy), P, out);
    TT_TRY(tt::launch_status("march_maps straight"));
    const MarchConsts mc{(float)(1.0 / hx), (float)(1.0 / hy), (float)(1.0 / hz), (float)hz};
    // staged tiles need a tile to span at most kMarchRows x kMarchCols node cells
    if ((long long)(nx - 1) <= P && (long long)(ny - 1) <= P) {
        const size_t smem = (size_t)kMarchRing * kMarchPlane * sizeof(float);
        const dim3 grid((P + kMarchCols - 1) / kMarchCols, (P + kMarchRows - 1) / kMarchRows, nfields);
        if (plane_stride == 1) {
            TT_TRY(tt::cuda_status(cudaFuncSetAttribute(march_staged_kernel<1>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                                   "march_maps attribute"));
            march_staged_kernel<1><<<grid, kMarchThreads, smem, s>>>(ws, wsf, nx, ny, nz, mc, k0, P, out);
        } else {
            TT_TRY(tt::cuda_status(cudaFuncSetAttribute(march_staged_kernel<2>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                                   "march_maps attribute"));
            march_staged_kernel<2><<<grid, kMarchThreads, smem, s>>>(ws, wsf, nx, ny, nz, mc, k0, P, out);
        }
    } else {
        march_kernel<<<dim3((n + 127) / 128, nfields), 128, 0, s>>>(ws, wsf, nx, ny, nz, mc, k0, P, plane_stride,
                                                                     out);
    }
    return tt::launch_status("march_maps");
}

extern "C" int tt_march_maps_batched(const void* const* ne, int nfields, int ne_dtype, int nx, int ny, int nz,
                                     const double* x, const double* y, const double* z, double lwl, double ne_max,
                                     int P, float* out, void* workspace, size_t workspace_bytes, void* stream)
{
    return tt_march_maps_batched_stride(ne, nfields, ne_dtype, nx, ny, nz, x, y, z, lwl, ne_max, P, 1, out, workspace,
                                        workspace_bytes, stream);
}

extern "C" int tt_march_maps(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x, const double* y,
                             const double* z, double lwl, double ne_max, int P, float* out, void* workspace,
                             size_t workspace_bytes, void* stream)
{
    const void* one[1] = {ne};
    return tt_march_maps_batched(one, 1, ne_dtype, nx, ny, nz, x, y, z, lwl, ne_max, P, out, workspace,
                                 workspace_bytes, stream);
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

// Map blockIdx.y of a batch: theta (2, P, P), I and div (P, P) per map; the
// drift is D, or Dv[blockIdx.y] when Dv is given.
__global__ void shadow_kernel(const float* __restrict__ theta, int P, float inv_h, float D, const double* __restrict__ Dv,
                              float* __restrict__ I, float* __restrict__ div)
{
    const int n = P * P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    theta += (size_t)blockIdx.y * 2 * n;
    if (I) I += (size_t)blockIdx.y * n;
    if (div) div += (size_t)blockIdx.y * n;
    if (Dv) D = (float)Dv[blockIdx.y];
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
                                                                       nullptr, intensity, div);
    return tt::launch_status("shadowgram");
}

extern "C" int tt_shadowgram_batched(const float* theta, int nmaps, int P, double pitch, const double* D,
                                     float* intensity, void* stream)
{
    if (!theta || !D || !intensity || nmaps < 1 || nmaps > 65535 || P < 2 || !(pitch > 0))
        return tt::invalid("shadowgram_batched: bad arguments");
    const int n = P * P;
    shadow_kernel<<<dim3((n + 255) / 256, nmaps), 256, 0, tt::as_stream(stream)>>>(theta, P, (float)(1.0 / pitch),
                                                                                    0.f, D, intensity, nullptr);
    return tt::launch_status("shadowgram_batched");
}

// ----------------------------------------------------------------------------- surrogate input and output
// The network's input encoding and the fallback's error estimate, fused.  The
// learned surrogate has no counterpart in the reference.
namespace {

// Block sums of three doubles in a fixed order (warp shuffles, then warp 0
// over the warps' partials); the result is valid in thread 0.
__device__ __forceinline__ void block_sum3(double& a, double& b, double& c)
{
    __shared__ double red[3][32];
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
        c += __shfl_xor_sync(0xffffffffu, c, off);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) red[0][warp] = a, red[1][warp] = b, red[2][warp] = c;
    __syncthreads();
    if (warp == 0) {
        a = lane < nw ? red[0][lane] : 0.0;
        b = lane < nw ? red[1][lane] : 0.0;
        c = lane < nw ? red[2][lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            b += __shfl_xor_sync(0xffffffffu, b, off);
            c += __shfl_xor_sync(0xffffffffu, c, off);
        }
    }
}

constexpr int kSurStatThreads = 1024;

// One block per field: s = rms of the straight-line deflection (planes 3, 4),
// the marched phase's mean and unbiased standard deviation (plane 2).  Each
// thread sums its pixels in FP32 (the phase shifted by the field's first
// value, so the variance does not cancel), the block adds the threads' sums
// in FP64.
__global__ void __launch_bounds__(kSurStatThreads) sur_encode_stats_kernel(const float* __restrict__ maps, int P,
                                                                           float* __restrict__ stats)
{
    const size_t N = (size_t)P * P;
    const float* __restrict__ m = maps + (size_t)blockIdx.x * 5 * N;
    const float ref = m[2 * N];
    float a = 0.f, b = 0.f, c = 0.f;
    for (size_t p = threadIdx.x; p < N; p += kSurStatThreads) {
        const float sx = m[3 * N + p], sy = m[4 * N + p], d = m[2 * N + p] - ref;
        a = fmaf(sx, sx, fmaf(sy, sy, a));
        b += d;
        c = fmaf(d, d, c);
    }
    double A = a, B = b, C = c;
    block_sum3(A, B, C);
    if (threadIdx.x == 0) {
        const float s = fmaxf((float)sqrt(A / (2.0 * (double)N)), 1e-30f);
        const double md = B / (double)N;
        const double var = fmax((C - B * md) / (double)(N - 1), 0.0);
        float* st = stats + 4 * (size_t)blockIdx.x;
        st[0] = s;
        st[1] = (float)((double)ref + md);
        st[2] = fmaxf((float)sqrt(var), 1e-30f);
        st[3] = log10f(s * (float)(P - 1));
    }
}

// X[f] = (straight x, y, marched x, y) / s, (phase - mean) / sd, log10(s (P - 1)).
__global__ void sur_encode_write_kernel(const float* __restrict__ maps, int P, const float* __restrict__ stats,
                                        float* __restrict__ X)
{
    const size_t N = (size_t)P * P;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const float* __restrict__ m = maps + (size_t)blockIdx.y * 5 * N;
    float* __restrict__ x = X + (size_t)blockIdx.y * 6 * N;
    const float4 st = reinterpret_cast<const float4*>(stats)[blockIdx.y];
    x[p] = m[3 * N + p] / st.x;
    x[N + p] = m[4 * N + p] / st.x;
    x[2 * N + p] = m[p] / st.x;
    x[3 * N + p] = m[N + p] / st.x;
    x[4 * N + p] = (m[2 * N + p] - st.y) / st.z;
    x[5 * N + p] = st.w;
}

// theta = marched deflection + s / gain * network output (planes 0, 1), and
// the marched deflection alone when theta_march is given.
__global__ void sur_decode_kernel(const float* __restrict__ maps, const float* __restrict__ net,
                                  const float* __restrict__ stats, const float* __restrict__ gain, int P,
                                  float* __restrict__ theta, float* __restrict__ theta_march)
{
    const size_t N = (size_t)P * P;
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const size_t f = blockIdx.y;
    const float s = stats[4 * f];
    const float* __restrict__ m = maps + f * 5 * N;
    const float* __restrict__ o = net + f * 3 * N;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const float mv = m[c * N + p];
        theta[(f * 2 + c) * N + p] = fmaf(s / gain[c], o[c * N + p], mv);
        if (theta_march) theta_march[(f * 2 + c) * N + p] = mv;
    }
}

// est[f] = kappa ||I_net - I_march|| / ||I_net|| (infinite when I_net is zero);
// FP32 sums per thread, FP64 across the block.
__global__ void __launch_bounds__(kSurStatThreads) sur_estimate_kernel(const float* __restrict__ In,
                                                                       const float* __restrict__ Im, int P,
                                                                       double kappa, float* __restrict__ est)
{
    const size_t N = (size_t)P * P;
    const float* __restrict__ a_ = In + (size_t)blockIdx.x * N;
    const float* __restrict__ b_ = Im + (size_t)blockIdx.x * N;
    float a = 0.f, b = 0.f;
    for (size_t p = threadIdx.x; p < N; p += kSurStatThreads) {
        const float x = a_[p], d = x - b_[p];
        a = fmaf(d, d, a);
        b = fmaf(x, x, b);
    }
    double A = a, B = b, C = 0.0;
    block_sum3(A, B, C);
    if (threadIdx.x == 0) est[blockIdx.x] = B > 0.0 ? (float)(kappa * sqrt(A / B)) : __int_as_float(0x7f800000);
}

}  // namespace

extern "C" int tt_surrogate_encode(const float* maps, int n, int P, float* X, float* stats, void* stream)
{
    if (!maps || !X || !stats || n < 1 || n > 65535 || P < 2 || P > 46340)
        return tt::invalid("surrogate_encode: bad arguments");
    if ((reinterpret_cast<uintptr_t>(stats) & 15) != 0) return tt::invalid("surrogate_encode: stats not 16-byte aligned");
    cudaStream_t s = tt::as_stream(stream);
    sur_encode_stats_kernel<<<n, kSurStatThreads, 0, s>>>(maps, P, stats);
    TT_TRY(tt::launch_status("surrogate_encode stats"));
    const size_t N = (size_t)P * P;
    sur_encode_write_kernel<<<dim3((unsigned)((N + 255) / 256), n), 256, 0, s>>>(maps, P, stats, X);
    return tt::launch_status("surrogate_encode");
}

extern "C" int tt_surrogate_decode(const float* maps, const float* net, const float* stats, const float* gain, int n,
                                   int P, float* theta, float* theta_march, void* stream)
{
    if (!maps || !net || !stats || !gain || !theta || n < 1 || n > 65535 || P < 2 || P > 46340)
        return tt::invalid("surrogate_decode: bad arguments");
    const size_t N = (size_t)P * P;
    sur_decode_kernel<<<dim3((unsigned)((N + 255) / 256), n), 256, 0, tt::as_stream(stream)>>>(
        maps, net, stats, gain, P, theta, theta_march);
    return tt::launch_status("surrogate_decode");
}

extern "C" int tt_surrogate_estimate(const float* I_net, const float* I_march, int n, int P, double kappa, float* est,
                                     void* stream)
{
    if (!I_net || !I_march || !est || n < 1 || n > 65535 || P < 2 || P > 46340 || !(kappa >= 0))
        return tt::invalid("surrogate_estimate: bad arguments");
    sur_estimate_kernel<<<n, kSurStatThreads, 0, tt::as_stream(stream)>>>(I_net, I_march, P, kappa, est);
    return tt::launch_status("surrogate_estimate");
}
