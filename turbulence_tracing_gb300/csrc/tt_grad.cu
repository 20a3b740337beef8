// K1: density gradient.
//
//  * tt_calc_dndr -- FP64 drop-in for ElectronCube.calc_dndr
//    (particle_tracking/particle_tracker.py:220-237).  Reproduces numpy's
//    arithmetic operation by operation (this file is compiled with
//    -fmad=false and uses round-to-nearest intrinsics), so ne_nc and dnd{x,y,z}
//    are bit-identical to the reference's numpy arrays.
//  * tt_volume_plan / tt_volume_build -- the FP32 brick-tiled node volume the
//    persistent tracer reads (layout documented in include/turbotrace.h).
//
// Both are HBM-streaming kernels: FP64 reads 8 B and writes 32 B per voxel,
// FP32 reads ~4-8 B and writes 16 B per stored node (apron nodes included).
#include <math.h>

#include <mutex>

#include "tt_common.cuh"

namespace {

// ---------------------------------------------------------------------------
// numpy.gradient coefficient tables, one per axis, in the workspace:
//   hdr[0] = uniform flag, hdr[1] = d0 (scalar spacing), hdr[2] = dx_first,
//   hdr[3] = dx_last, then a[n], b[n], c[n] (interior nodes 1..n-2).
struct AxisCoef {
    const double* hdr;
    const double* a;
    const double* b;
    const double* c;
};

__host__ __device__ inline size_t axis_table_doubles(int n) { return 4 + 3 * (size_t)n; }

__global__ void grad_coef_kernel(const double* __restrict__ coord, int n, double* __restrict__ tab)
{
    // one block per axis; the uniform test needs every diff
    __shared__ int nonuniform;
    if (threadIdx.x == 0) nonuniform = 0;
    __syncthreads();
    const double d0 = __dsub_rn(coord[1], coord[0]);
    for (int i = threadIdx.x; i < n - 1; i += blockDim.x) {
        const double di = __dsub_rn(coord[i + 1], coord[i]);
        if (di != d0) nonuniform = 1;  // benign race: every writer stores 1
    }
    __syncthreads();
    double* a = tab + 4;
    double* b = a + n;
    double* c = b + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double av = 0.0, bv = 0.0, cv = 0.0;
        if (i >= 1 && i <= n - 2) {
            const double dx1 = __dsub_rn(coord[i], coord[i - 1]);
            const double dx2 = __dsub_rn(coord[i + 1], coord[i]);
            const double s12 = __dadd_rn(dx1, dx2);
            av = __ddiv_rn(-dx2, __dmul_rn(dx1, s12));
            bv = __ddiv_rn(__dsub_rn(dx2, dx1), __dmul_rn(dx1, dx2));
            cv = __ddiv_rn(dx1, __dmul_rn(dx2, s12));
        }
        a[i] = av;
        b[i] = bv;
        c[i] = cv;
    }
    if (threadIdx.x == 0) {
        tab[0] = nonuniform ? 0.0 : 1.0;
        tab[1] = d0;
        tab[2] = d0;
        tab[3] = __dsub_rn(coord[n - 1], coord[n - 2]);
    }
}

template <typename T>
__global__ void ne_nc_kernel(const T* __restrict__ ne, size_t nv, double nc, double ne_max,
                             double* __restrict__ ne_nc)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv;
         i += (size_t)gridDim.x * blockDim.x) {
        double q = __ddiv_rn((double)ne[i], nc);
        if (q > ne_max) q = ne_max;
        ne_nc[i] = q;
    }
}

// numpy.gradient along one axis at index i with element stride `st`.
__device__ inline double grad1(const double* __restrict__ f, size_t idx, size_t st, int i, int n,
                               const double* __restrict__ tab)
{
    const bool uniform = tab[0] != 0.0;
    if (i == 0) {
        return __ddiv_rn(__dsub_rn(f[idx + st], f[idx]), tab[2]);
    }
    if (i == n - 1) {
        return __ddiv_rn(__dsub_rn(f[idx], f[idx - st]), uniform ? tab[1] : tab[3]);
    }
    const double fm = f[idx - st], f0 = f[idx], fp = f[idx + st];
    if (uniform) return __ddiv_rn(__dsub_rn(fp, fm), __dmul_rn(2.0, tab[1]));
    const double* a = tab + 4;
    const double* b = a + n;
    const double* c = b + n;
    return __dadd_rn(__dadd_rn(__dmul_rn(a[i], fm), __dmul_rn(b[i], f0)), __dmul_rn(c[i], fp));
}

__global__ void dndr_grad_kernel(const double* __restrict__ q, int nx, int ny, int nz,
                                 const double* __restrict__ tx, const double* __restrict__ ty,
                                 const double* __restrict__ tz, double k,
                                 double* __restrict__ gx, double* __restrict__ gy,
                                 double* __restrict__ gz)
{
    const size_t nv = (size_t)nx * ny * nz;
    const size_t syz = (size_t)ny * nz;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < nv;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(idx % nz);
        const size_t r = idx / nz;
        const int iy = (int)(r % ny);
        const int ix = (int)(r / ny);
        gx[idx] = __dmul_rn(k, grad1(q, idx, syz, ix, nx, tx));
        gy[idx] = __dmul_rn(k, grad1(q, idx, (size_t)nz, iy, ny, ty));
        gz[idx] = __dmul_rn(k, grad1(q, idx, 1, iz, nz, tz));
    }
}

int grid_for(size_t n, int block)
{
    size_t g = (n + block - 1) / block;
    const size_t cap = (size_t)tt::sm_count() * 32;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

extern "C" size_t tt_calc_dndr_workspace_bytes(int nx, int ny, int nz)
{
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    return sizeof(double) * (axis_table_doubles(nx) + axis_table_doubles(ny) + axis_table_doubles(nz));
}

extern "C" int tt_calc_dndr(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x,
                            const double* y, const double* z, double lwl, double ne_max,
                            double* ne_nc, double* dndx, double* dndy, double* dndz,
                            double* omega_out, void* workspace, size_t workspace_bytes,
                            void* stream)
{
    if (nx < 2 || ny < 2 || nz < 2)
        return tt::invalid("calc_dndr: every axis needs at least 2 points (numpy.gradient edge_order=1)");
    if (!ne || !x || !y || !z || !ne_nc || !dndx || !dndy || !dndz)
        return tt::invalid("calc_dndr: null pointer");
    if (ne_dtype != TT_F32 && ne_dtype != TT_F64) return tt::invalid("calc_dndr: ne_dtype must be TT_F32 or TT_F64");
    if (!(lwl > 0.0)) return tt::invalid("calc_dndr: lwl must be > 0");
    const size_t need = tt_calc_dndr_workspace_bytes(nx, ny, nz);
    if (!workspace || workspace_bytes < need) {
        tt::set_detail("calc_dndr: workspace needs %zu bytes", need);
        return TT_ERR_WORKSPACE_TOO_SMALL;
    }
    // Scalars formed the way Python forms them at particle_tracker.py:227-228, 235.
    const double omega = (2.0 * M_PI) * (TT_C_LIGHT / lwl);
    const double nc = 3.14207787e-4 * (omega * omega);
    const double k = -0.5 * (TT_C_LIGHT * TT_C_LIGHT);
    if (omega_out) *omega_out = omega;

    cudaStream_t s = tt::as_stream(stream);
    double* tx = static_cast<double*>(workspace);
    double* ty = tx + axis_table_doubles(nx);
    double* tz = ty + axis_table_doubles(ny);
    grad_coef_kernel<<<1, 256, 0, s>>>(x, nx, tx);
    grad_coef_kernel<<<1, 256, 0, s>>>(y, ny, ty);
    grad_coef_kernel<<<1, 256, 0, s>>>(z, nz, tz);
    TT_TRY(tt::launch_status("calc_dndr coefficient kernel"));
    const size_t nv = (size_t)nx * ny * nz;
    if (ne_dtype == TT_F64)
        ne_nc_kernel<double><<<grid_for(nv, 256), 256, 0, s>>>(static_cast<const double*>(ne), nv, nc,
                                                                ne_max, ne_nc);
    else
        ne_nc_kernel<float><<<grid_for(nv, 256), 256, 0, s>>>(static_cast<const float*>(ne), nv, nc,
                                                               ne_max, ne_nc);
    TT_TRY(tt::launch_status("calc_dndr ne_nc kernel"));
    dndr_grad_kernel<<<grid_for(nv, 256), 256, 0, s>>>(ne_nc, nx, ny, nz, tx, ty, tz, k, dndx, dndy, dndz);
    return tt::launch_status("calc_dndr gradient kernel");
}

// ===========================================================================
// calc_dndr without any allocation.
//
// For callers that cannot allocate device memory for the workspace: a host
// application whose memory manager owns every device buffer (a framework's
// caching allocator or a fixed device pool handed out up front) and forbids
// allocations behind its back.  The numpy.gradient coefficient tables then
// live in the fixed array below, which every GPU that loads this library
// keeps until the process exits.
// ===========================================================================
namespace {

constexpr int kNoAllocMaxAxis = 8192;  // nodes per axis the fixed tables can hold
constexpr size_t kNoAllocDoubles = 3 * (4 + 3 * (size_t)kNoAllocMaxAxis);  // 590 KB

}  // namespace

static __device__ __align__(256) double g_calc_dndr_tables[kNoAllocDoubles];

namespace {

std::mutex g_noalloc_mutex;
double* g_noalloc_tables[64] = {nullptr};  // device address of g_calc_dndr_tables, per device

// Device address of the fixed tables on the current device, looked up once per
// device at that device's first call (the host-side name of a __device__ array
// is not a device address; cudaGetSymbolAddress gives it, with the device
// current, and allocates nothing).  The address belongs to the device's
// context: a device reset after the first call is not supported.
int noalloc_tables(double** out)
{
    int dev = 0;
    TT_TRY(tt::cuda_status(cudaGetDevice(&dev), "calc_dndr_noalloc: cudaGetDevice"));
    if (dev < 0 || dev >= 64) return tt::invalid("calc_dndr_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_tables[dev]) {
        void* p = nullptr;
        TT_TRY(tt::cuda_status(cudaGetSymbolAddress(&p, g_calc_dndr_tables),
                               "calc_dndr_noalloc: cudaGetSymbolAddress"));
        g_noalloc_tables[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_tables[dev];
    return TT_OK;
}

}  // namespace

extern "C" int tt_calc_dndr_noalloc(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x,
                                    const double* y, const double* z, double lwl, double ne_max, double* ne_nc,
                                    double* dndx, double* dndy, double* dndz, double* omega_out, void* stream)
{
    if (nx < 2 || ny < 2 || nz < 2)
        return tt::invalid("calc_dndr_noalloc: every axis needs at least 2 points (numpy.gradient edge_order=1)");
    if (nx > kNoAllocMaxAxis || ny > kNoAllocMaxAxis || nz > kNoAllocMaxAxis) {
        tt::set_detail("calc_dndr_noalloc: at most %d nodes per axis (got %d x %d x %d); use tt_calc_dndr "
                       "with a workspace for larger grids", kNoAllocMaxAxis, nx, ny, nz);
        return TT_ERR_TOO_LARGE;
    }
    if (!ne || !x || !y || !z || !ne_nc || !dndx || !dndy || !dndz)
        return tt::invalid("calc_dndr_noalloc: null pointer");
    if (ne_dtype != TT_F32 && ne_dtype != TT_F64)
        return tt::invalid("calc_dndr_noalloc: ne_dtype must be TT_F32 or TT_F64");
    if (!(lwl > 0.0)) return tt::invalid("calc_dndr_noalloc: lwl must be > 0");
    double* tx = nullptr;
    TT_TRY(noalloc_tables(&tx));
    const double omega = (2.0 * M_PI) * (TT_C_LIGHT / lwl);
    const double nc = 3.14207787e-4 * (omega * omega);
    const double k = -0.5 * (TT_C_LIGHT * TT_C_LIGHT);
    if (omega_out) *omega_out = omega;
    cudaStream_t s = tt::as_stream(stream);
    // every table entry the gradient kernel reads is rewritten here first, so
    // nothing needs clearing between calls
    double* ty = tx + axis_table_doubles(nx);
    double* tz = ty + axis_table_doubles(ny);
    grad_coef_kernel<<<1, 256, 0, s>>>(x, nx, tx);
    grad_coef_kernel<<<1, 256, 0, s>>>(y, ny, ty);
    grad_coef_kernel<<<1, 256, 0, s>>>(z, nz, tz);
    TT_TRY(tt::launch_status("calc_dndr_noalloc coefficient kernel"));
    const size_t nv = (size_t)nx * ny * nz;
    if (ne_dtype == TT_F64)
        ne_nc_kernel<double><<<grid_for(nv, 256), 256, 0, s>>>(static_cast<const double*>(ne), nv, nc,
                                                                ne_max, ne_nc);
    else
        ne_nc_kernel<float><<<grid_for(nv, 256), 256, 0, s>>>(static_cast<const float*>(ne), nv, nc,
                                                               ne_max, ne_nc);
    TT_TRY(tt::launch_status("calc_dndr_noalloc ne_nc kernel"));
    dndr_grad_kernel<<<grid_for(nv, 256), 256, 0, s>>>(ne_nc, nx, ny, nz, tx, ty, tz, k, dndx, dndy, dndz);
    return tt::launch_status("calc_dndr_noalloc gradient kernel");
}

// ===========================================================================
// FP32 brick volume
// ===========================================================================
namespace {

__device__ __host__ inline uint32_t spread3(uint32_t v)
{
    return (v & 1u) | ((v & 2u) << 1) | ((v & 4u) << 2);
}
__device__ __host__ inline uint32_t compact3(uint32_t m)
{
    return (m & 1u) | ((m >> 1) & 2u) | ((m >> 2) & 4u);
}

struct VolGeom {
    int n[3];
    int strides[3];  // element strides of a, b, c in the C-ordered density
    int tiles[2];
    int st[2];
    int bricks_c;
    int bd;             // nodes per brick along c
    int brick_f4;       // float4 per brick (25 bd)
    long long tile_f4;  // float4 per tile column
    float inv_nc;
    float q_max;        // ne_max
    float ne_clip;      // ne_max * nc, clip in density units
    float scale_int[3]; // -0.5 / nc * spacing_c / (2 h_axis)
    float scale_edge[3];// -0.5 / nc * spacing_c / h_axis
    double scale_int_d[3];
    double scale_edge_d[3];
};

template <typename T>
__device__ inline void diff_axis(const T* __restrict__ ne, size_t base, int i, int n, int stride,
                                 const VolGeom& g, int ax, float& out)
{
    size_t ip, im;
    bool edge;
    if (i == 0) { ip = base + stride; im = base; edge = true; }
    else if (i == n - 1) { ip = base; im = base - stride; edge = true; }
    else { ip = base + stride; im = base - stride; edge = false; }
    if (sizeof(T) == 8) {
        double a = (double)ne[ip], b = (double)ne[im];
        const double clip = (double)g.ne_clip;
        a = a > clip ? clip : a;
        b = b > clip ? clip : b;
        out = (float)((a - b) * (edge ? g.scale_edge_d[ax] : g.scale_int_d[ax]));
    } else {
        float a = (float)ne[ip], b = (float)ne[im];
        a = a > g.ne_clip ? g.ne_clip : a;
        b = b > g.ne_clip ? g.ne_clip : b;
        out = (a - b) * (edge ? g.scale_edge[ax] : g.scale_int[ax]);  // a - b exact when within 2x
    }
}

template <typename T>
__global__ void volume_build_kernel(const T* __restrict__ ne, VolGeom g, long long total,
                                    float4* __restrict__ nodes)
{
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < total;
         li += (long long)gridDim.x * blockDim.x) {
        const long long tile = li / g.tile_f4;
        const int within = (int)(li - tile * g.tile_f4);
        const int brick = within / g.brick_f4;
        const int r = within - brick * g.brick_f4;
        const int al = r / (5 * g.bd);
        const int bl = (r / g.bd) % 5;
        const int cl = r & (g.bd - 1);
        const long long st = tile >> 6;
        const uint32_t m = (uint32_t)(tile & 63);
        const int ta = (int)(st / g.st[1]) * 8 + (int)compact3(m);
        const int tb = (int)(st % g.st[1]) * 8 + (int)compact3(m >> 1);
        const int a = ta * 4 + al, b = tb * 4 + bl, c = brick * g.bd + cl;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (a < g.n[0] && b < g.n[1] && c < g.n[2]) {
            const size_t base = (size_t)a * g.strides[0] + (size_t)b * g.strides[1] + (size_t)c * g.strides[2];
            diff_axis(ne, base, a, g.n[0], g.strides[0], g, 0, v.x);
            diff_axis(ne, base, b, g.n[1], g.strides[1], g, 1, v.y);
            diff_axis(ne, base, c, g.n[2], g.strides[2], g, 2, v.z);
            float q = (float)ne[base] * g.inv_nc;
            v.w = q > g.q_max ? g.q_max : q;
        }
        nodes[li] = v;
    }
}

bool uniform_axis(const double* c, int n, double* origin, double* spacing)
{
    const double d = (c[n - 1] - c[0]) / (n - 1);
    if (!(d > 0.0)) return false;
    for (int i = 0; i < n; ++i)
        if (fabs(c[i] - (c[0] + i * d)) > 1e-6 * d) return false;
    *origin = c[0];
    *spacing = d;
    return true;
}

}  // namespace

extern "C" int tt_volume_plan(int nx, int ny, int nz, const double* x_host, const double* y_host,
                              const double* z_host, int probing_axis, double lwl, double ne_max,
                              tt_volume* vol)
{
    if (!vol || !x_host || !y_host || !z_host) return tt::invalid("volume_plan: null pointer");
    if (nx < 2 || ny < 2 || nz < 2) return tt::invalid("volume_plan: every axis needs at least 2 points");
    if (probing_axis < 0 || probing_axis > 2) return tt::invalid("volume_plan: probing_axis must be 0, 1 or 2");
    if (!(lwl > 0.0)) return tt::invalid("volume_plan: lwl must be > 0");
    const int n_phys[3] = {nx, ny, nz};
    const double* cs[3] = {x_host, y_host, z_host};
    int ax[3];
    ax[2] = probing_axis;
    ax[0] = probing_axis == 0 ? 1 : 0;
    ax[1] = probing_axis == 2 ? 1 : 2;
    tt_volume v;
    for (int i = 0; i < 3; ++i) {
        v.axis[i] = ax[i];
        v.n[i] = n_phys[ax[i]];
        if (!uniform_axis(cs[ax[i]], v.n[i], &v.origin[i], &v.spacing[i])) {
            tt::set_detail("volume_plan: coordinates along axis %d are not uniformly spaced; "
                           "the FP32 tracer needs a uniform grid", ax[i]);
            return TT_ERR_UNSUPPORTED;
        }
    }
    for (int i = 0; i < 2; ++i) {
        const int cells = v.n[i] - 1;
        v.tiles[i] = (cells + 3) / 4;
        v.supertiles[i] = (v.tiles[i] + 7) / 8;
    }
    v.brick_depth = 8;
    v.bricks_c = (v.n[2] + v.brick_depth - 1) / v.brick_depth;
    v.omega = (2.0 * M_PI) * (TT_C_LIGHT / lwl);
    v.ne_max = ne_max;
    v.n_float4 = (int64_t)v.supertiles[0] * v.supertiles[1] * 64 * (int64_t)v.bricks_c * 25 * v.brick_depth;
    v.nodes = nullptr;
    *vol = v;
    return TT_OK;
}

extern "C" int tt_volume_set_brick_depth(tt_volume* vol, int brick_depth)
{
    if (!vol) return tt::invalid("volume_set_brick_depth: null volume");
    if (brick_depth < 4 || brick_depth > 32 || (brick_depth & (brick_depth - 1)) != 0)
        return tt::invalid("volume_set_brick_depth: depth must be 4, 8, 16 or 32");
    vol->brick_depth = brick_depth;
    vol->bricks_c = (vol->n[2] + brick_depth - 1) / brick_depth;
    vol->n_float4 = (int64_t)vol->supertiles[0] * vol->supertiles[1] * 64 * (int64_t)vol->bricks_c * 25 * brick_depth;
    vol->nodes = nullptr;
    return TT_OK;
}

extern "C" int tt_volume_build(const tt_volume* vol, const void* ne, int ne_dtype, void* stream)
{
    if (!vol || !ne || !vol->nodes) return tt::invalid("volume_build: null pointer");
    if (((uintptr_t)vol->nodes & 15u) != 0) return tt::invalid("volume_build: node buffer must be 16-byte aligned");
    if (ne_dtype != TT_F32 && ne_dtype != TT_F64) return tt::invalid("volume_build: bad ne_dtype");
    VolGeom g;
    int n_phys[3];
    for (int i = 0; i < 3; ++i) n_phys[vol->axis[i]] = vol->n[i];
    const int phys_stride[3] = {n_phys[1] * n_phys[2], n_phys[2], 1};
    const double nc = 3.14207787e-4 * (vol->omega * vol->omega);
    for (int i = 0; i < 3; ++i) {
        g.n[i] = vol->n[i];
        g.strides[i] = phys_stride[vol->axis[i]];
        const double base = -0.5 / nc * vol->spacing[2];
        g.scale_int_d[i] = base / (2.0 * vol->spacing[i]);
        g.scale_edge_d[i] = base / vol->spacing[i];
        g.scale_int[i] = (float)g.scale_int_d[i];
        g.scale_edge[i] = (float)g.scale_edge_d[i];
    }
    g.tiles[0] = vol->tiles[0];
    g.tiles[1] = vol->tiles[1];
    g.st[0] = vol->supertiles[0];
    g.st[1] = vol->supertiles[1];
    if (vol->brick_depth < 4 || vol->brick_depth > 32 || (vol->brick_depth & (vol->brick_depth - 1)) != 0)
        return tt::invalid("volume_build: bad brick_depth (use tt_volume_plan / tt_volume_set_brick_depth)");
    g.bricks_c = vol->bricks_c;
    g.bd = vol->brick_depth;
    g.brick_f4 = 25 * vol->brick_depth;
    g.tile_f4 = (long long)vol->bricks_c * g.brick_f4;
    g.inv_nc = (float)(1.0 / nc);
    g.q_max = (float)vol->ne_max;
    g.ne_clip = (float)(vol->ne_max * nc);
    const long long total = vol->n_float4;
    if (total != (long long)vol->supertiles[0] * vol->supertiles[1] * 64 * g.tile_f4)
        return tt::invalid("volume_build: descriptor is inconsistent (use tt_volume_plan)");
    cudaStream_t s = tt::as_stream(stream);
    float4* nodes = static_cast<float4*>(vol->nodes);
    if (ne_dtype == TT_F64)
        volume_build_kernel<double><<<grid_for((size_t)total, 256), 256, 0, s>>>(
            static_cast<const double*>(ne), g, total, nodes);
    else
        volume_build_kernel<float><<<grid_for((size_t)total, 256), 256, 0, s>>>(
            static_cast<const float*>(ne), g, total, nodes);
    return tt::launch_status("volume_build kernel");
}
