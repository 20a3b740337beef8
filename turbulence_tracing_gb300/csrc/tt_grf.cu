// K4: Gaussian random fields -- Philox4x32-10 noise, Hermitian spectral
// shaping on the half spectrum, cuFFT complex-to-real inverse transform.
//
//  * tt_grf_fft   replaces turboGen.gaussian3D_FFT (gaussian_fields/turboGen.py:488-537);
//    tt_grf_fft_nd also gaussian1D_FFT and gaussian2D_FFT (:388-485), the same
//    construction in one and two dimensions.
//  * tt_cos_field replaces the cosine-sum generators gaussian1Dcos, gaussian2Dcos,
//    gaussian3Dcos (:40-385): sums of random-phase modes at cell centres.
//  * tt_grf_field the band-limited, unit-variance field of the benchmark workloads.
//
// The shaping kernels write only the half spectrum (last axis 0..n/2) that a
// C2R transform reads; Hermitian symmetry of the full spectrum is implied by
// the transform, and on the self-paired planes (kz = 0, and kz = n/2 for even
// n) each pair (k, -k) gets conjugate values from one draw, so the transform's
// input is exactly Hermitian.  Both kernels stream the spectrum once (16 B
// per mode written); the FFT is a library call.
#include <cufft.h>
#include <math.h>

#include "tt_common.cuh"

namespace {

constexpr uint32_t kTagFFT = 0x47524630u;    // 'GRF0'
constexpr uint32_t kTagField = 0x47524631u;  // 'GRF1'

__device__ __host__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        if (r < 9) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
    }
}

// Two standard normals (Box-Muller) for mode counter `lin`.
__device__ inline void mode_noise(uint64_t lin, uint64_t seed, uint32_t tag, double& a, double& b)
{
    uint32_t c[4] = {(uint32_t)lin, (uint32_t)(lin >> 32), 0u, tag};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const double u0 = ((double)c[0] + 0.5) * (1.0 / 4294967296.0);
    const double u1 = ((double)c[1] + 0.5) * (1.0 / 4294967296.0);
    const double r = sqrt(-2.0 * log(u0));
    const double th = 2.0 * M_PI * u1;
    a = r * cos(th);
    b = r * sin(th);
}

// Noise for half-spectrum mode (i0, i1, i2) of an n x n x h grid with the
// conjugate-partner rule on self-paired planes.
__device__ inline void half_mode_noise(int i0, int i1, int i2, int n, int h, bool edge_plane, uint64_t seed,
                                       uint32_t tag, double& a, double& b)
{
    int s0 = i0, s1 = i1;
    bool conj = false, self = false;
    if (edge_plane) {
        const int p0 = (n - i0) % n, p1 = (n - i1) % n;
        const long long ls = (long long)i0 * n + i1, lp = (long long)p0 * n + p1;
        if (lp < ls) {
            s0 = p0;
            s1 = p1;
            conj = true;
        } else if (lp == ls) {
            self = true;
        }
    }
    const uint64_t lin = ((uint64_t)s0 * n + (uint64_t)s1) * (uint64_t)h + (uint64_t)i2;
    mode_noise(lin, seed, tag, a, b);
    if (conj) b = -b;
    if (self) b = 0.0;
}

// gaussian{1,2,3}D_FFT spectrum: M = 2N+1 points per axis, half length H = N+1
// on the last axis; dim < 3 leaves the leading axes of size 1 (index 0).
__global__ void shape_fft_kernel(uint64_t seed, int dim, int N, const double* __restrict__ sqrt_p,
                                 const double* __restrict__ Wr, const double* __restrict__ Wi,
                                 cufftDoubleComplex* __restrict__ F)
{
    const int M = 2 * N + 1, H = N + 1;
    const int M1 = dim >= 2 ? M : 1, M0 = dim >= 3 ? M : 1;
    const long long total = (long long)M0 * M1 * H;
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < total;
         li += (long long)gridDim.x * blockDim.x) {
        const int i2 = (int)(li % H);
        const long long r = li / H;
        const int i1 = (int)(r % M1);
        const int i0 = (int)(r / M1);
        double re, im;
        if (Wr) {
            // reference: W = (Wr + flip(Wr)) + 1j (Wi - flip(Wi)) on the centred grid;
            // standard index i sits at centred (i + N) % M, its mirror at (N - i) % M.
            const long long c0 = dim >= 3 ? (i0 + N) % M : 0, f0 = dim >= 3 ? (N - i0 + M) % M : 0;
            const long long c1 = dim >= 2 ? (i1 + N) % M : 0, f1 = dim >= 2 ? (N - i1 + M) % M : 0;
            const long long c = (c0 * M1 + c1) * M + (i2 + N) % M;
            const long long f = (f0 * M1 + f1) * M + (N - i2 + M) % M;
            re = Wr[c] + Wr[f];
            im = Wi[c] - Wi[f];
        } else {
            double a, b;
            // tags 'GRF0' (3D), 'GRF2' (2D), 'GRF3' (1D): one stream per dimension
            half_mode_noise(i0, i1, i2, M, H, i2 == 0, seed, dim == 3 ? kTagFFT : kTagFFT + (uint32_t)(4 - dim),
                            a, b);
            re = a * M_SQRT2;  // variance 2 per part, as Wr(k) + Wr(-k)
            im = b * M_SQRT2;
        }
        const double s = sqrt_p[li];
        cufftDoubleComplex v;
        v.x = re * s;
        v.y = im * s;
        if (li == 0) {
            v.x = 0.0;
            v.y = 0.0;
        }
        F[li] = v;
    }
}

// Cosine-sum fields (turboGen.py:40-385) at cell centres xc_i = dx/2 + i dx (and y, z):
//   dim 1: sum_m amp_m sqrt2 cos(kx xc + p0)
//   dim 2: sum_m amp_m sqrt2 (cos(kx xc + ky yc + p0) + cos(kx xc - ky yc + p1))
//   dim 3: sum_m amp_m sqrt2 (cos(kx xc + ky yc + kz zc + p0) + cos(kx xc + ky yc - kz zc + p1)
//                           + cos(kx xc - ky yc + kz zc + p2) + cos(kx xc - ky yc - kz zc + p3))
// with the reference's operation order (explicitly rounded, no contraction).
// k: (3, nm) wavevectors, p: (4, nm) phases, amp: (nm); out C-ordered (nx[, ny[, nz]]).
__global__ void cos_field_kernel(int dim, int nx, int ny, int nz, double dx, double dy, double dz, int nm,
                                 const double* __restrict__ k, const double* __restrict__ p,
                                 const double* __restrict__ amp, double* __restrict__ out)
{
    const long long total = (long long)nx * ny * nz;
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < total;
         li += (long long)gridDim.x * blockDim.x) {
        const int kk = (int)(li % nz);
        const long long r = li / nz;
        const int j = (int)(r % ny);
        const int i = (int)(r / ny);
        const double xc = __dadd_rn(dx / 2.0, __dmul_rn((double)i, dx));
        const double yc = __dadd_rn(dy / 2.0, __dmul_rn((double)j, dy));
        const double zc = __dadd_rn(dz / 2.0, __dmul_rn((double)kk, dz));
        double sum = 0.0;
        for (int m = 0; m < nm; ++m) {
            const double ax = __dmul_rn(k[m], xc);
            const double w = __dmul_rn(amp[m], M_SQRT2);
            double c;
            if (dim == 1) {
                c = cos(__dadd_rn(ax, p[m]));
            } else {
                const double ay = __dmul_rn(k[nm + m], yc);
                const double xpy = __dadd_rn(ax, ay), xmy = __dsub_rn(ax, ay);
                if (dim == 2) {
                    c = __dadd_rn(cos(__dadd_rn(xpy, p[m])), cos(__dadd_rn(xmy, p[nm + m])));
                } else {
                    const double az = __dmul_rn(k[2 * nm + m], zc);
                    c = __dadd_rn(__dadd_rn(__dadd_rn(cos(__dadd_rn(__dadd_rn(xpy, az), p[m])),
                                                      cos(__dadd_rn(__dsub_rn(xpy, az), p[nm + m]))),
                                            cos(__dadd_rn(__dadd_rn(xmy, az), p[2 * nm + m]))),
                                  cos(__dadd_rn(__dsub_rn(xmy, az), p[3 * nm + m])));
                }
            }
            sum = __dadd_rn(sum, __dmul_rn(w, c));
        }
        out[li] = sum;
    }
}

__global__ void scale_kernel(double* __restrict__ x, long long n, double s)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] *= s;
}

// workload field spectrum on n x n x h (h = n/2+1); band on integer m.m
__global__ void shape_field_kernel(uint64_t seed, int n, double mlo2, double mhi2, double alpha4,
                                   cufftDoubleComplex* __restrict__ F)
{
    const int h = n / 2 + 1;
    const long long total = (long long)n * n * h;
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < total;
         li += (long long)gridDim.x * blockDim.x) {
        const int i2 = (int)(li % h);
        const long long r = li / h;
        const int i1 = (int)(r % n);
        const int i0 = (int)(r / n);
        const long long m0 = i0 <= (n - 1) / 2 ? i0 : i0 - n;
        const long long m1 = i1 <= (n - 1) / 2 ? i1 : i1 - n;
        const long long m2i = i2 <= (n - 1) / 2 ? i2 : i2 - n;
        const double m2 = (double)(m0 * m0 + m1 * m1 + m2i * m2i);
        cufftDoubleComplex v;
        v.x = 0.0;
        v.y = 0.0;
        if (m2 > 0.0 && m2 >= mlo2 && m2 <= mhi2) {
            const bool edge = i2 == 0 || ((n % 2 == 0) && i2 == h - 1);
            double a, b;
            half_mode_noise(i0, i1, i2, n, h, edge, seed, kTagField, a, b);
            const double amp = pow(m2, alpha4);
            v.x = a * amp;
            v.y = b * amp;
        }
        F[li] = v;
    }
}

// deterministic two-level reduction of sum and sum of squares over the
// in-place C2R output (rows padded to 2h doubles)
__global__ void stats_partial_kernel(const double* __restrict__ f, int n, int rowpad, double* __restrict__ part)
{
    __shared__ double s1[256], s2[256];
    const long long total = (long long)n * n * n;
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long row = i / n;
        const int k = (int)(i - row * n);
        const double v = f[row * rowpad + k];
        a += v;
        b += v * v;
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s1[0];
        part[2 * blockIdx.x + 1] = s2[0];
    }
}

__global__ void stats_final_kernel(double* __restrict__ part, int nparts, double count)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < nparts; ++i) {
            a += part[2 * i];
            b += part[2 * i + 1];
        }
        const double mean = a / count;
        double var = b / count - mean * mean;
        if (!(var > 0.0)) var = 1.0;
        part[0] = mean;
        part[1] = 1.0 / sqrt(var);
    }
}

template <typename T>
__global__ void density_kernel(const double* __restrict__ f, int n, int rowpad, const double* __restrict__ st,
                               double ne0, double delta, T* __restrict__ out)
{
    const double mean = st[0], inv_std = st[1];
    const long long total = (long long)n * n * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long row = i / n;
        const int k = (int)(i - row * n);
        const double g = (f[row * rowpad + k] - mean) * inv_std;
        double ne = ne0 * (1.0 + delta * g);
        if (ne < 0.0) ne = 0.0;
        out[i] = (T)ne;
    }
}

__global__ void philox_kernel(uint64_t seed, uint32_t tag, long long count, uint32_t* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        uint32_t c[4] = {(uint32_t)i, (uint32_t)((unsigned long long)i >> 32), 0u, tag};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        for (int k = 0; k < 4; ++k) out[(size_t)k * count + i] = c[k];
    }
}

int grid_for(long long n)
{
    long long g = (n + 255) / 256;
    const long long cap = (long long)tt::sm_count() * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

int cufft_status(cufftResult r, const char* where)
{
    if (r == CUFFT_SUCCESS) return TT_OK;
    tt::set_detail("%s: cuFFT error %d", where, (int)r);
    return TT_ERR_CUFFT;
}

int make_z2d_plan(cufftHandle p, int dim, int n, size_t* w)
{
    if (dim == 1) return cufft_status(cufftMakePlan1d(p, n, CUFFT_Z2D, 1, w), "cufftMakePlan1d");
    if (dim == 2) return cufft_status(cufftMakePlan2d(p, n, n, CUFFT_Z2D, w), "cufftMakePlan2d");
    return cufft_status(cufftMakePlan3d(p, n, n, n, CUFFT_Z2D, w), "cufftMakePlan3d");
}

// Size of the Z2D work area cuFFT needs for an n^dim transform (plan made and destroyed).
int z2d_work_bytes(int n, size_t* bytes, int dim = 3)
{
    cufftHandle p;
    TT_TRY(cufft_status(cufftCreate(&p), "cufftCreate"));
    int rc = cufft_status(cufftSetAutoAllocation(p, 0), "cufftSetAutoAllocation");
    size_t w = 0;
    if (rc == TT_OK) rc = make_z2d_plan(p, dim, n, &w);
    cufftDestroy(p);
    *bytes = w;
    return rc;
}

int run_z2d(int n, cufftDoubleComplex* in, double* out, void* work, cudaStream_t s, int dim = 3)
{
    cufftHandle p;
    TT_TRY(cufft_status(cufftCreate(&p), "cufftCreate"));
    size_t w = 0;
    int rc = cufft_status(cufftSetAutoAllocation(p, 0), "cufftSetAutoAllocation");
    if (rc == TT_OK) rc = make_z2d_plan(p, dim, n, &w);
    if (rc == TT_OK) rc = cufft_status(cufftSetWorkArea(p, work), "cufftSetWorkArea");
    if (rc == TT_OK) rc = cufft_status(cufftSetStream(p, s), "cufftSetStream");
    if (rc == TT_OK) rc = cufft_status(cufftExecZ2D(p, in, out), "cufftExecZ2D");
    cufftDestroy(p);
    return rc;
}

struct FftWs {
    size_t spec_off, work_off, total;
};

FftWs fft_ws(int N, size_t work, int dim = 3)
{
    const long long M = 2LL * N + 1, H = N + 1;
    const long long lead = dim == 3 ? M * M : (dim == 2 ? M : 1);
    FftWs L;
    L.spec_off = 0;
    L.work_off = tt::align_up(sizeof(cufftDoubleComplex) * (size_t)(lead * H), 256);
    L.total = tt::align_up(L.work_off + work, 256);
    return L;
}

struct FieldWs {
    size_t spec_off, part_off, work_off, total;
    int nparts;
};

FieldWs field_ws(int n, size_t work)
{
    const long long h = n / 2 + 1;
    FieldWs L;
    L.nparts = 1024;
    L.spec_off = 0;  // in-place: complex half spectrum, then the real field in the same bytes
    L.part_off = tt::align_up(sizeof(cufftDoubleComplex) * (size_t)((long long)n * n * h), 256);
    L.work_off = tt::align_up(L.part_off + sizeof(double) * 2 * L.nparts, 256);
    L.total = tt::align_up(L.work_off + work, 256);
    return L;
}

}  // namespace

extern "C" size_t tt_grf_fft_nd_workspace_bytes(int dim, int N)
{
    if (N < 1 || dim < 1 || dim > 3) return 0;
    size_t w = 0;
    if (z2d_work_bytes(2 * N + 1, &w, dim) != TT_OK) return 0;
    return fft_ws(N, w, dim).total;
}

extern "C" int tt_grf_fft_nd(uint64_t seed, int dim, int N, const double* sqrt_p, const double* Wr, const double* Wi,
                             double* out, void* workspace, size_t workspace_bytes, void* stream)
{
    if (dim < 1 || dim > 3) return tt::invalid("grf_fft: dim must be 1, 2 or 3");
    if (N < 1) return tt::invalid("grf_fft: N must be >= 1");
    if (!sqrt_p || !out) return tt::invalid("grf_fft: null pointer");
    if ((Wr == nullptr) != (Wi == nullptr)) return tt::invalid("grf_fft: give both Wr and Wi or neither");
    const int M = 2 * N + 1;
    size_t w = 0;
    TT_TRY(z2d_work_bytes(M, &w, dim));
    const FftWs L = fft_ws(N, w, dim);
    if (!workspace || workspace_bytes < L.total) {
        tt::set_detail("grf_fft: workspace needs %zu bytes", L.total);
        return TT_ERR_WORKSPACE_TOO_SMALL;
    }
    cudaStream_t s = tt::as_stream(stream);
    char* ws = static_cast<char*>(workspace);
    cufftDoubleComplex* F = reinterpret_cast<cufftDoubleComplex*>(ws + L.spec_off);
    const long long lead = dim == 3 ? (long long)M * M : (dim == 2 ? M : 1);
    const long long nh = lead * (N + 1);
    shape_fft_kernel<<<grid_for(nh), 256, 0, s>>>(seed, dim, N, sqrt_p, Wr, Wi, F);
    TT_TRY(tt::launch_status("grf_fft shaping kernel"));
    TT_TRY(run_z2d(M, F, out, ws + L.work_off, s, dim));
    const long long nv = lead * M;
    scale_kernel<<<grid_for(nv), 256, 0, s>>>(out, nv, 1.0 / (double)nv);
    return tt::launch_status("grf_fft scale kernel");
}

extern "C" size_t tt_grf_fft_workspace_bytes(int N) { return tt_grf_fft_nd_workspace_bytes(3, N); }

extern "C" int tt_cos_field(int dim, int nx, int ny, int nz, double dx, double dy, double dz, int nmodes,
                            const double* k, const double* phase, const double* amp, double* out, void* stream)
{
    if (dim < 1 || dim > 3) return tt::invalid("cos_field: dim must be 1, 2 or 3");
    if (nx < 1 || (dim >= 2 && ny < 1) || (dim == 3 && nz < 1) || nmodes < 0) return tt::invalid("cos_field: sizes");
    if (!k || !phase || !amp || !out) return tt::invalid("cos_field: null pointer");
    const int Ny = dim >= 2 ? ny : 1, Nz = dim == 3 ? nz : 1;
    const long long total = (long long)nx * Ny * Nz;
    cos_field_kernel<<<grid_for(total), 256, 0, tt::as_stream(stream)>>>(dim, nx, Ny, Nz, dx, dy, dz, nmodes, k, phase,
                                                                         amp, out);
    return tt::launch_status("cos_field kernel");
}

extern "C" int tt_grf_fft(uint64_t seed, int N, const double* sqrt_p, const double* Wr, const double* Wi, double* out,
                          void* workspace, size_t workspace_bytes, void* stream)
{
    return tt_grf_fft_nd(seed, 3, N, sqrt_p, Wr, Wi, out, workspace, workspace_bytes, stream);
}

extern "C" size_t tt_grf_field_workspace_bytes(int n)
{
    if (n < 2) return 0;
    size_t w = 0;
    if (z2d_work_bytes(n, &w) != TT_OK) return 0;
    return field_ws(n, w).total;
}

extern "C" int tt_grf_field(uint64_t seed, int n, double L, double alpha, double kmin, double kmax, double ne0,
                            double delta, int out_dtype, void* out, void* workspace, size_t workspace_bytes,
                            void* stream)
{
    if (n < 2) return tt::invalid("grf_field: n must be >= 2");
    if (!(L > 0.0)) return tt::invalid("grf_field: L must be > 0");
    if (!out) return tt::invalid("grf_field: out is null");
    if (out_dtype != TT_F32 && out_dtype != TT_F64) return tt::invalid("grf_field: bad out_dtype");
    size_t w = 0;
    TT_TRY(z2d_work_bytes(n, &w));
    const FieldWs W = field_ws(n, w);
    if (!workspace || workspace_bytes < W.total) {
        tt::set_detail("grf_field: workspace needs %zu bytes", W.total);
        return TT_ERR_WORKSPACE_TOO_SMALL;
    }
    cudaStream_t s = tt::as_stream(stream);
    char* ws = static_cast<char*>(workspace);
    cufftDoubleComplex* F = reinterpret_cast<cufftDoubleComplex*>(ws + W.spec_off);
    double* part = reinterpret_cast<double*>(ws + W.part_off);
    const double mlo = kmin * L / (2.0 * M_PI), mhi = kmax * L / (2.0 * M_PI);
    const int h = n / 2 + 1;
    const long long nh = (long long)n * n * h;
    shape_field_kernel<<<grid_for(nh), 256, 0, s>>>(seed, n, mlo * mlo, mhi * mhi, alpha / 4.0, F);
    TT_TRY(tt::launch_status("grf_field shaping kernel"));
    double* f = reinterpret_cast<double*>(F);  // in-place C2R: rows padded to 2h doubles
    TT_TRY(run_z2d(n, F, f, ws + W.work_off, s));
    stats_partial_kernel<<<W.nparts, 256, 0, s>>>(f, n, 2 * h, part);
    stats_final_kernel<<<1, 32, 0, s>>>(part, W.nparts, (double)n * n * n);
    TT_TRY(tt::launch_status("grf_field statistics"));
    const long long nv = (long long)n * n * n;
    if (out_dtype == TT_F32)
        density_kernel<float><<<grid_for(nv), 256, 0, s>>>(f, n, 2 * h, part, ne0, delta, static_cast<float*>(out));
    else
        density_kernel<double><<<grid_for(nv), 256, 0, s>>>(f, n, 2 * h, part, ne0, delta, static_cast<double*>(out));
    return tt::launch_status("grf_field density kernel");
}

extern "C" int tt_philox(uint64_t seed, uint32_t tag, int64_t count, uint32_t* out, void* stream)
{
    if (count < 0) return tt::invalid("philox: count < 0");
    if (count == 0) return TT_OK;
    if (!out) return tt::invalid("philox: out is null");
    philox_kernel<<<grid_for(count), 256, 0, tt::as_stream(stream)>>>(seed, tag, count, out);
    return tt::launch_status("philox kernel");
}
