/*
 * turbotrace.h -- C ABI of libturbotrace.so, the GB300 (sm_103a) implementation
 * of the ray-integration path of jdhare/turbulence_tracing.
 *
 * Conventions
 *   - Every array pointer is DEVICE memory owned by the caller unless the
 *     comment says "host".  The library keeps no pointer after a call returns.
 *   - Volumes are C-ordered [ix][iy][iz] like the reference's numpy arrays.
 *     Ray arrays are structure-of-arrays rows like the reference's (6, Np) s0
 *     and (4, Np) rf: element (row, ray) lives at row * np + ray.
 *   - stream is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     All work is enqueued on it; no call synchronises the host unless noted.
 *   - Scratch memory is a caller-provided device workspace whose size comes
 *     from the matching *_workspace_bytes query.
 *   - Every entry point returns a tt_status (0 = TT_OK).  Per-ray outcomes
 *     are reported in int32 status arrays (tt_ray_status).
 */
#ifndef TURBOTRACE_H
#define TURBOTRACE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TT_ABI_VERSION 1

/* Per-ray cap on attempted integration steps when the caller passes 0. */
#define TT_DEFAULT_MAX_STEPS (1LL << 22)

typedef enum tt_status {
    TT_OK = 0,
    TT_ERR_INVALID_ARGUMENT = 1,
    TT_ERR_WORKSPACE_TOO_SMALL = 2,
    TT_ERR_CUDA = 3,
    TT_ERR_CUFFT = 4,
    TT_ERR_UNSUPPORTED = 5,
    TT_ERR_TOO_LARGE = 6
} tt_status;

typedef enum tt_ray_status {
    TT_RAY_OK = 0,              /* reached t_end */
    TT_RAY_STEP_TOO_SMALL = 1,  /* solve_ivp's TOO_SMALL_STEP */
    TT_RAY_MAX_STEPS = 2,       /* per-ray step cap hit (stiff); state left where it stopped */
    TT_RAY_NAN = 3              /* non-finite state */
} tt_ray_status;

typedef enum tt_dtype { TT_F32 = 0, TT_F64 = 1 } tt_dtype;

/* ABI version and error text.  tt_last_error_detail() is per host thread. */
int tt_abi_version(void);
const char* tt_strerror(int status);
const char* tt_last_error_detail(void);

/* ------------------------------------------------------------------------ */
/* K1  calc_dndr -- replaces ElectronCube.calc_dndr,
 *     particle_tracking/particle_tracker.py:220-237.
 * omega = 2 pi c / lwl, n_c = 3.14207787e-4 omega^2, ne_nc = min(ne / n_c, ne_max),
 * dndi = -0.5 c^2 numpy.gradient(ne_nc, coord_i, axis=i)  (edge_order 1,
 * non-uniform coordinates allowed).  FP64 results are bit-identical to numpy.
 * ne: (nx,ny,nz) of ne_dtype; x,y,z: device coordinate arrays (length nx,ny,nz). */
size_t tt_calc_dndr_workspace_bytes(int nx, int ny, int nz);
int tt_calc_dndr(const void* ne, int ne_dtype, int nx, int ny, int nz,
                 const double* x, const double* y, const double* z,
                 double lwl, double ne_max,
                 double* ne_nc, double* dndx, double* dndy, double* dndz,
                 double* omega_out /* host, may be NULL */,
                 void* workspace, size_t workspace_bytes, void* stream);

/* tt_calc_dndr_noalloc -- no counterpart in the reference.  The same results
 * as tt_calc_dndr for callers that cannot allocate device memory: a host
 * application whose memory manager owns every device buffer (a framework's
 * caching allocator, or a fixed device pool handed out up front) and does not
 * allow allocations behind its back.  It allocates nothing: its scratch is a
 * fixed 590 KB device array inside the library, present on every GPU that
 * loads it until the process exits, so every axis is limited to 8192 nodes
 * (TT_ERR_TOO_LARGE beyond).  The first call on a device looks up that
 * array's device address (no allocation) and keeps it for the device's
 * context: make that first call before any stream capture, and do not reset
 * the device after it.  All calls share the array: calls whose work overlaps
 * on the GPU (other streams, other threads) race and must be serialised by
 * the caller. */
int tt_calc_dndr_noalloc(const void* ne, int ne_dtype, int nx, int ny, int nz,
                         const double* x, const double* y, const double* z,
                         double lwl, double ne_max,
                         double* ne_nc, double* dndx, double* dndy, double* dndz,
                         double* omega_out /* host, may be NULL */, void* stream);

/* dndr -- replaces ElectronCube.dndr, particle_tracker.py:243-256 (the
 * RegularGridInterpolator lookups built at :239-241): trilinear, fill 0
 * outside the grid, NaN in -> NaN out.  pts: (3, npts) SoA; out: (nvol, npts)
 * for the nvol volumes in vols[] (host array of device pointers, nvol <= 4). */
int tt_dndr(const double* const* vols, int nvol, int nx, int ny, int nz,
            const double* x, const double* y, const double* z,
            const double* pts, int64_t npts, double* out, void* stream);

/* ------------------------------------------------------------------------ */
/* FP32 brick volume for the persistent tracer (K1, FP32 form).
 * Nodes are float4 {H_a, H_b, H_c, ne_nc} with H = -0.5 d(ne_nc)/dx * spacing_c,
 * i.e. the deflection per cell length of the probing axis.  Layout: the
 * probing axis c is fastest; the transverse axes a, b are cut into 4x4-cell
 * tiles stored with a one-node apron (5x5 node columns), each tile column cut
 * into bricks of brick_depth nodes along c; tiles are ordered by Morton code
 * inside 8x8 super-tiles, super-tiles row-major.  Requires uniformly spaced
 * coordinates. */
typedef struct tt_volume {
    int32_t n[3];          /* nodes along a, b, c */
    int32_t axis[3];       /* physical axis (0=x, 1=y, 2=z) of a, b, c */
    int32_t tiles[2];      /* 4-cell tiles along a, b */
    int32_t supertiles[2]; /* 8x8-tile super-tiles along a, b */
    int32_t bricks_c;      /* bricks along c */
    int32_t brick_depth;   /* nodes per brick along c (power of two, 4..32; tt_volume_plan sets 8) */
    double origin[3];      /* coordinate (m) of node 0 along a, b, c */
    double spacing[3];     /* node spacing (m) along a, b, c */
    double omega;          /* laser angular frequency (rad/s) */
    double ne_max;         /* clip applied to n_e/n_c */
    int64_t n_float4;      /* float4 elements in the node buffer */
    void* nodes;           /* device node buffer, 16-byte aligned, set by the caller */
} tt_volume;

/* Fill *vol (all fields but nodes) for a grid with host coordinate arrays and
 * a probing axis (0=x, 1=y, 2=z); returns TT_ERR_UNSUPPORTED for non-uniform
 * coordinates.  The node buffer needs vol->n_float4 * 16 bytes. */
int tt_volume_plan(int nx, int ny, int nz, const double* x_host, const double* y_host,
                   const double* z_host, int probing_axis, double lwl, double ne_max,
                   tt_volume* vol);
/* Change the brick depth (power of two, 4..32) of a planned volume; updates
 * bricks_c and n_float4.  Call before sizing and building the node buffer. */
int tt_volume_set_brick_depth(tt_volume* vol, int brick_depth);
/* Write the node buffer from a density (nx,ny,nz) of ne_dtype. */
int tt_volume_build(const tt_volume* vol, const void* ne, int ne_dtype, void* stream);

/* ------------------------------------------------------------------------ */
/* K2  trace -- replaces ElectronCube.solve + dsdt + dndr + ray_at_exit,
 *     particle_tracker.py:312-380, 398-419.  Each ray integrates
 *     x' = v, v' = grad from t = 0 to t_end with its own Dormand-Prince 5(4)
 *     step control.  Outputs (any may be NULL): sf (6,np) state at t_end;
 *     rf (4,np) [pos, angle, pos, angle] back-projected to the exit plane at
 *     +extent along the probing axis (ray_at_exit); phase (np) = k0 int (n-1) ds
 *     with n = sqrt(1 - ne_nc) (needs with_phase); status (np) tt_ray_status;
 *     nsteps (np) accepted steps. */
typedef struct tt_trace_opts {
    double rtol;        /* FP64: as solve_ivp.  FP32: relative tolerance on velocity/phase */
    double atol;        /* FP64: as solve_ivp (SI units).  FP32: absolute position tolerance in cells */
    double atol_phase;  /* FP32 only: absolute phase tolerance (rad) */
    int64_t max_steps;  /* per-ray cap on attempted steps; 0 = TT_DEFAULT_MAX_STEPS */
    int32_t with_phase; /* integrate the phase as an extra state */
    int32_t block_size; /* FP32 tracer: threads per block, 64, 128 or 256 (0 = 256) */
    int32_t ray_chunk;  /* FP32 tracer: consecutive (bucketed) rays a warp takes from the work
                           counter at a time, a multiple of 32 up to 1024; 0 = 32 */
    int32_t phase_f64;  /* FP32 tracer with phase: accumulate the phase sum in FP64 (one double add
                           per accepted step) instead of a Neumaier-compensated FP32 pair */
    int32_t refill_lanes; /* FP32 tracer: a warp takes new rays only once at least this many of its
                           32 lanes are idle, 1..32 (0 = 2).  1 refills every idle lane at once;
                           32 traces each warp's 32 neighbouring rays to the end together, which
                           keeps the lanes' node reads coherent.  Results do not depend on it. */
} tt_trace_opts;

/* Plain FP64 drop-in: scipy RK45 controller per ray (safety 0.9, factors
 * [0.2, 10], exponent -1/5, RMS norm over the ray's components, scipy's
 * initial-step rule), lookups as tt_dndr.  probing_axis selects ray_at_exit's
 * branch; extent is the exit-plane coordinate (cube.extent). */
int tt_trace_f64(const double* dndx, const double* dndy, const double* dndz, const double* ne_nc,
                 int nx, int ny, int nz, const double* x, const double* y, const double* z,
                 double omega, const double* s0, int64_t np, double t_end,
                 int probing_axis, double extent, const tt_trace_opts* opts,
                 double* sf, double* rf, double* phase, int32_t* status, int32_t* nsteps,
                 void* stream);

/* An explicit Runge-Kutta pair in the form scipy.integrate's RungeKutta
 * classes hold it (RK23, RK45, DOP853: class attributes A, B, C, E / E3, E5,
 * error_estimator_order), for tt_trace_f64_rk -- the `method` argument of
 * ElectronCube.solve, particle_tracker.py:312, 323.  n_stages s is 3, 6 or
 * 12; A is strictly lower triangular with row sums C; B (s) sums to 1; E
 * (s + 1 weights, the last on the FSAL evaluation at the new point) sums to 0.
 * error_kind 0: err = h K^T E, RMS norm (RK23, RK45); error_kind 1 (12 stages
 * only): DOP853's norm |h| |K^T E5|^2 / sqrt((|K^T E5|^2 + 0.01 |K^T E3|^2) n)
 * with E5 in E and E3 in E3.  The step factor exponent is -1/(error_order+1),
 * the initial-step exponent 1/(error_order+1). */
#define TT_RK_MAX_STAGES 16
typedef struct tt_rk_tableau {
    int32_t n_stages;
    int32_t error_order;
    int32_t error_kind;
    int32_t reserved;
    double A[TT_RK_MAX_STAGES][TT_RK_MAX_STAGES];
    double B[TT_RK_MAX_STAGES];
    double C[TT_RK_MAX_STAGES];
    double E[TT_RK_MAX_STAGES + 1];
    double E3[TT_RK_MAX_STAGES + 1];
} tt_rk_tableau;

/* tt_trace_f64 with the caller's method: solve(method='RK23' | 'DOP853')
 * (particle_tracker.py:312, 323 hands `method` to solve_ivp).  Same arguments
 * and outputs as tt_trace_f64; tableau is a host struct. */
int tt_trace_f64_rk(const double* dndx, const double* dndy, const double* dndz, const double* ne_nc,
                    int nx, int ny, int nz, const double* x, const double* y, const double* z,
                    double omega, const double* s0, int64_t np, double t_end,
                    int probing_axis, double extent, const tt_trace_opts* opts,
                    const tt_rk_tableau* tableau,
                    double* sf, double* rf, double* phase, int32_t* status, int32_t* nsteps,
                    void* stream);

/* Persistent FP32 tracer over a tt_volume: rays binned by entry tile in the
 * volume's Morton order, one ray per thread pulled from a work queue, steps
 * ended on cell faces so each step integrates one cell's trilinear
 * polynomial, compensated (Neumaier) position/phase sums. */
size_t tt_trace_f32_workspace_bytes(const tt_volume* vol, int64_t np);
int tt_trace_f32(const tt_volume* vol, const double* s0, int64_t np, double t_end, double extent,
                 const tt_trace_opts* opts, double* sf, double* rf, double* phase,
                 int32_t* status, int32_t* nsteps, void* workspace, size_t workspace_bytes,
                 void* stream);

/* Batched form: ninst field realisations (each its own tt_volume, grid size,
 * t_end and exit plane) traced in ONE persistent launch.  Arrays are
 * instance-blocked: instance i owns rays [ray_offsets[i], ray_offsets[i+1]),
 * n_i of them, and its s0 is a (6, n_i) block starting at element
 * 6 * ray_offsets[i] of s0 (sf likewise, rf a (4, n_i) block at
 * 4 * ray_offsets[i], phase/status/nsteps at ray_offsets[i]), so each
 * instance's results are ordinary arrays for tt_detect.  Rays are bucketed by
 * (instance, entry tile) and pulled from one work queue, each lane carrying
 * its ray's instance.  vols, ray_offsets, t_end and extent are host arrays; at
 * most TT_MAX_INSTANCES instances. */
#define TT_MAX_INSTANCES 128
size_t tt_trace_f32_batched_workspace_bytes(const tt_volume* vols, int ninst, int64_t ntot);
int tt_trace_f32_batched(const tt_volume* vols, int ninst, const int64_t* ray_offsets, const double* t_end,
                         const double* extent, const double* s0, const tt_trace_opts* opts,
                         double* sf, double* rf, double* phase, int32_t* status, int32_t* nsteps,
                         void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* K3  detectors -- replaces Rays.__init__/solve/histogram and the filters of
 *     particle_tracking/ray_transfer_matrix.py:37-195 (diagnostic chains at
 *     :214-299).  Each ray of rf (4,n) is pushed through the optic chain
 *     (host array; a diagnostic starts with TT_OPTIC_M_TO_MM as Rays.__init__
 *     does), rejected rays become NaN, and the survivors are binned like
 *     numpy.histogram2d over [x0,x1]x[y0,y1] (nbx x nby bins, last bin
 *     closed) into H (nby, nbx) -- the transposed layout Rays.histogram leaves
 *     in self.H.  Hw gets the same histogram weighted by weights (e.g. phase).
 *     H/Hw are added to when accumulate != 0, else overwritten.  r_out (4,n),
 *     if given, receives the rays after the chain (Rays.rf).  With H == NULL
 *     only the chain runs (the module-level matrix and filter functions). */
typedef enum tt_optic_kind {
    TT_OPTIC_DISTANCE = 0,       /* p0 = d               distance(), :62-71 */
    TT_OPTIC_LENS = 1,           /* p0 = f1, p1 = f2     lens(), :42-54 */
    TT_OPTIC_CIRC_APERTURE = 2,  /* p0 = R   reject r^2 > R^2, :73-79 */
    TT_OPTIC_CIRC_STOP = 3,      /* p0 = R   reject r^2 < R^2, :81-87 */
    TT_OPTIC_ANNULUS_STOP = 4,   /* p0 = R1, p1 = R2  reject R1^2 < r^2 < R2^2 (one annulus of angular_filter, :89-111) */
    TT_OPTIC_RECT_APERTURE = 5,  /* p0 = Lx, p1 = Ly  reject x^2 > Lx^2 AND y^2 > Ly^2, :128-136 */
    TT_OPTIC_KNIFE_EDGE = 6,     /* p0 = offset, p1 = axis (0 = x, 2 = y), p2 = direction sign, :138-154 */
    TT_OPTIC_M_TO_MM = 7         /* rows 0 and 2 times 1e3, m_to_mm() :37-40 */
} tt_optic_kind;

typedef struct tt_optic {
    int32_t kind;
    int32_t reserved;
    double p[3];
} tt_optic;

#define TT_MAX_OPTICS 64

int tt_detect(const double* rf, int64_t n, const tt_optic* chain_host, int n_optics,
              int nbx, int nby, double x0, double x1, double y0, double y1,
              const double* weights, double* H, double* Hw, double* r_out,
              int accumulate, void* stream);

/* ------------------------------------------------------------------------ */
/* K4  Gaussian random fields -- replaces turboGen.gaussian3D_FFT,
 *     gaussian_fields/turboGen.py:488-537.
 * tt_grf_fft: M = 2N+1 points per axis; complex Gaussian noise Hermitian
 * symmetrised (W(-k) = conj W(k), Re/Im variance 2 each as the reference's
 * Wr + flip(Wr), Wi - flip(Wi)), times sqrt_p (the caller's k_func(|k|)
 * square-rooted, on the half spectrum M x M x (N+1), |k| in cycles/sample),
 * zero mean, inverse FFT / M^3, real part -> out (M,M,M) float64.
 * Noise comes from Philox4x32-10 keyed by seed, or, when Wr and Wi (M^3,
 * the reference's centred layout) are given, from those arrays. */
size_t tt_grf_fft_workspace_bytes(int N);
int tt_grf_fft(uint64_t seed, int N, const double* sqrt_p, const double* Wr, const double* Wi,
               double* out, void* workspace, size_t workspace_bytes, void* stream);

/* The same construction in dim = 1, 2 or 3 dimensions: gaussian1D_FFT,
 * gaussian2D_FFT, gaussian3D_FFT (turboGen.py:388-537).  sqrt_p on the half
 * spectrum M^(dim-1) x (N+1); Wr, Wi (M^dim, centred) or NULL for Philox noise;
 * out M^dim float64.  tt_grf_fft is dim = 3. */
size_t tt_grf_fft_nd_workspace_bytes(int dim, int N);
int tt_grf_fft_nd(uint64_t seed, int dim, int N, const double* sqrt_p, const double* Wr, const double* Wi,
                  double* out, void* workspace, size_t workspace_bytes, void* stream);

/* tt_cos_field -- replaces the mode sums of gaussian1Dcos, gaussian2Dcos and
 * gaussian3Dcos (turboGen.py:40-385): at cell centres x_i = dx/2 + i dx,
 *   out = sum_m amp_m sqrt(2) (sum over the 1, 2 or 4 sign patterns s of
 *         cos(kx x + s_y ky y + s_z kz z + phase_s,m)),
 * sign patterns (+), (+,+ / +,-) and (++,+-,-+,--) in the reference's order.
 * k: (3, nmodes) device array (rows kx, ky, kz), phase: (4, nmodes), amp:
 * (nmodes); out: (nx[, ny[, nz]]) float64, C-ordered. */
int tt_cos_field(int dim, int nx, int ny, int nz, double dx, double dy, double dz, int nmodes, const double* k,
                 const double* phase, const double* amp, double* out, void* stream);

/* tt_grf_field: the band-limited field of the benchmark workloads on an n^3
 * grid of side L: complex Gaussian noise (Philox4x32-10, counter = mode index)
 * times |k|^(alpha/2) for kmin <= |k| <= kmax (rad/m), inverse real FFT,
 * normalised to zero mean and unit variance g, then
 * ne = ne0 (1 + delta g) clipped at >= 0, written as out_dtype. */
size_t tt_grf_field_workspace_bytes(int n);
int tt_grf_field(uint64_t seed, int n, double L, double alpha, double kmin, double kmax,
                 double ne0, double delta, int out_dtype, void* out,
                 void* workspace, size_t workspace_bytes, void* stream);

/* Raw Philox4x32-10 blocks for counters (i, 0, 0, tag), i in [0, count), key = seed:
 * out (4, count) uint32.  Exposed for known-answer tests of the generator. */
int tt_philox(uint64_t seed, uint32_t tag, int64_t count, uint32_t* out, void* stream);

/* Straight-line path integrals through an n_e grid along z, at the centres of
 * a P x P pixel grid over the box face (pixel (i, j) at x0 + (i + 0.5)(xN - x0)/P,
 * y0 + (j + 0.5)(yN - y0)/P): out FP32 [3 + 2 nslab][P][P] =
 *   -1/2 integral dq/dx dz, -1/2 integral dq/dy dz (straight-line deflection, rad),
 *   k0 integral (sqrt(1 - q) - 1) dz (straight-line phase, rad),
 *   then for each of nslab (0..8) equal slabs of cells along z the two
 *   deflection integrals over that slab,
 * q = min(ne / n_c, ne_max) with n_c and k0 = omega / c as calc_dndr forms them
 * (particle_tracker.py:227-232), gradients by numpy.gradient's rule, all fields
 * trilinear (the phase by 2-point Gauss per cell).  x, y, z: host arrays of
 * uniform node coordinates. */
int tt_straight_line_maps(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x, const double* y,
                          const double* z, double lwl, double ne_max, int P, int nslab, float* out, void* stream);

/* Marched pixel-centre rays, the surrogate's coarse solution: the same P x P
 * pixel-centre rays as tt_straight_line_maps, entering along +z at z0 and
 * stepped from node plane to node plane (one step per cell along z, second
 * order) through the ray equation with z as the parameter,
 *   dt/dz = -1/2 (1 + |t|^2) / (1 + q0 - q) (grad_perp q - t dq/dz),
 * t the slopes (dx/dz, dy/dz), q0 = q at the entry point, fields as the tracer
 * interpolates them (numpy.gradient derivatives, bilinear on the node planes,
 * zero outside).  out FP32 [5][P][P]: the marched exit angles arctan(t_x),
 * arctan(t_y) (rad, as ray_at_exit, particle_tracker.py:333-380) and phase
 * k0 integral (sqrt(1 - q) - 1) ds (rad), then the straight-line deflection of
 * the same rays (tt_straight_line_maps' first two outputs), all from one pass
 * over the density.  workspace: device scratch of
 * tt_march_maps_workspace_bytes(nx, ny, nz) bytes, 16-byte aligned (q stored
 * plane by plane with a ghost border, and its column sums); nx <= 65535. */
size_t tt_march_maps_workspace_bytes(int nx, int ny, int nz);
int tt_march_maps(const void* ne, int ne_dtype, int nx, int ny, int nz, const double* x, const double* y,
                  const double* z, double lwl, double ne_max, int P, float* out, void* workspace,
                  size_t workspace_bytes, void* stream);

/* tt_march_maps over nfields (1..TT_MAX_MARCH_FIELDS) fields of one shape in
 * one pass: ne is a host array of nfields device pointers, out FP32
 * [nfields][5][P][P], workspace of tt_march_maps_batched_workspace_bytes
 * bytes.  Fields march side by side, which fills the GPU where one field's
 * P x P rays do not. */
#define TT_MAX_MARCH_FIELDS 32
size_t tt_march_maps_batched_workspace_bytes(int nfields, int nx, int ny, int nz);
int tt_march_maps_batched(const void* const* ne, int nfields, int ne_dtype, int nx, int ny, int nz, const double* x,
                          const double* y, const double* z, double lwl, double ne_max, int P, float* out,
                          void* workspace, size_t workspace_bytes, void* stream);

/* tt_march_maps_batched stepping plane_stride (1 or 2) node planes per step:
 * with 2, the marched rays take one kick-drift-kick step of 2 h_z per two
 * planes (the fields sampled on the even planes, d/dz still from the
 * neighbouring planes) and a last single step to an odd last plane -- half
 * the march's work, and an answer that aliases the grid-scale gradient (the
 * surrogate's network learns the correction).  The straight-line maps are
 * unchanged (every plane). */
int tt_march_maps_batched_stride(const void* const* ne, int nfields, int ne_dtype, int nx, int ny, int nz,
                                 const double* x, const double* y, const double* z, double lwl, double ne_max,
                                 int P, int plane_stride, float* out, void* workspace, size_t workspace_bytes,
                                 void* stream);

/* Geometric-optics shadowgram of a deflection map theta FP32 [2][P][P] (angles
 * of rays leaving the centres of a P x P pixel grid of pitch `pitch` m):
 * intensity [P][P] = 1 / max(|det(I + D grad theta)|, 1e-3) after a free drift
 * of D m, and div [P][P] = d theta_x/dx + d theta_y/dy (either output may be
 * NULL); differences central inside, one-sided at the edges. */
int tt_shadowgram(const float* theta, int P, double pitch, double D, float* intensity, float* div, void* stream);
/* tt_shadowgram's intensity for nmaps maps at once: theta FP32 [nmaps][2][P][P],
 * D a device array of nmaps drifts (m), intensity FP32 [nmaps][P][P]. */
int tt_shadowgram_batched(const float* theta, int nmaps, int P, double pitch, const double* D, float* intensity,
                          void* stream);

/* The surrogate's network input from n march outputs maps FP32 [n][5][P][P]
 * (tt_march_maps layout).  stats FP32 [n][4] (16-byte aligned) = (s, mean and
 * unbiased standard deviation of the marched phase, log10(s (P - 1))), s the
 * rms of the straight-line deflection; FP32 sums per thread, FP64 across
 * them.  X FP32 [n][6][P][P] = (straight x, y, marched x, y) / s,
 * (phase - mean) / sd, log10(s (P - 1)).  The learned surrogate has no
 * counterpart in the reference. */
int tt_surrogate_encode(const float* maps, int n, int P, float* X, float* stats, void* stream);
/* theta FP32 [n][2][P][P] = maps[:, 0:2] + s / gain[0:2] * net[:, 0:2] (net
 * FP32 [n][3][P][P] the network output, stats from tt_surrogate_encode, gain
 * FP32 [3] the per-channel target gain), and theta_march FP32 [n][2][P][P] =
 * maps[:, 0:2] when not NULL. */
int tt_surrogate_decode(const float* maps, const float* net, const float* stats, const float* gain, int n, int P,
                        float* theta, float* theta_march, void* stream);
/* The fallback's error estimate: est FP32 [n] = kappa ||I_net - I_march|| /
 * ||I_net|| over each P x P intensity map (FP32 sums per thread, FP64 across
 * them; infinite when I_net is zero, so such a map falls back). */
int tt_surrogate_estimate(const float* I_net, const float* I_march, int n, int P, double kappa, float* est,
                          void* stream);

/* ---- Learned surrogate: 2D Fourier neural operator ----------------------------
 * No reference interface: the reference has no surrogate.  The network maps
 * straight-line path-integrated gradient maps to the full-trace deflection and
 * phase correction on the same S x S grid (S in {128, 256}): a pointwise lift
 * of the in_ch data channels plus two coordinate channels (row, column, each
 * (i + 0.5) 2/S - 1) to width 32, `layers` Fourier layers (truncated DFT
 * keeping 16 x 32 modes, per-mode complex 32 x 32 mixing, inverse DFT, plus a
 * 1x1 convolution and bias, then GELU in its tanh form), and a pointwise projection to out_ch.
 * Activations are bfloat16 with FP32 accumulation; every contraction over
 * pixels runs on the tcgen05 tensor cores.
 *
 * Parameters are one FP32 array, in this order (C = 32, M = 512 modes, cin = in_ch + 2):
 *   P [C][cin], pb [C], then per layer: W [C][C], b [C], R [M][C][C][2] (complex
 *   R[mode][out][in], mode = kyi * 16 + kx, kyi < 16: ky = kyi, else ky = S - 32 + kyi),
 *   then Q [out_ch][C], qb [out_ch].
 * Inputs a: FP32 [batch][in_ch][S][S]; targets and outputs: FP32 [batch][out_ch][S][S]. */
#define TT_FNO_WIDTH 32
#define TT_FNO_MODES 16
#define TT_FNO_MAX_LAYERS 8
#define TT_FNO_MAX_IN 16
#define TT_FNO_MAX_OUT 4

typedef struct tt_fno_dims {
    int32_t batch;
    int32_t size;   /* S */
    int32_t in_ch;  /* data channels, 1..TT_FNO_MAX_IN */
    int32_t out_ch; /* 1..TT_FNO_MAX_OUT */
    int32_t layers; /* 1..TT_FNO_MAX_LAYERS */
} tt_fno_dims;

size_t tt_fno_param_count(const tt_fno_dims* d);
/* training != 0: room for the activations the backward pass needs. */
size_t tt_fno_workspace_bytes(const tt_fno_dims* d, int training);

/* Inference: out = network(a). */
int tt_fno_forward(const tt_fno_dims* d, const float* params, const float* a, float* out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* One forward + backward pass: *loss (device) += sum_k w_k sum (out - target)^2 / (batch S^2)
 * and grads (same layout as params) += its gradient.  channel_weights: host array of
 * out_ch weights (NULL = all 1); out (optional) receives the prediction. */
int tt_fno_train_step(const tt_fno_dims* d, const float* params, float* grads, const float* a, const float* target,
                      const float* channel_weights, float* loss, float* out, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Adam update of n parameters (bias-corrected, step counts from 1); zeroes grads. */
int tt_fno_adam(int64_t n, float* params, float* grads, float* m, float* v, float lr, float beta1, float beta2,
                float eps, int64_t step, void* stream);

/* The same with the learning rate (*lr) and step counter (*step, incremented
 * first) in device memory, for training steps captured in a CUDA graph. */
int tt_fno_adam_device(int64_t n, float* params, float* grads, float* m, float* v, const float* lr, float beta1,
                       float beta2, float eps, int64_t* step, void* stream);

/* Device error flag in a workspace (1 after a bounded tensor-core wait ran out). Synchronous. */
int tt_fno_error_flag(const void* workspace, int* host_flag);

/* The tensor-core building blocks, for tests.  Operands "packed" are bf16
 * matrices in the canonical K-major tcgen05 layout written by tt_fno_pack
 * (rows % 8 == 0, k % 8 == 0).  workspace: >= 256 bytes, zeroed (error flag).
 *   rowdft: out[r][j] = sum_x in[r][x] mat[j][x]; in bf16 [rows][S], rows % 128 == 0,
 *           mat packed [32][S], out FP32 [rows][32].
 *   mix:    acc[x][o] = sum_c in[b][c][y][x] w[o][c] + sum_j a[x][j] sp[b][o][y][j] over every
 *           (b, y, x); w packed [32][32], a packed [S][32], sp FP32 [B][32][S][32].
 *           mode 0: out0 = bf16(acc + bias) (if out0), out1 = bf16(GELU(out0));
 *           mode 1: out0 = bf16(acc * GELU'(zprev)) (zprev NULL: acc).  Outputs bf16 [B][32][S][S].
 *   wgrad:  dW[o][c] += sum_{b,p} dz[b][o][p] v[b][c][p], db[o] += sum dz[b][o][p]; dz, v bf16 [B][32][S*S]. */
int tt_fno_pack(int64_t rows, int k, const float* src, void* dst, void* stream);
int tt_fno_rowdft(int S, int64_t rows, const void* in, const void* mat_packed, float* out, void* workspace,
                  void* stream);
int tt_fno_mix(int S, int B, int mode, const void* in, const void* w_packed, const void* a_packed, const float* sp,
               const float* bias, const void* zprev, void* out0, void* out1, void* workspace, void* stream);
int tt_fno_wgrad(int S, int B, const void* dz, const void* v, float* dW, float* db, void* workspace, void* stream);

/* Test of the bounded-wait error path (no reference counterpart): tt_fno_rowdft
 * with every mbarrier wait limited to wait_cycles SM clocks (1000..2e9) and
 * the copies of each CTA's first tile left out, so that tile's barrier never
 * completes.  Each CTA's wait runs out, it sets the error flag (workspace word
 * 0, read with tt_fno_error_flag), frees its TMEM and returns; no copy is in
 * flight when it does.  out is left unwritten. */
int tt_fno_rowdft_timeout_test(int S, int64_t rows, const void* in, const void* mat_packed, float* out,
                               void* workspace, int64_t wait_cycles, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TURBOTRACE_H */
