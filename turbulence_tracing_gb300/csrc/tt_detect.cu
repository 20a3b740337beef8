// K3: detector chain and histogram.
//
// Replaces Rays.__init__ (m_to_mm), the diagnostics' solve() chains and
// Rays.histogram of particle_tracking/ray_transfer_matrix.py:37-195, 214-299.
// One thread carries one ray through the optic chain (4x4 transfer matrices
// applied as numpy.matmul does: the block-diagonal terms alone while the ray
// is finite, which round identically, the full product with its zero terms
// otherwise so inf/NaN propagate the same way; filters set every component
// of a rejected ray to NaN), then bins
// the survivors with numpy.histogram2d's rule: edges = linspace(lo, hi, n+1)
// computed as numpy computes them, bin = searchsorted(edges, v, 'right') - 1,
// the right edge belongs to the last bin, out-of-range and NaN dropped.
// Compiled with -fmad=false so each product/sum rounds like numpy's.
//
// Counting: when the detector fits in shared memory (<= kSmemBins bins) every
// block keeps a private uint32 histogram and merges it once; otherwise lanes
// that hit the same bin are merged with __match_any_sync and one lane per bin
// does a global atomic (the histogram then lives in L2).
#include <math.h>

#include "tt_common.cuh"

namespace {

struct Chain {
    int n;
    tt_optic op[TT_MAX_OPTICS];
};

struct Axis {
    double lo, hi, step;
    int nb;
};

constexpr int kSmemBins = 12288;  // 48 KB of uint32 counters per block

__device__ inline double edge(const Axis& A, int i)
{
    if (i >= A.nb) return A.hi;
    return __dadd_rn(__dmul_rn((double)i, A.step), A.lo);
}

// bin index or -1 when dropped
__device__ inline int bin_of(const Axis& A, double v)
{
    if (!(v >= A.lo && v <= A.hi)) return -1;  // also NaN
    int g = (int)floor((v - A.lo) / A.step);
    if (g < 0) g = 0;
    if (g > A.nb - 1) g = A.nb - 1;
    for (int it = 0; it < 4 && g + 1 <= A.nb && edge(A, g + 1) <= v; ++it) ++g;
    for (int it = 0; it < 4 && g >= 0 && edge(A, g) > v; ++it) --g;
    if (g >= A.nb) g = A.nb - 1;  // v == hi
    if (g < 0) return -1;
    return g;
}

__device__ inline void set_nan(double r[4])
{
    r[0] = r[1] = r[2] = r[3] = CUDART_NAN;
}

// Every component finite (exponent field not all ones): then the zero terms
// of a transfer matrix add exact zeros and its unit terms are exact, so the
// block-diagonal products below round exactly as the full 4x4 product does
// (up to the sign of a zero result); otherwise the full product runs so that
// inf and NaN spread across components as numpy's matmul spreads them.
__device__ inline bool all_finite(const double r[4])
{
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) ok = ok && (((unsigned)__double2hiint(r[k]) & 0x7ff00000u) != 0x7ff00000u);
    return ok;
}

__device__ inline void apply_chain(const Chain& C, double r[4])
{
    for (int k = 0; k < C.n; ++k) {
        const tt_optic& o = C.op[k];
        switch (o.kind) {
            case TT_OPTIC_DISTANCE: {
                // [[1,d],[0,1]] blocks: out0 = 1 r0 + d r1 + 0 r2 + 0 r3, ...
                const double d = o.p[0];
                if (all_finite(r)) {
                    r[0] = r[0] + d * r[1];
                    r[2] = r[2] + d * r[3];
                    break;
                }
                const double a0 = 1.0 * r[0] + d * r[1] + 0.0 * r[2] + 0.0 * r[3];
                const double a1 = 0.0 * r[0] + 1.0 * r[1] + 0.0 * r[2] + 0.0 * r[3];
                const double a2 = 0.0 * r[0] + 0.0 * r[1] + 1.0 * r[2] + d * r[3];
                const double a3 = 0.0 * r[0] + 0.0 * r[1] + 0.0 * r[2] + 1.0 * r[3];
                r[0] = a0; r[1] = a1; r[2] = a2; r[3] = a3;
                break;
            }
            case TT_OPTIC_LENS: {
                const double m1 = o.p[0], m2 = o.p[1];  // -1/f1, -1/f2, formed on the host
                if (all_finite(r)) {
                    r[1] = m1 * r[0] + r[1];
                    r[3] = m2 * r[2] + r[3];
                    break;
                }
                const double a0 = 1.0 * r[0] + 0.0 * r[1] + 0.0 * r[2] + 0.0 * r[3];
                const double a1 = m1 * r[0] + 1.0 * r[1] + 0.0 * r[2] + 0.0 * r[3];
                const double a2 = 0.0 * r[0] + 0.0 * r[1] + 1.0 * r[2] + 0.0 * r[3];
                const double a3 = 0.0 * r[0] + 0.0 * r[1] + m2 * r[2] + 1.0 * r[3];
                r[0] = a0; r[1] = a1; r[2] = a2; r[3] = a3;
                break;
            }
            case TT_OPTIC_CIRC_APERTURE: {
                const double R = o.p[0];
                if (r[0] * r[0] + r[2] * r[2] > R * R) set_nan(r);
                break;
            }
            case TT_OPTIC_CIRC_STOP: {
                const double R = o.p[0];
                if (r[0] * r[0] + r[2] * r[2] < R * R) set_nan(r);
                break;
            }
            case TT_OPTIC_ANNULUS_STOP: {
                const double q = r[0] * r[0] + r[2] * r[2];
                if (q > o.p[0] * o.p[0] && q < o.p[1] * o.p[1]) set_nan(r);
                break;
            }
            case TT_OPTIC_RECT_APERTURE: {
                if (r[0] * r[0] > o.p[0] * o.p[0] && r[2] * r[2] > o.p[1] * o.p[1]) set_nan(r);
                break;
            }
            case TT_OPTIC_KNIFE_EDGE: {
                const double v = o.p[1] > 1.0 ? r[2] : r[0];
                const bool rej = o.p[2] > 0 ? (v > o.p[0]) : (v < o.p[0]);
                if (rej) set_nan(r);
                break;
            }
            case TT_OPTIC_M_TO_MM: {
                r[0] *= 1e3;
                r[2] *= 1e3;
                break;
            }
            default: break;
        }
    }
}

template <bool SMEM>
__global__ void __launch_bounds__(256) detect_kernel(Chain C, Axis AX, Axis AY, const double* __restrict__ rf,
                                                     long long n, const double* __restrict__ w,
                                                     double* __restrict__ H, double* __restrict__ Hw,
                                                     double* __restrict__ rout)
{
    extern __shared__ unsigned sh[];
    const int nbins = AX.nb * AY.nb;
    if (SMEM) {
        for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0u;
        __syncthreads();
    }
    for (long long base = blockIdx.x * (long long)blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
        const long long i = base + threadIdx.x;
        int bin = -1;
        double wt = 0.0;
        if (i < n) {
            double r[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) r[k] = rf[(size_t)k * n + i];
            apply_chain(C, r);
            if (rout) {
#pragma unroll
                for (int k = 0; k < 4; ++k) rout[(size_t)k * n + i] = r[k];
            }
            const int bx = H ? bin_of(AX, r[0]) : -1;
            const int by = H ? bin_of(AY, r[2]) : -1;
            if (bx >= 0 && by >= 0) {
                bin = by * AX.nb + bx;  // transposed layout (H.T), row = y bin
                if (w) wt = w[i];
            }
        }
        // warp-aggregate equal bins
        const unsigned act = __ballot_sync(0xffffffffu, bin >= 0);
        if (bin >= 0) {
            const unsigned peers = __match_any_sync(act, bin);
            const int leader = __ffs(peers) - 1;
            const unsigned lane = threadIdx.x & 31u;
            double wsum = wt;
            if (Hw) {
                // sum weights over peers (small groups; serial over the mask keeps it exact-ordered)
                unsigned m = peers;
                wsum = 0.0;
                while (m) {
                    const int src = __ffs(m) - 1;
                    m &= m - 1;
                    wsum += __shfl_sync(peers, wt, src);
                }
            }
            if ((int)lane == leader) {
                const unsigned cnt = (unsigned)__popc(peers);
                if (SMEM) atomicAdd(sh + bin, cnt);
                else atomicAdd(H + bin, (double)cnt);
                if (Hw) atomicAdd(Hw + bin, wsum);
            }
        }
    }
    if (SMEM) {
        __syncthreads();
        for (int i = threadIdx.x; i < nbins; i += blockDim.x)
            if (sh[i]) atomicAdd(H + i, (double)sh[i]);
    }
}

}  // namespace

extern "C" int tt_detect(const double* rf, int64_t n, const tt_optic* chain_host, int n_optics, int nbx, int nby,
                         double x0, double x1, double y0, double y1, const double* weights, double* H, double* Hw,
                         double* r_out, int accumulate, void* stream)
{
    if (n < 0) return tt::invalid("detect: n < 0");
    if (nbx < 1 || nby < 1) return tt::invalid("detect: need at least one bin per axis");
    if ((long long)nbx * nby > (1LL << 31)) return tt::invalid("detect: too many bins");
    if (n_optics < 0 || n_optics > TT_MAX_OPTICS) return tt::invalid("detect: 0..TT_MAX_OPTICS optics");
    if (n_optics > 0 && !chain_host) return tt::invalid("detect: null chain");
    if (!H && !r_out) return tt::invalid("detect: need H or r_out");
    if (!H && Hw) return tt::invalid("detect: Hw needs H");
    if (Hw && !weights) return tt::invalid("detect: Hw needs weights");
    if (H && (!(x1 > x0) || !(y1 > y0))) return tt::invalid("detect: need x0 < x1 and y0 < y1");
    if (n > 0 && !rf) return tt::invalid("detect: rf is null");
    Chain C;
    C.n = n_optics;
    for (int k = 0; k < n_optics; ++k) {
        C.op[k] = chain_host[k];
        const int kind = C.op[k].kind;
        if (kind < TT_OPTIC_DISTANCE || kind > TT_OPTIC_M_TO_MM) return tt::invalid("detect: unknown optic kind");
        if (kind == TT_OPTIC_KNIFE_EDGE && C.op[k].p[2] == 0.0)
            return tt::invalid("detect: knife edge direction must be < 0 or > 0");
        if (kind == TT_OPTIC_LENS) {  // the matrix entries -1/f, rounded once as numpy rounds them
            C.op[k].p[0] = -1.0 / C.op[k].p[0];
            C.op[k].p[1] = -1.0 / C.op[k].p[1];
        }
    }
    Axis AX{x0, x1, (x1 - x0) / (double)nbx, nbx};
    Axis AY{y0, y1, (y1 - y0) / (double)nby, nby};
    cudaStream_t s = tt::as_stream(stream);
    const size_t hb = sizeof(double) * (size_t)nbx * nby;
    if (!accumulate && H) {
        TT_TRY(tt::cuda_status(cudaMemsetAsync(H, 0, hb, s), "detect clear H"));
        if (Hw) TT_TRY(tt::cuda_status(cudaMemsetAsync(Hw, 0, hb, s), "detect clear Hw"));
    }
    if (n == 0) return TT_OK;
    const int nbins = nbx * nby;
    long long g = (n + 255) / 256;
    const bool smem = H && nbins <= kSmemBins;
    const long long cap = (long long)tt::sm_count() * (smem ? 4 : 8);
    if (g > cap) g = cap;
    if (smem)
        detect_kernel<true><<<(int)g, 256, sizeof(unsigned) * nbins, s>>>(C, AX, AY, rf, n, weights, H, Hw, r_out);
    else
        detect_kernel<false><<<(int)g, 256, 0, s>>>(C, AX, AY, rf, n, weights, H, Hw, r_out);
    return tt::launch_status("detect kernel");
}
