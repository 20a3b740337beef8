// Learned surrogate: a 2D Fourier neural operator (width 32, 16 retained modes
// per direction) trained and evaluated by the kernels in this file.
//
// Every contraction over pixels runs on the fifth-generation tensor cores
// (tcgen05.mma, BF16 operands staged in shared memory, FP32 accumulators in
// TMEM, read back with tcgen05.ld):
//   rowdft  out[r, j] = sum_x in[r, x] M[j, x]            truncated row DFT along x
//                                                        (forward, and the adjoint of
//                                                        the inverse in the backward pass)
//   mix     out[x, o] = sum_c in[c, x] W[o, c] + sum_j A[x, j] S[o, j]
//                                                        1x1 channel mixing + inverse row
//                                                        DFT, fused, with a bias + GELU or
//                                                        a GELU' epilogue
//   wgrad   dW[o, c] += sum_p dz[o, p] v[c, p]           1x1 weight gradient
// rowdft's input tiles arrive by TMA (cp.async.bulk.tensor); mix and wgrad
// stage their operands through registers (mix transposes to K-major on the
// way).  The DFT along y over the 32 retained ky (and its inverse), and the per-mode
// complex channel mixing, are small and run on the FP32 pipes.  The oracle's
// restatement of the whole network is oracle/fno.py.
//
// Layouts (all device memory owned by the caller):
//   activations  bf16 [B][32][S][S]  (channel-major; one row of x contiguous)
//   row spectra  f32  [B][32][S][32] (j < 16: Re kx = j, j >= 16: Im kx = j - 16)
//   mode spectra f32x2 [B][512][32]  (mode = kyi * 16 + kx, kyi < 16: ky = kyi,
//                                     else ky = S - 32 + kyi)
#include "tt_common.cuh"
#include "tt_umma.cuh"

#include <cuda.h>
#include <cuda_bf16.h>

namespace {

using bf16 = __nv_bfloat16;
using tt::umma::core_offset;

constexpr int W = TT_FNO_WIDTH;  // 32 channels
constexpr int MD = TT_FNO_MODES;  // 16 modes per direction
constexpr int NJ = 2 * MD;         // 32 row-spectrum columns
constexpr int NM = 2 * MD * MD;    // 512 retained modes

// GELU in its tanh form (Hendrycks & Gimpel, 2016),
//   GELU(z) = z/2 (1 + tanh(a(z))),  a(z) = sqrt(2/pi) (z + 0.044715 z^3),
// with the hardware tanh approximation: one MUFU operation instead of an erf.
// Its error (about 2^-11 relative in tanh) is below the bfloat16 rounding of
// every value the kernels store.
constexpr float kGeluA = 0.7978845608028654f;          // sqrt(2/pi)
constexpr float kGeluB = 0.7978845608028654f * 0.044715f;

__device__ __forceinline__ float tanh_approx(float x)
{
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(x));
    return t;
}

__device__ __forceinline__ float gelu_f(float z)
{
    const float t = tanh_approx(z * fmaf(kGeluB, z * z, kGeluA));
    const float h = 0.5f * z;
    return fmaf(h, t, h);
}

// d GELU / dz = (1 + t)/2 + z/2 (1 - t^2) a'(z),  a'(z) = sqrt(2/pi) (1 + 3 * 0.044715 z^2)
__device__ __forceinline__ float gelu_grad_f(float z)
{
    const float z2 = z * z;
    const float t = tanh_approx(z * fmaf(kGeluB, z2, kGeluA));
    const float da = fmaf(3.f * kGeluB, z2, kGeluA);
    return fmaf(0.5f, t, 0.5f) + (0.5f * z) * fmaf(-t, t, 1.f) * da;
}

__device__ __forceinline__ void flag_error(int* err)
{
    if (err) atomicExch(err, 1);
}

// ----------------------------------------------------------------------------- constants
// Row-DFT matrix value at (j, x): kind 0 = forward (cos / -sin), kind 1 =
// inverse with the Hermitian weights c_kx / S^2 (c_0 = 1, c_k = 2).
__device__ float dft_value(int kind, int j, int x, int S)
{
    const int k = j % MD;
    const bool im = j >= MD;
    const int t = (k * x) % S;
    double s, c;
    sincospi(2.0 * (double)t / (double)S, &s, &c);
    double v = im ? -s : c;
    if (kind == 1) v *= (k == 0 ? 1.0 : 2.0) / ((double)S * (double)S);
    return (float)v;
}

// Packed tcgen05 operands of the DFT matrices, and the twiddles of the y DFT:
//   fxt [32 x S] (rowdft B operand, forward), g [32 x S] (rowdft, backward),
//   gt [S x 32] (mix A operand, forward: G transposed), fx [S x 32] (mix, backward).
__global__ void fno_consts_kernel(int S, bf16* fxt, bf16* g, bf16* gt, bf16* fx, float2* tw)
{
    const int n = NJ * S;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int j = i / S, x = i % S;
        const float vf = dft_value(0, j, x, S), vi = dft_value(1, j, x, S);
        fxt[core_offset(j, x, S) / 2] = __float2bfloat16_rn(vf);
        g[core_offset(j, x, S) / 2] = __float2bfloat16_rn(vi);
        gt[core_offset(x, j, NJ) / 2] = __float2bfloat16_rn(vi);
        fx[core_offset(x, j, NJ) / 2] = __float2bfloat16_rn(vf);
        if (j == 0) {
            double s, c;
            sincospi(2.0 * (double)x / (double)S, &s, &c);
            tw[x] = make_float2((float)c, (float)s);
        }
    }
}

// Pack a row-major FP32 matrix [rows x K] into the canonical K-major bf16 layout.
__global__ void fno_pack_kernel(long long rows, int K, const float* __restrict__ src, bf16* __restrict__ dst)
{
    const long long n = rows * K;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / K;
        const int k = (int)(i % K);
        const long long off = (r >> 3) * (long long)(K >> 3) * 128 + core_offset((int)(r & 7), k, K);
        dst[off / 2] = __float2bfloat16_rn(src[i]);
    }
}

struct ParamLayout {
    long long P, pb, Wl[TT_FNO_MAX_LAYERS], bl[TT_FNO_MAX_LAYERS], Rl[TT_FNO_MAX_LAYERS], Q, qb, total;
};

ParamLayout param_layout(const tt_fno_dims& d)
{
    ParamLayout L{};
    const int cin = d.in_ch + 2;
    long long off = 0;
    L.P = off;
    off += (long long)W * cin;
    L.pb = off;
    off += W;
    for (int l = 0; l < d.layers; ++l) {
        L.Wl[l] = off;
        off += W * W;
        L.bl[l] = off;
        off += W;
        L.Rl[l] = off;
        off += (long long)NM * W * W * 2;
    }
    L.Q = off;
    off += (long long)d.out_ch * W;
    L.qb = off;
    off += d.out_ch;
    L.total = off;
    return L;
}

// 1x1 weights of every layer as packed B operands: wf (n = o, k = c) for the
// forward pass, wb (n = c, k = o) for the backward pass; 2 KB each.
struct WPackArgs {
    long long woff[TT_FNO_MAX_LAYERS];
    int layers;
};
__global__ void fno_pack_weights_kernel(WPackArgs a, const float* __restrict__ params, bf16* __restrict__ wpack)
{
    const int l = blockIdx.x;
    if (l >= a.layers) return;
    const float* Wm = params + a.woff[l];
    bf16* wf = wpack + (size_t)l * 2 * W * W;
    bf16* wb = wf + W * W;
    for (int i = threadIdx.x; i < W * W; i += blockDim.x) {
        const int o = i / W, c = i % W;
        const bf16 v = __float2bfloat16_rn(Wm[i]);
        wf[core_offset(o, c, W) / 2] = v;
        wb[core_offset(c, o, W) / 2] = v;
    }
}

// ----------------------------------------------------------------------------- rowdft (tcgen05)
// out[r, 0:32] = sum_x in[r, x] * M[j, x] for r in [0, rows), rows % 128 == 0.
// One 128-row tile per iteration: the tile (128 x S bf16) arrives in shared
// memory by TMA, S/16 MMAs (M = 128, N = 32, K = 16) accumulate into 32 TMEM
// columns.  The tensor map views `in` as rows of S bf16; a tile is S/8 boxes of
// 8 columns x 128 rows, and box kg lands at sA + kg * 2048 as 16 core matrices
// (8 rows x 16 B) stacked along the rows.  So in the A descriptor the core
// matrices adjacent along K are 2048 B apart and the 8-row groups 128 B.
// wait_cycles bounds every mbarrier wait; skip_first_copy (tests only) leaves
// out the copies of each CTA's first tile, so its tile barrier never completes
// and the kernel takes its timeout path (error flag, TMEM freed, return) with
// no copy in flight.
template <int S>
__global__ void __launch_bounds__(128) fno_rowdft_kernel(const __grid_constant__ CUtensorMap amap, long long rows,
                                                         const uint4* __restrict__ mpack, float* __restrict__ out,
                                                         int* __restrict__ err, long long wait_cycles,
                                                         int skip_first_copy)
{
    namespace U = tt::umma;
    constexpr int KG = S / 8;
    constexpr int A_BYTES = 128 * S * 2;
    constexpr int B_BYTES = NJ * S * 2;
    constexpr int KG_BYTES = 128 * 16;  // one box: 128 rows x 8 columns
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + A_BYTES;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + A_BYTES + B_BYTES);  // the MMAs of a tile are done
    uint64_t* tbar = bar + 1;                                              // a tile has arrived
    uint32_t* holder = reinterpret_cast<uint32_t*>(tbar + 1);
    int* abort_flag = reinterpret_cast<int*>(holder + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < B_BYTES / 16; i += 128) reinterpret_cast<uint4*>(sB)[i] = mpack[i];
    U::fence_proxy_async();  // sB written by the threads, read by the tensor cores
    if (tid == 0) {
        U::mbar_init(bar, 1);
        U::mbar_init(tbar, 1);
        *abort_flag = 0;
    }
    if (warp == 0) U::tmem_alloc(holder, 32);
    U::fence_before();
    __syncthreads();
    U::fence_after();
    const uint32_t tmem = *holder;
    const uint32_t idesc = U::idesc_bf16(128, NJ);
    const long long ntiles = rows / 128;
    uint32_t phase = 0, tphase = 0;
    // thread 0: the copies of tile t, issued as soon as the MMAs have read the
    // previous tile, so they land under its epilogue
    auto stage = [&](long long t) {
        U::mbar_arrive_expect_tx(tbar, A_BYTES);
        if (skip_first_copy && t == (long long)blockIdx.x) return;
        for (int kg = 0; kg < KG; ++kg) U::tma_load_2d(sA + kg * KG_BYTES, &amap, kg * 8, (int)(t * 128), tbar);
    };
    if (tid == 0 && (long long)blockIdx.x < ntiles) stage(blockIdx.x);
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        if (tid == 0) {
            if (!U::mbar_wait(tbar, tphase, wait_cycles)) {
                flag_error(err);
                U::mbar_wait(tbar, tphase, wait_cycles);
                *abort_flag = 1;
            } else {
                U::fence_after();
                const uint32_t a0 = U::smem_u32(sA), b0 = U::smem_u32(sB);
#pragma unroll 4
                for (int kk = 0; kk < S / 16; ++kk)
                    U::mma_bf16(tmem, U::desc(a0 + kk * 2 * KG_BYTES, KG_BYTES, 128),
                                U::desc(b0 + kk * 256, 128, KG * 128), idesc, kk > 0);
                U::mma_commit(bar);
                if (!U::mbar_wait(bar, phase, wait_cycles)) {
                    flag_error(err);
                    U::mbar_wait(bar, phase, wait_cycles);
                    *abort_flag = 1;
                }
            }
        }
        phase ^= 1u;
        tphase ^= 1u;
        __syncthreads();
        if (*abort_flag) break;
        if (tid == 0 && t + gridDim.x < ntiles) stage(t + gridDim.x);  // the MMAs are done with sA
        U::fence_after();
        float v[32];
        U::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
        float4* dst = reinterpret_cast<float4*>(out + (t * 128 + warp * 32 + lane) * (long long)NJ);
#pragma unroll
        for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        U::fence_before();
        __syncthreads();
    }
    __syncthreads();
    if (warp == 0) U::tmem_dealloc(tmem, 32);
}

// ----------------------------------------------------------------------------- mix (tcgen05)
// Tile (b, y, x0..x0+127):
//   acc[x, o] = sum_c in[b, c, y, x] Wp[o, c] + sum_j Ap[x, j] sp[b, o, y, j]
// MODE 0 (forward):  z = bf16(acc + bias[o]); out0 = z (if given); out1 = bf16(GELU(z))
// MODE 1 (backward): d = acc, times GELU'(zprev) when zprev is given; out0 = bf16(d)
// The grid size is a multiple of S/128, so each CTA keeps one x tile and its A2 operand.
template <int S, int MODE>
__global__ void __launch_bounds__(128) fno_mix_kernel(int B, const bf16* __restrict__ in,
                                                      const uint4* __restrict__ wpack, const uint4* __restrict__ apack,
                                                      const float* __restrict__ sp, const float* __restrict__ bias,
                                                      const bf16* __restrict__ zprev, bf16* __restrict__ out0,
                                                      bf16* __restrict__ out1, int* __restrict__ err)
{
    namespace U = tt::umma;
    constexpr int XT = S / 128;
    __shared__ __align__(1024) uint8_t sA1[128 * W * 2];
    __shared__ __align__(1024) uint8_t sA2[128 * NJ * 2];
    __shared__ __align__(128) uint8_t sB1[W * W * 2];
    __shared__ __align__(128) uint8_t sB2[W * NJ * 2];
    __shared__ uint64_t bar;
    __shared__ uint32_t holder;
    __shared__ int abort_flag;
    __shared__ float sbias[W];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int xt = blockIdx.x % XT;
    const int x0 = xt * 128;

    for (int i = tid; i < W * W * 2 / 16; i += 128) reinterpret_cast<uint4*>(sB1)[i] = wpack[i];
    for (int i = tid; i < 128 * NJ * 2 / 16; i += 128)
        reinterpret_cast<uint4*>(sA2)[i] = apack[(size_t)xt * (128 * NJ * 2 / 16) + i];
    if (tid < W) sbias[tid] = (MODE == 0 && bias) ? bias[tid] : 0.f;
    if (tid == 0) {
        U::mbar_init(&bar, 1);
        abort_flag = 0;
    }
    if (warp == 0) U::tmem_alloc(&holder, 32);
    U::fence_before();
    __syncthreads();
    U::fence_after();
    const uint32_t tmem = holder;
    const uint32_t idesc = U::idesc_bf16(128, W);
    const long long ntiles = (long long)B * S * XT;
    const size_t plane = (size_t)S * S;
    uint32_t phase = 0;
    // The global loads of tile t + gridDim.x are issued before the epilogue of
    // tile t and land in registers while it runs; the next iteration moves them
    // to shared memory.
    uint4 pin[4];   // in[b, c, y, x0 + 8 xg .. + 8] for xg = 4 warp + it, c = lane
    float4 psp[2];  // sp[b, o, y, 8 jg .. + 8] for o = tid / 4, jg = tid % 4
    auto fetch = [&](long long t) {
        const long long by = t / XT;
        const int b = (int)(by / S), y = (int)(by % S);
        const bf16* row = in + ((size_t)b * W + (tid & 31)) * plane + (size_t)y * S + x0;
#pragma unroll
        for (int it = 0; it < 4; ++it)
            pin[it] = __ldg(reinterpret_cast<const uint4*>(row + ((tid >> 5) * 4 + it) * 8));
        const float4* sv = reinterpret_cast<const float4*>(sp + (((size_t)b * W + (tid >> 2)) * S + y) * NJ +
                                                           (tid & 3) * 8);
        psp[0] = __ldg(sv);
        psp[1] = __ldg(sv + 1);
    };
    if ((long long)blockIdx.x < ntiles) fetch(blockIdx.x);
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long by = t / XT;
        const int b = (int)(by / S), y = (int)(by % S);
        // A1: in[b, c, y, x0:x0+128] transposed into K-major [x][c]; each thread
        // holds 64 contiguous bytes of one channel row
        {
            const int c = tid & 31;
#pragma unroll
            for (int it = 0; it < 4; ++it) {
                const int xg = (tid >> 5) * 4 + it;  // 8-column group, 0..15
                const bf16* e = reinterpret_cast<const bf16*>(&pin[it]);
                uint8_t* base = sA1 + (xg * 4 + (c >> 3)) * 128 + (c & 7) * 2;
#pragma unroll
                for (int i = 0; i < 8; ++i) *reinterpret_cast<bf16*>(base + i * 16) = e[i];
            }
        }
        // B2: sp[b, o, y, 0:32] -> bf16 K-major [o][j]
        {
            const int o = tid >> 2, jg = tid & 3;
            const float4 p0 = psp[0], p1 = psp[1];
            __align__(16) bf16 h[8] = {__float2bfloat16_rn(p0.x), __float2bfloat16_rn(p0.y), __float2bfloat16_rn(p0.z),
                                       __float2bfloat16_rn(p0.w), __float2bfloat16_rn(p1.x), __float2bfloat16_rn(p1.y),
                                       __float2bfloat16_rn(p1.z), __float2bfloat16_rn(p1.w)};
            *reinterpret_cast<uint4*>(sB2 + ((o >> 3) * 4 + jg) * 128 + (o & 7) * 16) = *reinterpret_cast<uint4*>(h);
        }
        U::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            U::fence_after();
            const uint32_t a1 = U::smem_u32(sA1), a2 = U::smem_u32(sA2);
            const uint32_t b1 = U::smem_u32(sB1), b2 = U::smem_u32(sB2);
            U::mma_bf16(tmem, U::desc(a1, 128, 512), U::desc(b1, 128, 512), idesc, 0);
            U::mma_bf16(tmem, U::desc(a1 + 256, 128, 512), U::desc(b1 + 256, 128, 512), idesc, 1);
            U::mma_bf16(tmem, U::desc(a2, 128, 512), U::desc(b2, 128, 512), idesc, 1);
            U::mma_bf16(tmem, U::desc(a2 + 256, 128, 512), U::desc(b2 + 256, 128, 512), idesc, 1);
            U::mma_commit(&bar);
            if (!U::mbar_wait(&bar, phase)) {
                flag_error(err);
                U::mbar_wait(&bar, phase);
                abort_flag = 1;
            }
        }
        phase ^= 1u;
        __syncthreads();
        if (abort_flag) break;
        if (t + gridDim.x < ntiles) fetch(t + gridDim.x);
        U::fence_after();
        float acc[32];
        U::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), acc);
        const int x = x0 + warp * 32 + lane;
        const size_t pix = (size_t)y * S + x;
#pragma unroll  // acc stays in registers
        for (int o = 0; o < W; ++o) {
            const size_t idx = ((size_t)b * W + o) * plane + pix;
            if (MODE == 0) {
                const bf16 zb = __float2bfloat16_rn(acc[o] + sbias[o]);
                if (out0) out0[idx] = zb;
                out1[idx] = __float2bfloat16_rn(gelu_f(__bfloat162float(zb)));
            } else {
                float d = acc[o];
                if (zprev) d *= gelu_grad_f(__bfloat162float(zprev[idx]));
                out0[idx] = __float2bfloat16_rn(d);
            }
        }
        U::fence_before();
        __syncthreads();
    }
    __syncthreads();
    if (warp == 0) U::tmem_dealloc(tmem, 32);
}

// ----------------------------------------------------------------------------- wgrad (tcgen05)
// dW[o, c] += sum_p dz[b, o, p] v[b, c, p], db[o] += sum_p dz[b, o, p].
// A chunk is 256 consecutive pixels of one sample, split into four 64-pixel
// slices q; A rows (q, o) = dz slices, B rows (q, c) = v slices, and one
// M = 128, N = 128 accumulator whose diagonal 32 x 32 blocks hold the four
// partial products (the off-diagonal blocks are not read).  Two smem stages:
// the next chunk is staged while the tensor cores work on the current one.
template <int S>
__global__ void __launch_bounds__(128) fno_wgrad_kernel(int B, const bf16* __restrict__ dz, const bf16* __restrict__ v,
                                                        float* __restrict__ dW, float* __restrict__ db,
                                                        int* __restrict__ err)
{
    namespace U = tt::umma;
    constexpr int TILE = 128 * 64 * 2;  // 16 KB per operand tile
    constexpr long long PIX = (long long)S * S;
    constexpr long long CPS = PIX / 256;  // chunks per sample
    extern __shared__ __align__(1024) uint8_t sm[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 4 * TILE);
    uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 2);
    int* abort_flag = reinterpret_cast<int*>(holder + 1);
    float* sdb = reinterpret_cast<float*>(abort_flag + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long nch = (long long)B * CPS;
    const long long per = (nch + gridDim.x - 1) / gridDim.x;
    const long long c_begin = blockIdx.x * per;
    const long long c_end = c_begin + per < nch ? c_begin + per : nch;
    if (c_begin >= c_end) return;  // uniform across the block: no TMEM taken

    if (tid < W) sdb[tid] = 0.f;
    if (tid == 0) {
        U::mbar_init(&bars[0], 1);
        U::mbar_init(&bars[1], 1);
        *abort_flag = 0;
    }
    if (warp == 0) U::tmem_alloc(holder, 128);
    U::fence_before();
    __syncthreads();
    U::fence_after();
    const uint32_t tmem = *holder;
    const uint32_t idesc = U::idesc_bf16(128, 128);
    uint32_t phase[2] = {0u, 0u};
    bool pending[2] = {false, false};
    // a thread's staged rows of dz always fall on two channels (one per parity
    // of the staging iteration): db is summed in two registers, not atomics
    float dba[2] = {0.f, 0.f};

    for (long long ch = c_begin; ch < c_end; ++ch) {
        const int s = (int)((ch - c_begin) & 1);
        if (pending[s]) {  // the MMAs that read this stage must be done before it is overwritten
            if (tid == 0 && !U::mbar_wait(&bars[s], phase[s])) {
                flag_error(err);
                U::mbar_wait(&bars[s], phase[s]);
                *abort_flag = 1;
            }
            phase[s] ^= 1u;
            pending[s] = false;
            __syncthreads();
            if (*abort_flag) break;
        }
        const long long b = ch / CPS, p0 = (ch % CPS) * 256;
        uint8_t* sA = sm + s * 2 * TILE;
        uint8_t* sB = sA + TILE;
#pragma unroll
        for (int it = 0; it < 8; ++it) {
            const int q = it * 128 + tid;
            const int r8 = q & 7, kg = (q >> 3) & 7, rg = q >> 6;
            const int r = rg * 8 + r8, sl = r >> 5, ch_ = r & 31;
            const size_t g = ((size_t)b * W + ch_) * PIX + p0 + sl * 64 + kg * 8;
            const uint4 va = __ldg(reinterpret_cast<const uint4*>(dz + g));
            const uint4 vb = __ldg(reinterpret_cast<const uint4*>(v + g));
            *reinterpret_cast<uint4*>(sA + (rg * 8 + kg) * 128 + r8 * 16) = va;
            *reinterpret_cast<uint4*>(sB + (rg * 8 + kg) * 128 + r8 * 16) = vb;
            const bf16* e = reinterpret_cast<const bf16*>(&va);
            float sum = 0.f;
#pragma unroll
            for (int i = 0; i < 8; ++i) sum += __bfloat162float(e[i]);
            dba[it & 1] += sum;  // channel ((tid >> 6) + 2 * (it & 1)) * 8 + (tid & 7)
        }
        U::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            U::fence_after();
            const uint32_t a0 = U::smem_u32(sA), b0 = U::smem_u32(sB);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                U::mma_bf16(tmem, U::desc(a0 + kk * 256, 128, 1024), U::desc(b0 + kk * 256, 128, 1024), idesc,
                            (ch > c_begin || kk > 0) ? 1u : 0u);
            U::mma_commit(&bars[s]);
        }
        pending[s] = true;
    }
    // drain: wait for every stage still in flight
    for (int s = 0; s < 2; ++s) {
        if (pending[s]) {
            if (tid == 0 && !U::mbar_wait(&bars[s], phase[s])) {
                flag_error(err);
                U::mbar_wait(&bars[s], phase[s]);
                *abort_flag = 1;
            }
            phase[s] ^= 1u;
        }
    }
#pragma unroll
    for (int p = 0; p < 2; ++p) atomicAdd(&sdb[(((tid >> 6) + 2 * p) & 3) * 8 + (tid & 7)], dba[p]);
    __syncthreads();
    if (!*abort_flag) {
        U::fence_after();
        float acc[32];
        // warp q reads TMEM lanes (q, o = lane), columns of block q: dW partial for slice q
        U::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(warp * 32), acc);
        // sum the four slice partials in shared memory (the operand stages are
        // free now; rows padded to 33 floats), then one coalesced atomic per
        // element of dW from this block
        float* part = reinterpret_cast<float*>(sm);
#pragma unroll
        for (int c = 0; c < W; ++c) part[(warp * W + lane) * (W + 1) + c] = acc[c];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < W * W / 128; ++i) {
            const int a = tid + 128 * i, o = a / W, c = a % W;
            float tot = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) tot += part[(q * W + o) * (W + 1) + c];
            atomicAdd(&dW[a], tot);
        }
        if (tid < W) atomicAdd(&db[tid], sdb[tid]);
    }
    U::fence_before();
    __syncthreads();
    if (warp == 0) U::tmem_dealloc(tmem, 128);
}

// ----------------------------------------------------------------------------- y DFTs (FP32)
// Y[b, m, c] = sum_y X[b, c, y, kx] exp(-2 pi i ky y / S) over the 32 retained ky.
// One block per (b, c): kYdftSplit groups of 128 threads each sum a quarter of
// the rows y for a 2 (ky) x 2 (kx) tile of modes per thread (4 shared loads
// for 16 FMAs a row); the partial sums are added in shared memory in a fixed
// order.
constexpr int kYdftTile = 128;
constexpr int kYdftSplit = 4;
constexpr int kYdftThreads = kYdftTile * kYdftSplit;

template <int S>
__global__ void __launch_bounds__(kYdftThreads) fno_ydft_kernel(const float* __restrict__ X,
                                                                const float2* __restrict__ tw, float2* __restrict__ Y)
{
    static_assert(kYdftTile == (MD / 2) * (NJ / 2), "one 2 x 2 tile of modes per thread of a group");
    static_assert(S % kYdftSplit == 0, "whole row quarters");
    __shared__ __align__(16) float xs[S * NJ];
    __shared__ float2 tws[S];
    __shared__ float4 part[kYdftSplit - 1][kYdftTile][2];
    const int bc = blockIdx.x, b = bc / W, c = bc % W;
    const float4* src = reinterpret_cast<const float4*>(X + (size_t)bc * S * NJ);
    for (int i = threadIdx.x; i < S * NJ / 4; i += kYdftThreads) reinterpret_cast<float4*>(xs)[i] = __ldg(src + i);
    for (int i = threadIdx.x; i < S; i += kYdftThreads) tws[i] = tw[i];
    __syncthreads();
    const int t = threadIdx.x % kYdftTile, g = threadIdx.x / kYdftTile;
    const int kx0 = 2 * (t % (MD / 2)), kyi0 = 2 * (t / (MD / 2));
    int ky[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) ky[q] = kyi0 + q < MD ? kyi0 + q : S - NJ + kyi0 + q;
    float ar[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, ai[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    constexpr int RY = S / kYdftSplit;
#pragma unroll 4
    for (int y = g * RY; y < (g + 1) * RY; ++y) {
        const float2 xr = *reinterpret_cast<const float2*>(xs + y * NJ + kx0);
        const float2 xi = *reinterpret_cast<const float2*>(xs + y * NJ + MD + kx0);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const float2 e = tws[(ky[q] * y) & (S - 1)];
            ar[q][0] = fmaf(xr.x, e.x, fmaf(xi.x, e.y, ar[q][0]));
            ai[q][0] = fmaf(xi.x, e.x, fmaf(-xr.x, e.y, ai[q][0]));
            ar[q][1] = fmaf(xr.y, e.x, fmaf(xi.y, e.y, ar[q][1]));
            ai[q][1] = fmaf(xi.y, e.x, fmaf(-xr.y, e.y, ai[q][1]));
        }
    }
    if (g > 0) {
        part[g - 1][t][0] = make_float4(ar[0][0], ai[0][0], ar[0][1], ai[0][1]);
        part[g - 1][t][1] = make_float4(ar[1][0], ai[1][0], ar[1][1], ai[1][1]);
    }
    __syncthreads();
    if (g == 0) {
#pragma unroll
        for (int h = 0; h < kYdftSplit - 1; ++h) {
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float4 v = part[h][t][q];
                ar[q][0] += v.x, ai[q][0] += v.y, ar[q][1] += v.z, ai[q][1] += v.w;
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int j = 0; j < 2; ++j)
                Y[((size_t)b * NM + (kyi0 + q) * MD + kx0 + j) * W + c] = make_float2(ar[q][j], ai[q][j]);
    }
}

// X[b, c, y, kx] = sum_ky Y[b, m(ky, kx), c] exp(+2 pi i ky y / S).
// One block per (b, c) of 2 S threads; a thread owns a kx pair and 4 rows y
// (a 4 x 2 tile: 6 shared loads for 32 FMAs a ky).
template <int S>
__global__ void __launch_bounds__(2 * S) fno_iydft_kernel(const float2* __restrict__ Y, const float2* __restrict__ tw,
                                                          float* __restrict__ X)
{
    constexpr int KXP = MD / 2;      // kx pairs
    constexpr int YG = 2 * S / KXP;  // row groups: rows yg + YG r, r = 0..3
    static_assert(4 * YG == S, "4 rows a thread");
    __shared__ __align__(16) float2 ys[NM];
    __shared__ float2 tws[S];
    const int bc = blockIdx.x, b = bc / W, c = bc % W;
    for (int m = threadIdx.x; m < NM; m += 2 * S) ys[m] = Y[((size_t)b * NM + m) * W + c];
    for (int i = threadIdx.x; i < S; i += 2 * S) tws[i] = tw[i];
    __syncthreads();
    float* dst = X + (size_t)bc * S * NJ;
    const int kx0 = 2 * (threadIdx.x % KXP), yg = threadIdx.x / KXP;
    float xr[4][2] = {}, xi[4][2] = {};
#pragma unroll 4
    for (int kyi = 0; kyi < NJ; ++kyi) {
        const int ky = kyi < MD ? kyi : S - NJ + kyi;
        const float4 u = *reinterpret_cast<const float4*>(ys + kyi * MD + kx0);  // (u0.x, u0.y, u1.x, u1.y)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const float2 e = tws[(ky * (yg + r * YG)) & (S - 1)];
            xr[r][0] = fmaf(u.x, e.x, fmaf(-u.y, e.y, xr[r][0]));
            xi[r][0] = fmaf(u.x, e.y, fmaf(u.y, e.x, xi[r][0]));
            xr[r][1] = fmaf(u.z, e.x, fmaf(-u.w, e.y, xr[r][1]));
            xi[r][1] = fmaf(u.z, e.y, fmaf(u.w, e.x, xi[r][1]));
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int y = yg + r * YG;
        *reinterpret_cast<float2*>(dst + y * NJ + kx0) = make_float2(xr[r][0], xr[r][1]);
        *reinterpret_cast<float2*>(dst + y * NJ + MD + kx0) = make_float2(xi[r][0], xi[r][1]);
    }
}

// ----------------------------------------------------------------------------- mode mixing (FP32)
// U[b, m, o] = sum_c R[m, o, c] T2[b, m, c]   (complex)
__global__ void __launch_bounds__(256) fno_specmix_fwd_kernel(int B, const float2* __restrict__ R,
                                                              const float2* __restrict__ T2, float2* __restrict__ Uo)
{
    __shared__ float2 rm[W][W + 1];
    __shared__ float2 ts[8][W];
    const int m = blockIdx.x;
    for (int i = threadIdx.x; i < W * W; i += 256) rm[i / W][i % W] = R[(size_t)m * W * W + i];
    const int bi = threadIdx.x / W, o = threadIdx.x % W;
    for (int b0 = 0; b0 < B; b0 += 8) {
        __syncthreads();
        if (b0 + bi < B) ts[bi][o] = T2[((size_t)(b0 + bi) * NM + m) * W + o];
        __syncthreads();
        if (b0 + bi < B) {
            float ur = 0.f, ui = 0.f;
#pragma unroll 8
            for (int c = 0; c < W; ++c) {
                const float2 r = rm[o][c], t = ts[bi][c];
                ur = fmaf(r.x, t.x, fmaf(-r.y, t.y, ur));
                ui = fmaf(r.x, t.y, fmaf(r.y, t.x, ui));
            }
            Uo[((size_t)(b0 + bi) * NM + m) * W + o] = make_float2(ur, ui);
        }
    }
}

// dT2[b, m, c] = sum_o conj(R[m, o, c]) dU[b, m, o];  dR[m, o, c] += sum_b dU[b, m, o] conj(T2[b, m, c])
__global__ void __launch_bounds__(256) fno_specmix_bwd_kernel(int B, const float2* __restrict__ R,
                                                              const float2* __restrict__ T2,
                                                              const float2* __restrict__ dU, float2* __restrict__ dT2,
                                                              float2* __restrict__ dR)
{
    __shared__ float2 rm[W][W + 1];
    __shared__ float2 ts[8][W];
    __shared__ float2 us[8][W];
    const int m = blockIdx.x;
    for (int i = threadIdx.x; i < W * W; i += 256) rm[i / W][i % W] = R[(size_t)m * W * W + i];
    const int bi = threadIdx.x / W, c = threadIdx.x % W;
    float2 acc[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    for (int b0 = 0; b0 < B; b0 += 8) {
        __syncthreads();
        if (b0 + bi < B) {
            ts[bi][c] = T2[((size_t)(b0 + bi) * NM + m) * W + c];
            us[bi][c] = dU[((size_t)(b0 + bi) * NM + m) * W + c];
        } else {
            ts[bi][c] = make_float2(0.f, 0.f);
            us[bi][c] = make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (b0 + bi < B) {
            float gr = 0.f, gi = 0.f;
#pragma unroll 8
            for (int o = 0; o < W; ++o) {
                const float2 r = rm[o][c], u = us[bi][o];
                gr = fmaf(r.x, u.x, fmaf(r.y, u.y, gr));  // conj(r) * u
                gi = fmaf(r.x, u.y, fmaf(-r.y, u.x, gi));
            }
            dT2[((size_t)(b0 + bi) * NM + m) * W + c] = make_float2(gr, gi);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int p = threadIdx.x + 256 * k, o = p / W, cc = p % W;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float2 u = us[j][o], t = ts[j][cc];
                acc[k].x = fmaf(u.x, t.x, fmaf(u.y, t.y, acc[k].x));  // u * conj(t)
                acc[k].y = fmaf(u.y, t.x, fmaf(-u.x, t.y, acc[k].y));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int p = threadIdx.x + 256 * k;
        float2* d = dR + (size_t)m * W * W + p;
        *d = make_float2(d->x + acc[k].x, d->y + acc[k].y);
    }
}

// ----------------------------------------------------------------------------- lift / projection
// v0[b, c, p] = bf16(sum_i P[c, i] in_i + pb[c]), in = (data channels, row coordinate, column coordinate)
constexpr int MAXC = TT_FNO_MAX_IN + 2;

__device__ __forceinline__ void lift_inputs(const float* __restrict__ a, int cd, long long b, long long p, int S,
                                            long long plane, float (&in)[MAXC])
{
#pragma unroll
    for (int k = 0; k < MAXC; ++k) in[k] = 0.f;
#pragma unroll
    for (int k = 0; k < TT_FNO_MAX_IN; ++k)
        if (k < cd) in[k] = a[(b * cd + k) * plane + p];
    const float ry = ((float)(p / S) + 0.5f) * (2.0f / S) - 1.0f;
    const float rx = ((float)(p % S) + 0.5f) * (2.0f / S) - 1.0f;
#pragma unroll
    for (int k = 0; k < MAXC; ++k) {
        if (k == cd) in[k] = ry;
        if (k == cd + 1) in[k] = rx;
    }
}

__global__ void fno_lift_kernel(int B, int S, int cd, const float* __restrict__ a, const float* __restrict__ P,
                                const float* __restrict__ pb, bf16* __restrict__ v0)
{
    __shared__ float sP[W * MAXC];
    __shared__ float spb[W];
    const int cin = cd + 2;
    for (int i = threadIdx.x; i < W * MAXC; i += blockDim.x) {
        const int c = i / MAXC, k = i % MAXC;
        sP[i] = k < cin ? P[c * cin + k] : 0.f;
    }
    for (int i = threadIdx.x; i < W; i += blockDim.x) spb[i] = pb[i];
    __syncthreads();
    const long long plane = (long long)S * S, n = (long long)B * plane;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long b = i / plane, p = i % plane;
        float in[MAXC];
        lift_inputs(a, cd, b, p, S, plane, in);
#pragma unroll 4
        for (int c = 0; c < W; ++c) {
            float s = spb[c];
#pragma unroll
            for (int k = 0; k < MAXC; ++k) s = fmaf(sP[c * MAXC + k], in[k], s);
            v0[(b * W + c) * plane + p] = __float2bfloat16_rn(s);
        }
    }
}

// dP[c, i] += sum g0[b, c, p] in_i,  dpb[c] += sum g0[b, c, p].  Warp w handles
// channels w, w + 8, w + 16, w + 24; lanes stride over the block's pixels.
__global__ void __launch_bounds__(256) fno_lift_bwd_kernel(int B, int S, int cd, const bf16* __restrict__ g0,
                                                           const float* __restrict__ a, float* __restrict__ dP,
                                                           float* __restrict__ dpb)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cin = cd + 2;
    const long long plane = (long long)S * S, n = (long long)B * plane;
    const long long per = (n + gridDim.x - 1) / gridDim.x;
    const long long i0 = blockIdx.x * per, i1 = i0 + per < n ? i0 + per : n;
    float acc[4][MAXC + 1];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int k = 0; k < MAXC + 1; ++k) acc[q][k] = 0.f;
    for (long long i = i0 + lane; i < i1; i += 32) {
        const long long b = i / plane, p = i % plane;
        float in[MAXC];
        lift_inputs(a, cd, b, p, S, plane, in);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = warp + 8 * q;
            const float g = __bfloat162float(g0[(b * W + c) * plane + p]);
#pragma unroll
            for (int k = 0; k < MAXC; ++k) acc[q][k] = fmaf(g, in[k], acc[q][k]);
            acc[q][MAXC] += g;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = warp + 8 * q;
#pragma unroll
        for (int k = 0; k < MAXC + 1; ++k) {
            float s = acc[q][k];
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
            if (lane == 0) {
                if (k == MAXC) atomicAdd(&dpb[c], s);
                else if (k < cin) atomicAdd(&dP[c * cin + k], s);
            }
        }
    }
}

// Projection out[b, k, p] = sum_c Q[k, c] v[b, c, p] + qb[k].  With a target
// (training): loss += sum_k w_k (out - t)^2 / (B S^2), dout = 2 w_k (out - t) / (B S^2),
// dz[b, c, p] = bf16((sum_k Q[k, c] dout_k) GELU'(z[b, c, p])), dQ += dout v, dqb += dout.
struct ProjW {
    float w[TT_FNO_MAX_OUT];
};
template <int COUT, bool TRAIN>
__global__ void __launch_bounds__(256) fno_proj_kernel(int B, int S, const bf16* __restrict__ v,
                                                       const float* __restrict__ Q, const float* __restrict__ qb,
                                                       const float* __restrict__ tgt, ProjW cw,
                                                       const bf16* __restrict__ z, float* __restrict__ out,
                                                       bf16* __restrict__ dz, float* __restrict__ dQ,
                                                       float* __restrict__ dqb, float* __restrict__ loss)
{
    __shared__ float sQ[COUT * W];
    __shared__ float red[COUT * W + COUT + 1];
    for (int i = threadIdx.x; i < COUT * W; i += blockDim.x) sQ[i] = Q[i];
    for (int i = threadIdx.x; i < COUT * W + COUT + 1; i += blockDim.x) red[i] = 0.f;
    __syncthreads();
    const long long plane = (long long)S * S, n = (long long)B * plane;
    const float inv_n = 1.0f / (float)n;
    float aQ[TRAIN ? COUT * W : 1];
    float aq[COUT], al = 0.f;
#pragma unroll
    for (int i = 0; i < (TRAIN ? COUT * W : 1); ++i) aQ[i] = 0.f;
#pragma unroll
    for (int k = 0; k < COUT; ++k) aq[k] = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long b = i / plane, p = i % plane;
        float vv[W];
#pragma unroll
        for (int c = 0; c < W; ++c) vv[c] = __bfloat162float(v[(b * W + c) * plane + p]);
        float o[COUT];
#pragma unroll
        for (int k = 0; k < COUT; ++k) {
            float s = qb[k];
#pragma unroll
            for (int c = 0; c < W; ++c) s = fmaf(sQ[k * W + c], vv[c], s);
            o[k] = s;
        }
        if (!TRAIN) {
#pragma unroll
            for (int k = 0; k < COUT; ++k) out[(b * COUT + k) * plane + p] = o[k];
        } else {
            float dout[COUT];
#pragma unroll
            for (int k = 0; k < COUT; ++k) {
                const float d = o[k] - tgt[(b * COUT + k) * plane + p];
                al = fmaf(cw.w[k] * d, d, al);
                dout[k] = 2.0f * cw.w[k] * d * inv_n;
                aq[k] += dout[k];
                if (out) out[(b * COUT + k) * plane + p] = o[k];
            }
#pragma unroll
            for (int c = 0; c < W; ++c) {
                float g = 0.f;
#pragma unroll
                for (int k = 0; k < COUT; ++k) {
                    g = fmaf(sQ[k * W + c], dout[k], g);
                    aQ[k * W + c] = fmaf(dout[k], vv[c], aQ[k * W + c]);
                }
                const size_t idx = (b * W + c) * plane + p;
                dz[idx] = __float2bfloat16_rn(g * gelu_grad_f(__bfloat162float(z[idx])));
            }
        }
    }
    if (!TRAIN) return;
    const int lane = threadIdx.x & 31;
    auto wsum = [&](float s) {
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        return s;
    };
#pragma unroll
    for (int i = 0; i < COUT * W; ++i) {
        const float s = wsum(aQ[i]);
        if (lane == 0) atomicAdd(&red[i], s);
    }
#pragma unroll
    for (int k = 0; k < COUT; ++k) {
        const float s = wsum(aq[k]);
        if (lane == 0) atomicAdd(&red[COUT * W + k], s);
    }
    {
        const float s = wsum(al);
        if (lane == 0) atomicAdd(&red[COUT * W + COUT], s);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < COUT * W; i += blockDim.x) atomicAdd(&dQ[i], red[i]);
    for (int k = threadIdx.x; k < COUT; k += blockDim.x) atomicAdd(&dqb[k], red[COUT * W + k]);
    if (threadIdx.x == 0) atomicAdd(loss, red[COUT * W + COUT] * inv_n);
}

// ----------------------------------------------------------------------------- Adam
__global__ void fno_adam_kernel(long long n, float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
        const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        g[i] = 0.f;
    }
}

// The same update with the learning rate and the step counter in device
// memory, so a captured training step can be replayed with a schedule.
__global__ void fno_step_inc_kernel(long long* step) { *step += 1; }

__global__ void fno_adam_dev_kernel(long long n, float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                                    float* __restrict__ v, const float* __restrict__ lr_dev, float b1, float b2,
                                    float eps, const long long* __restrict__ step)
{
    __shared__ float sc[3];
    if (threadIdx.x == 0) {
        const float t = (float)*step;
        sc[0] = *lr_dev;
        sc[1] = 1.0f - powf(b1, t);
        sc[2] = 1.0f - powf(b2, t);
    }
    __syncthreads();
    const float lr = sc[0], bc1 = sc[1], bc2 = sc[2];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
        const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        g[i] = 0.f;
    }
}

// ----------------------------------------------------------------------------- host side
int check_dims(const tt_fno_dims* d)
{
    if (!d) return tt::invalid("tt_fno: dims is NULL");
    if (d->size != 128 && d->size != 256) return tt::invalid("tt_fno: size must be 128 or 256");
    if (d->batch < 1) return tt::invalid("tt_fno: batch must be >= 1");
    if (d->in_ch < 1 || d->in_ch > TT_FNO_MAX_IN) return tt::invalid("tt_fno: in_ch out of range");
    if (d->out_ch < 1 || d->out_ch > TT_FNO_MAX_OUT) return tt::invalid("tt_fno: out_ch out of range");
    if (d->layers < 1 || d->layers > TT_FNO_MAX_LAYERS) return tt::invalid("tt_fno: layers out of range");
    return TT_OK;
}

struct WsLayout {
    size_t err, fxt, g, gt, fx, tw, wpack, v, z, rowbuf, t2, u, dt2, dz, total;
    size_t act;  // bytes of one activation tensor
};

WsLayout ws_layout(const tt_fno_dims& d, bool training)
{
    WsLayout L{};
    const size_t S = (size_t)d.size, B = (size_t)d.batch;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = tt::align_up(off + bytes, 1024);
        return o;
    };
    L.act = B * W * S * S * 2;
    L.err = take(256);
    L.fxt = take(NJ * S * 2);
    L.g = take(NJ * S * 2);
    L.gt = take(NJ * S * 2);
    L.fx = take(NJ * S * 2);
    L.tw = take(S * sizeof(float2));
    L.wpack = take((size_t)d.layers * 2 * W * W * 2);
    L.v = take(L.act * (training ? (size_t)d.layers + 1 : 2));
    L.z = take(training ? L.act * d.layers : 0);
    L.rowbuf = take(B * W * S * NJ * 4);
    L.t2 = take(B * NM * W * sizeof(float2) * (training ? d.layers : 1));
    L.u = take(B * NM * W * sizeof(float2));
    L.dt2 = take(training ? B * NM * W * sizeof(float2) : 0);
    L.dz = take(training ? 2 * L.act : 0);
    L.total = off;
    return L;
}

template <typename T>
T* at(void* ws, size_t off)
{
    return reinterpret_cast<T*>(static_cast<uint8_t*>(ws) + off);
}

int grid_for(long long work, int per_sm)
{
    const long long g = (long long)tt::sm_count() * per_sm;
    return (int)(work < g ? (work > 0 ? work : 1) : g);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return EncodeTiledFn{nullptr};
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

template <int S>
int launch_rowdft(const bf16* in, long long rows, const void* mpack, float* out, int* err, cudaStream_t st,
                  long long wait_cycles = tt::umma::kWaitCycles, int skip_first_copy = 0)
{
    constexpr int smem = 128 * S * 2 + NJ * S * 2 + 64;
    // the tensor map: rows of S bf16 (S * 2 bytes apart), boxes of 8 columns x 128 rows
    if ((reinterpret_cast<uintptr_t>(in) & 15) != 0 || rows % 128 != 0 || rows > 0x7fffffffLL)
        return tt::invalid("fno_rowdft: rows must be 16-byte aligned, a multiple of 128 and below 2^31");
    const EncodeTiledFn enc = encode_tiled();
    if (!enc) {
        tt::set_detail("fno_rowdft: cuTensorMapEncodeTiled is not available from the driver");
        return TT_ERR_CUDA;
    }
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)S, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)S * 2};
    const cuuint32_t box[2] = {8, 128};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(in), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        tt::set_detail("fno_rowdft: cuTensorMapEncodeTiled failed (%d)", (int)r);
        return TT_ERR_CUDA;
    }
    TT_TRY(tt::cuda_status(cudaFuncSetAttribute(fno_rowdft_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                smem),
                           "fno_rowdft attribute"));
    fno_rowdft_kernel<S><<<grid_for(rows / 128, 2), 128, smem, st>>>(map, rows, (const uint4*)mpack, out, err,
                                                                      wait_cycles, skip_first_copy);
    return tt::launch_status("fno_rowdft_kernel");
}

template <int S, int MODE>
int launch_mix(int B, const bf16* in, const void* wpack, const void* apack, const float* sp, const float* bias,
               const bf16* zprev, bf16* out0, bf16* out1, int* err, cudaStream_t st)
{
    constexpr int XT = S / 128;
    int g = grid_for((long long)B * S * XT, 6);  // 80 registers: 6 blocks per SM
    g = (g / XT) * XT;
    if (g < XT) g = XT;
    fno_mix_kernel<S, MODE><<<g, 128, 0, st>>>(B, in, (const uint4*)wpack, (const uint4*)apack, sp, bias, zprev, out0,
                                               out1, err);
    return tt::launch_status("fno_mix_kernel");
}

template <int S>
int launch_wgrad(int B, const bf16* dz, const bf16* v, float* dW, float* db, int* err, cudaStream_t st)
{
    constexpr int smem = 4 * 128 * 64 * 2 + 256;
    TT_TRY(tt::cuda_status(cudaFuncSetAttribute(fno_wgrad_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                smem),
                           "fno_wgrad attribute"));
    const long long nch = (long long)B * S * S / 256;
    fno_wgrad_kernel<S><<<grid_for(nch, 2), 128, smem, st>>>(B, dz, v, dW, db, err);
    return tt::launch_status("fno_wgrad_kernel");
}

int build_consts(const tt_fno_dims& d, const WsLayout& L, void* ws, cudaStream_t st)
{
    fno_consts_kernel<<<64, 256, 0, st>>>(d.size, at<bf16>(ws, L.fxt), at<bf16>(ws, L.g), at<bf16>(ws, L.gt),
                                          at<bf16>(ws, L.fx), at<float2>(ws, L.tw));
    return tt::launch_status("fno_consts_kernel");
}

int pack_weights(const tt_fno_dims& d, const ParamLayout& P, const float* params, const WsLayout& L, void* ws,
                 cudaStream_t st)
{
    WPackArgs a{};
    a.layers = d.layers;
    for (int l = 0; l < d.layers; ++l) a.woff[l] = P.Wl[l];
    fno_pack_weights_kernel<<<d.layers, 256, 0, st>>>(a, params, at<bf16>(ws, L.wpack));
    return tt::launch_status("fno_pack_weights_kernel");
}

template <int S>
int forward_layers(const tt_fno_dims& d, const ParamLayout& P, const float* params, const float* a, const WsLayout& L,
                   void* ws, bool training, cudaStream_t st)
{
    const int B = d.batch;
    int* err = at<int>(ws, L.err);
    auto v = [&](int l) { return at<bf16>(ws, L.v + L.act * (training ? (size_t)l : (size_t)(l & 1))); };
    float* row = at<float>(ws, L.rowbuf);
    float2* U = at<float2>(ws, L.u);
    const float2* tw = at<float2>(ws, L.tw);
    fno_lift_kernel<<<grid_for((long long)B * S * S / 256, 4), 256, 0, st>>>(B, S, d.in_ch, a, params + P.P,
                                                                            params + P.pb, v(0));
    TT_TRY(tt::launch_status("fno_lift_kernel"));
    for (int l = 0; l < d.layers; ++l) {
        float2* T2 = at<float2>(ws, L.t2) + (training ? (size_t)l * B * NM * W : 0);
        TT_TRY(launch_rowdft<S>(v(l), (long long)B * W * S, at<void>(ws, L.fxt), row, err, st));
        fno_ydft_kernel<S><<<B * W, kYdftThreads, 0, st>>>(row, tw, T2);
        TT_TRY(tt::launch_status("fno_ydft_kernel"));
        fno_specmix_fwd_kernel<<<NM, 256, 0, st>>>(B, reinterpret_cast<const float2*>(params + P.Rl[l]), T2, U);
        TT_TRY(tt::launch_status("fno_specmix_fwd_kernel"));
        fno_iydft_kernel<S><<<B * W, 2 * S, 0, st>>>(U, tw, row);
        TT_TRY(tt::launch_status("fno_iydft_kernel"));
        bf16* z = training ? at<bf16>(ws, L.z + L.act * (size_t)l) : nullptr;
        TT_TRY((launch_mix<S, 0>(B, v(l), at<bf16>(ws, L.wpack) + (size_t)l * 2 * W * W, at<void>(ws, L.gt), row,
                                 params + P.bl[l], nullptr, z, v(l + 1), err, st)));
    }
    return TT_OK;
}

template <int S, int COUT>
int run_forward(const tt_fno_dims& d, const float* params, const float* a, float* out, void* ws, cudaStream_t st)
{
    const ParamLayout P = param_layout(d);
    const WsLayout L = ws_layout(d, false);
    TT_TRY(build_consts(d, L, ws, st));
    TT_TRY(pack_weights(d, P, params, L, ws, st));
    TT_TRY(forward_layers<S>(d, P, params, a, L, ws, false, st));
    const bf16* vL = at<bf16>(ws, L.v + L.act * (size_t)(d.layers & 1));
    fno_proj_kernel<COUT, false><<<grid_for((long long)d.batch * S * S / 256, 4), 256, 0, st>>>(
        d.batch, S, vL, params + P.Q, params + P.qb, nullptr, ProjW{}, nullptr, out, nullptr, nullptr, nullptr,
        nullptr);
    return tt::launch_status("fno_proj_kernel");
}

template <int S, int COUT>
int run_train(const tt_fno_dims& d, const float* params, float* grads, const float* a, const float* tgt,
              const float* cw, float* loss, float* out, void* ws, cudaStream_t st)
{
    const ParamLayout P = param_layout(d);
    const WsLayout L = ws_layout(d, true);
    const int B = d.batch;
    int* err = at<int>(ws, L.err);
    TT_TRY(build_consts(d, L, ws, st));
    TT_TRY(pack_weights(d, P, params, L, ws, st));
    TT_TRY(forward_layers<S>(d, P, params, a, L, ws, true, st));
    auto v = [&](int l) { return at<bf16>(ws, L.v + L.act * (size_t)l); };
    auto z = [&](int l) { return at<bf16>(ws, L.z + L.act * (size_t)l); };
    auto dzb = [&](int i) { return at<bf16>(ws, L.dz + L.act * (size_t)(i & 1)); };
    ProjW w{};
    for (int k = 0; k < COUT; ++k) w.w[k] = cw ? cw[k] : 1.0f;
    fno_proj_kernel<COUT, true><<<grid_for((long long)B * S * S / 256, 4), 256, 0, st>>>(
        B, S, v(d.layers), params + P.Q, params + P.qb, tgt, w, z(d.layers - 1), out, dzb(0), grads + P.Q,
        grads + P.qb, loss);
    TT_TRY(tt::launch_status("fno_proj_kernel"));
    float* row = at<float>(ws, L.rowbuf);
    float2* dU = at<float2>(ws, L.u);
    float2* dT2 = at<float2>(ws, L.dt2);
    const float2* tw = at<float2>(ws, L.tw);
    int cur = 0;
    for (int l = d.layers - 1; l >= 0; --l) {
        const bf16* dz = dzb(cur);
        bf16* nxt = dzb(cur + 1);
        const float2* T2 = at<float2>(ws, L.t2) + (size_t)l * B * NM * W;
        TT_TRY(launch_wgrad<S>(B, dz, v(l), grads + P.Wl[l], grads + P.bl[l], err, st));
        TT_TRY(launch_rowdft<S>(dz, (long long)B * W * S, at<void>(ws, L.g), row, err, st));
        fno_ydft_kernel<S><<<B * W, kYdftThreads, 0, st>>>(row, tw, dU);
        TT_TRY(tt::launch_status("fno_ydft_kernel"));
        fno_specmix_bwd_kernel<<<NM, 256, 0, st>>>(B, reinterpret_cast<const float2*>(params + P.Rl[l]), T2, dU, dT2,
                                                   reinterpret_cast<float2*>(grads + P.Rl[l]));
        TT_TRY(tt::launch_status("fno_specmix_bwd_kernel"));
        fno_iydft_kernel<S><<<B * W, 2 * S, 0, st>>>(dT2, tw, row);
        TT_TRY(tt::launch_status("fno_iydft_kernel"));
        TT_TRY((launch_mix<S, 1>(B, dz, at<bf16>(ws, L.wpack) + (size_t)l * 2 * W * W + W * W, at<void>(ws, L.fx), row,
                                 nullptr, l > 0 ? z(l - 1) : nullptr, nxt, nullptr, err, st)));
        cur += 1;
    }
    fno_lift_bwd_kernel<<<grid_for((long long)B * S * S / 1024, 4), 256, 0, st>>>(B, S, d.in_ch, dzb(cur), a,
                                                                                grads + P.P, grads + P.pb);
    return tt::launch_status("fno_lift_bwd_kernel");
}

template <int S>
int dispatch_train(const tt_fno_dims& d, const float* params, float* grads, const float* a, const float* tgt,
                   const float* cw, float* loss, float* out, void* ws, cudaStream_t st)
{
    switch (d.out_ch) {
        case 1: return run_train<S, 1>(d, params, grads, a, tgt, cw, loss, out, ws, st);
        case 2: return run_train<S, 2>(d, params, grads, a, tgt, cw, loss, out, ws, st);
        case 3: return run_train<S, 3>(d, params, grads, a, tgt, cw, loss, out, ws, st);
        default: return run_train<S, 4>(d, params, grads, a, tgt, cw, loss, out, ws, st);
    }
}

template <int S>
int dispatch_forward(const tt_fno_dims& d, const float* params, const float* a, float* out, void* ws, cudaStream_t st)
{
    switch (d.out_ch) {
        case 1: return run_forward<S, 1>(d, params, a, out, ws, st);
        case 2: return run_forward<S, 2>(d, params, a, out, ws, st);
        case 3: return run_forward<S, 3>(d, params, a, out, ws, st);
        default: return run_forward<S, 4>(d, params, a, out, ws, st);
    }
}

}  // namespace

extern "C" {

size_t tt_fno_param_count(const tt_fno_dims* d)
{
    if (check_dims(d) != TT_OK) return 0;
    return (size_t)param_layout(*d).total;
}

size_t tt_fno_workspace_bytes(const tt_fno_dims* d, int training)
{
    if (check_dims(d) != TT_OK) return 0;
    return ws_layout(*d, training != 0).total;
}

int tt_fno_forward(const tt_fno_dims* d, const float* params, const float* a, float* out, void* ws,
                   size_t ws_bytes, void* stream)
{
    TT_TRY(check_dims(d));
    if (!params || !a || !out || !ws) return tt::invalid("tt_fno_forward: NULL pointer");
    if (ws_bytes < ws_layout(*d, false).total) return tt::invalid("tt_fno_forward: workspace too small");
    cudaStream_t st = tt::as_stream(stream);
    return d->size == 128 ? dispatch_forward<128>(*d, params, a, out, ws, st)
                          : dispatch_forward<256>(*d, params, a, out, ws, st);
}

int tt_fno_train_step(const tt_fno_dims* d, const float* params, float* grads, const float* a, const float* target,
                      const float* channel_weights, float* loss, float* out, void* ws, size_t ws_bytes, void* stream)
{
    TT_TRY(check_dims(d));
    if (!params || !grads || !a || !target || !loss || !ws) return tt::invalid("tt_fno_train_step: NULL pointer");
    if (ws_bytes < ws_layout(*d, true).total) return tt::invalid("tt_fno_train_step: workspace too small");
    cudaStream_t st = tt::as_stream(stream);
    return d->size == 128 ? dispatch_train<128>(*d, params, grads, a, target, channel_weights, loss, out, ws, st)
                          : dispatch_train<256>(*d, params, grads, a, target, channel_weights, loss, out, ws, st);
}

int tt_fno_adam(int64_t n, float* params, float* grads, float* m, float* v, float lr, float beta1, float beta2,
                float eps, int64_t step, void* stream)
{
    if (n <= 0 || !params || !grads || !m || !v) return tt::invalid("tt_fno_adam: bad arguments");
    if (step < 1) return tt::invalid("tt_fno_adam: step counts from 1");
    const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
    fno_adam_kernel<<<grid_for(n / 256 + 1, 4), 256, 0, tt::as_stream(stream)>>>(n, params, grads, m, v, lr, beta1,
                                                                                 beta2, eps, bc1, bc2);
    return tt::launch_status("fno_adam_kernel");
}

int tt_fno_adam_device(int64_t n, float* params, float* grads, float* m, float* v, const float* lr, float beta1,
                       float beta2, float eps, int64_t* step, void* stream)
{
    if (n <= 0 || !params || !grads || !m || !v || !lr || !step) return tt::invalid("tt_fno_adam_device: bad arguments");
    cudaStream_t st = tt::as_stream(stream);
    fno_step_inc_kernel<<<1, 1, 0, st>>>(reinterpret_cast<long long*>(step));
    TT_TRY(tt::launch_status("fno_step_inc_kernel"));
    fno_adam_dev_kernel<<<grid_for(n / 256 + 1, 4), 256, 0, st>>>(n, params, grads, m, v, lr, beta1, beta2, eps,
                                                                 reinterpret_cast<const long long*>(step));
    return tt::launch_status("fno_adam_dev_kernel");
}

int tt_fno_error_flag(const void* ws, int* host_flag)
{
    if (!ws || !host_flag) return tt::invalid("tt_fno_error_flag: NULL pointer");
    return tt::cuda_status(cudaMemcpy(host_flag, ws, sizeof(int), cudaMemcpyDeviceToHost), "tt_fno_error_flag");
}

int tt_fno_pack(int64_t rows, int k, const float* src, void* dst, void* stream)
{
    if (rows <= 0 || rows % 8 || k <= 0 || k % 8 || !src || !dst) return tt::invalid("tt_fno_pack: bad arguments");
    fno_pack_kernel<<<grid_for(rows * k / 256 + 1, 4), 256, 0, tt::as_stream(stream)>>>(rows, k, src, (bf16*)dst);
    return tt::launch_status("fno_pack_kernel");
}

int tt_fno_rowdft(int S, int64_t rows, const void* in, const void* mat_packed, float* out, void* ws, void* stream)
{
    if ((S != 128 && S != 256) || rows <= 0 || rows % 128 || !in || !mat_packed || !out || !ws)
        return tt::invalid("tt_fno_rowdft: bad arguments");
    cudaStream_t st = tt::as_stream(stream);
    int* err = static_cast<int*>(ws);
    return S == 128 ? launch_rowdft<128>((const bf16*)in, rows, mat_packed, out, err, st)
                    : launch_rowdft<256>((const bf16*)in, rows, mat_packed, out, err, st);
}

int tt_fno_rowdft_timeout_test(int S, int64_t rows, const void* in, const void* mat_packed, float* out, void* ws,
                               int64_t wait_cycles, void* stream)
{
    if ((S != 128 && S != 256) || rows <= 0 || rows % 128 || !in || !mat_packed || !out || !ws)
        return tt::invalid("tt_fno_rowdft_timeout_test: bad arguments");
    if (wait_cycles < 1000 || wait_cycles > tt::umma::kWaitCycles)
        return tt::invalid("tt_fno_rowdft_timeout_test: wait_cycles must be in [1000, 2e9]");
    cudaStream_t st = tt::as_stream(stream);
    int* err = static_cast<int*>(ws);
    return S == 128 ? launch_rowdft<128>((const bf16*)in, rows, mat_packed, out, err, st, wait_cycles, 1)
                    : launch_rowdft<256>((const bf16*)in, rows, mat_packed, out, err, st, wait_cycles, 1);
}

int tt_fno_mix(int S, int B, int mode, const void* in, const void* w_packed, const void* a_packed, const float* sp,
               const float* bias, const void* zprev, void* out0, void* out1, void* ws, void* stream)
{
    if ((S != 128 && S != 256) || B < 1 || (mode != 0 && mode != 1) || !in || !w_packed || !a_packed || !sp || !ws)
        return tt::invalid("tt_fno_mix: bad arguments");
    if (mode == 0 && !out1) return tt::invalid("tt_fno_mix: forward needs out1");
    if (mode == 1 && !out0) return tt::invalid("tt_fno_mix: backward needs out0");
    cudaStream_t st = tt::as_stream(stream);
    int* err = static_cast<int*>(ws);
    const bf16* x = (const bf16*)in;
    const bf16* zp = (const bf16*)zprev;
    bf16* o0 = (bf16*)out0;
    bf16* o1 = (bf16*)out1;
    if (S == 128)
        return mode == 0 ? launch_mix<128, 0>(B, x, w_packed, a_packed, sp, bias, zp, o0, o1, err, st)
                         : launch_mix<128, 1>(B, x, w_packed, a_packed, sp, bias, zp, o0, o1, err, st);
    return mode == 0 ? launch_mix<256, 0>(B, x, w_packed, a_packed, sp, bias, zp, o0, o1, err, st)
                     : launch_mix<256, 1>(B, x, w_packed, a_packed, sp, bias, zp, o0, o1, err, st);
}

int tt_fno_wgrad(int S, int B, const void* dz, const void* v, float* dW, float* db, void* ws, void* stream)
{
    if ((S != 128 && S != 256) || B < 1 || !dz || !v || !dW || !db || !ws)
        return tt::invalid("tt_fno_wgrad: bad arguments");
    cudaStream_t st = tt::as_stream(stream);
    int* err = static_cast<int*>(ws);
    return S == 128 ? launch_wgrad<128>(B, (const bf16*)dz, (const bf16*)v, dW, db, err, st)
                    : launch_wgrad<256>(B, (const bf16*)dz, (const bf16*)v, dW, db, err, st);
}

}  // extern "C"
