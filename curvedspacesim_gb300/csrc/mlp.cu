// Learned distance screen: a 14 -> 64 -> 64 -> 64 -> 1 MLP with GELU that predicts the geodesic excess of a
// candidate pair, (d - |chord|) / sigma, from local features.  No reference counterpart: it decides which
// candidate pairs the exact propagation may skip (pairs predicted beyond sigma + margin); the exact solver still
// produces every distance that is used.
//
// Kernels:
//   * screen_features  - 14 rotation-invariant features per (source, target) pair, BF16, padded to K = 16
//   * mlp_infer_tc     - inference on the 5th-generation tensor cores: tcgen05.mma (kind::f16, BF16 in, FP32
//                        accumulate) with operands in shared memory and the 128 x 64 accumulator in tensor memory,
//                        read back with tcgen05.ld; bias + GELU epilogues in registers; the 64 -> 1 head on CUDA cores
//   * mlp_train_fwd_bwd- FP32 CUDA-core forward + backward of a mini-batch (BF16-rounded weights, like inference),
//                        weight gradients as per-block reductions in shared memory, then one atomicAdd per weight
//   * mlp_adam         - Adam update of the FP32 master weights and refresh of the BF16 copies
// Every wait on an mbarrier is bounded; on timeout the kernel records an error flag, frees its tensor memory and
// returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "cssg_internal.cuh"

namespace {

constexpr int NIN = 16;   // 14 features + 2 zero pads (K must be a multiple of 16 for kind::f16)
constexpr int NH = 64;
constexpr int TILE_M = 128;

// parameter block layout (FP32 master copy)
constexpr int OFF_W1 = 0;                     // [64][16]
constexpr int OFF_B1 = OFF_W1 + NH * NIN;     // [64]
constexpr int OFF_W2 = OFF_B1 + NH;           // [64][64]
constexpr int OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH;           // [64][64]
constexpr int OFF_B3 = OFF_W3 + NH * NH;
constexpr int OFF_W4 = OFF_B3 + NH;           // [64]
constexpr int OFF_B4 = OFF_W4 + NH;           // [1]
constexpr int NPARAM = OFF_B4 + 1;

__device__ __forceinline__ float gelu(float x)
{
    // tanh form of GELU
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    float u = k0 * (x + k1 * x * x * x);
    return 0.5f * x * (1.0f + tanhf(u));
}

__device__ __forceinline__ float gelu_grad(float x)
{
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    float x2 = x * x;
    float u = k0 * (x + k1 * x2 * x);
    float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * (1.0f + 3.0f * k1 * x2);
}

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16(x)); }

// GELU for the inference epilogue: the same tanh form, with tanh(u) = 1 - 2 / (exp(2u) + 1) from the fast exponential
// and division intrinsics (absolute error ~1e-7, far below the BF16 rounding of the activations that follows;
// exp(2u) = inf gives tanh = 1, exp(2u) = 0 gives -1)
__device__ __forceinline__ float gelu_fast(float x)
{
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    const float u = k0 * (x + k1 * x * x * x);
    const float t = 1.0f - __fdividef(2.0f, __expf(2.0f * u) + 1.0f);
    return 0.5f * x * (1.0f + t);
}

// eight BF16 values as one 16-byte word (k-contiguous run of a core matrix row)
__device__ __forceinline__ uint4 pack8_bf16(const float* v)
{
    uint4 w;
    uint32_t* p = reinterpret_cast<uint32_t*>(&w);
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        p[i] = *reinterpret_cast<const uint32_t*>(&b);
    }
    return w;
}

// ---- features ------------------------------------------------------------------------------------------------
// In the frame of the source face with u = in-plane chord direction and w = n_i x u:
//   rho/s, c.n_i/s, n_j.u, n_j.w, n_j.n_i, |c|/s, H_i s, K_i s^2, H_j s, K_j s^2, c.n_j/s, e_i/s, e_j/s, |c|^2/s^2
__global__ void screen_features(const SysDesc* __restrict__ sys, const int* __restrict__ sysOf, int nPairs,
                                const int* __restrict__ nPairsDev, const int* __restrict__ pi,
                                const int* __restrict__ pj, const int* __restrict__ face,
                                const double* __restrict__ pos, __nv_bfloat16* __restrict__ X,
                                float* __restrict__ chordOverSigma)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (nPairsDev) nPairs = min(nPairs, *nPairsDev);
    if (p >= nPairs) return;
    int i = pi[p], j = pj[p];
    const SysDesc& D = sys[sysOf ? sysOf[i] : 0];
    const DevMesh& M = D.mesh;
    double s = D.sigma;
    double c[3];
    for (int q = 0; q < 3; ++q) c[q] = pos[3 * j + q] - pos[3 * i + q];
    int fi = face[i], fj = face[j];
    const double* ni = &M.N[3 * fi];
    const double* nj = &M.N[3 * fj];
    double cn = c[0] * ni[0] + c[1] * ni[1] + c[2] * ni[2];
    double ip[3] = {c[0] - cn * ni[0], c[1] - cn * ni[1], c[2] - cn * ni[2]};
    double rho = sqrt(ip[0] * ip[0] + ip[1] * ip[1] + ip[2] * ip[2]);
    double u[3] = {1, 0, 0};
    if (rho > 0)
        for (int q = 0; q < 3; ++q) u[q] = ip[q] / rho;
    double w[3] = {ni[1] * u[2] - ni[2] * u[1], ni[2] * u[0] - ni[0] * u[2], ni[0] * u[1] - ni[1] * u[0]};
    double clen = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    float f[NIN];
    f[0] = (float)(rho / s);
    f[1] = (float)(cn / s);
    f[2] = (float)(nj[0] * u[0] + nj[1] * u[1] + nj[2] * u[2]);
    f[3] = (float)(nj[0] * w[0] + nj[1] * w[1] + nj[2] * w[2]);
    f[4] = (float)(nj[0] * ni[0] + nj[1] * ni[1] + nj[2] * ni[2]);
    f[5] = (float)(clen / s);
    f[6] = (float)(M.fcurv[3 * fi] * s);
    f[7] = (float)(M.fcurv[3 * fi + 1] * s * s);
    f[8] = (float)(M.fcurv[3 * fj] * s);
    f[9] = (float)(M.fcurv[3 * fj + 1] * s * s);
    f[10] = (float)((c[0] * nj[0] + c[1] * nj[1] + c[2] * nj[2]) / s);
    f[11] = (float)(M.fcurv[3 * fi + 2] / s);
    f[12] = (float)(M.fcurv[3 * fj + 2] / s);
    f[13] = (float)(clen * clen / (s * s));
    f[14] = 0.f;
    f[15] = 0.f;
    for (int q = 0; q < NIN; ++q) X[(size_t)p * NIN + q] = __float2bfloat16(f[q]);
    if (chordOverSigma) chordOverSigma[p] = (float)(clen / s);
}

// ---- tcgen05 inference ------------------------------------------------------------------------------------------
// Shared-memory operands in the canonical no-swizzle K-major layout: 8-row x 16-byte core matrices stored as
// 128 contiguous bytes; element (r, k) of a tile with K columns sits at
//   (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2      bytes
// so the leading (K-direction) byte offset between core matrices is 128 and the stride (row-direction) offset is
// 16 * K.  A K = 16 slice starting at column 16 q begins 256 q bytes into the tile.
__device__ __forceinline__ uint32_t core_off(int r, int k, int K)
{
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                 // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, M = 128, N = 64
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ uint32_t cvta_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// bounded wait on an mbarrier phase; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float* v)
{
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,"
        "%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,"
        "%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]),
          "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]),
          "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]),
          "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
          "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    for (int q = 0; q < 64; ++q) v[q] = __uint_as_float(r[q]);
}

struct __align__(128) InferSmem {
    __nv_bfloat16 A[TILE_M * NH];   // activations of the tile (K = 16 layout for layer 1, K = 64 after)
    __nv_bfloat16 W1[NH * NIN];     // B operands: [N = 64 rows][K] in the same core-matrix layout
    __nv_bfloat16 W2[NH * NH];
    __nv_bfloat16 W3[NH * NH];
    float b1[NH], b2[NH], b3[NH], w4[NH];
    float b4;
    uint64_t mbar;
    uint32_t tmem;
};

// one CTA of 128 threads: thread t owns row t of each 128-pair tile (TMEM lane t)
__global__ void __launch_bounds__(128) mlp_infer_tc(const __nv_bfloat16* __restrict__ X, int n,
                                                   const int* __restrict__ nDev, const float* __restrict__ params,
                                                   float* __restrict__ yOut, int* __restrict__ errFlag)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    if (nDev) n = min(n, *nDev);
    InferSmem& S = *reinterpret_cast<InferSmem*>(smraw);
    const int t = threadIdx.x, warp = t >> 5;
    // stage weights (BF16, core-matrix layout) and epilogue constants
    for (int q = t; q < NH * NIN; q += 128) {
        int nrow = q / NIN, k = q % NIN;
        S.W1[core_off(nrow, k, NIN) / 2] = __float2bfloat16(params[OFF_W1 + q]);
    }
    for (int q = t; q < NH * NH; q += 128) {
        int nrow = q / NH, k = q % NH;
        S.W2[core_off(nrow, k, NH) / 2] = __float2bfloat16(params[OFF_W2 + q]);
        S.W3[core_off(nrow, k, NH) / 2] = __float2bfloat16(params[OFF_W3 + q]);
    }
    if (t < NH) {
        S.b1[t] = params[OFF_B1 + t];
        S.b2[t] = params[OFF_B2 + t];
        S.b3[t] = params[OFF_B3 + t];
        S.w4[t] = params[OFF_W4 + t];
    }
    if (t == 0) {
        S.b4 = params[OFF_B4];
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cvta_smem(&S.mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(cvta_smem(&S.tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = S.tmem;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
    const uint32_t mbar = cvta_smem(&S.mbar);
    const uint32_t sA = cvta_smem(S.A), sW1 = cvta_smem(S.W1), sW2 = cvta_smem(S.W2), sW3 = cvta_smem(S.W3);
    uint32_t phase = 0;
    bool ok = true;
    float h[NH];
    for (int tile = blockIdx.x; tile * TILE_M < n && ok; tile += gridDim.x) {
        const int row = tile * TILE_M + t;
        // layer 1 operand: this thread's 16 features (32 bytes of its row: two 16-byte words, each the k-contiguous
        // run of one core matrix row)
        {
            uint4 x0 = make_uint4(0, 0, 0, 0), x1 = x0;
            if (row < n) {
                const uint4* xr = reinterpret_cast<const uint4*>(X + (size_t)row * NIN);
                x0 = __ldg(xr);
                x1 = __ldg(xr + 1);
            }
            *reinterpret_cast<uint4*>(reinterpret_cast<char*>(S.A) + core_off(t, 0, NIN)) = x0;
            *reinterpret_cast<uint4*>(reinterpret_cast<char*>(S.A) + core_off(t, 8, NIN)) = x1;
        }
        for (int layer = 0; layer < 3 && ok; ++layer) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (t == 0) {
                if (layer == 0) {
                    mma_bf16(tmem, smem_desc(sA, 128, 16 * NIN), smem_desc(sW1, 128, 16 * NIN), 0);
                } else {
                    uint32_t sW = layer == 1 ? sW2 : sW3;
                    for (int q = 0; q < NH / 16; ++q)
                        mma_bf16(tmem, smem_desc(sA + 256 * q, 128, 16 * NH), smem_desc(sW + 256 * q, 128, 16 * NH),
                                 q > 0 ? 1u : 0u);
                }
                mma_commit(mbar);
            }
            const bool arrived = mbar_wait(mbar, phase);
            if (!__syncthreads_and(arrived)) {  // uniform decision before any warp-collective tensor-memory load
                ok = false;
                if (errFlag && t == 0) atomicExch(errFlag, 1);
                break;
            }
            phase ^= 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            tmem_ld64(taddr, h);
            const float* b = layer == 0 ? S.b1 : (layer == 1 ? S.b2 : S.b3);
            for (int q = 0; q < NH; ++q) h[q] = gelu_fast(h[q] + b[q]);
            if (layer < 2)
                for (int g = 0; g < NH / 8; ++g)
                    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(S.A) + core_off(t, 8 * g, NH)) =
                        pack8_bf16(&h[8 * g]);
        }
        if (ok && row < n) {
            float y = S.b4;
            for (int q = 0; q < NH; ++q) y += h[q] * S.w4[q];
            yOut[row] = y;
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        ok = __syncthreads_and(ok);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

// ---- training: FP32 forward + backward (BF16-rounded weights, like inference) -----------------------------------
constexpr int TB = 128;  // samples per block

__global__ void __launch_bounds__(TB) mlp_train_fwd_bwd(const __nv_bfloat16* __restrict__ X, const float* __restrict__ y,
                                                         int n, const float* __restrict__ params,
                                                         float* __restrict__ grad, float* __restrict__ loss)
{
    extern __shared__ float sm[];
    float* W = sm;                         // NPARAM (BF16-rounded)
    float* Z1 = W + NPARAM + 3;            // [TB][64] pre-activations
    float* Z2 = Z1 + TB * NH;
    float* Z3 = Z2 + TB * NH;
    float* G = Z3 + TB * NH;               // [TB][64] scratch for back-propagated gradients
    float* XS = G + TB * NH;               // [TB][16]
    const int t = threadIdx.x;
    for (int q = t; q < NPARAM; q += TB) W[q] = (q >= OFF_B1 && q < OFF_W2) || (q >= OFF_B2 && q < OFF_W3) ||
                                                        (q >= OFF_B3)
                                                    ? params[q]
                                                    : bf16r(params[q]);
    __syncthreads();
    const int row = blockIdx.x * TB + t;
    const bool valid = row < n;
    float x[NIN];
    for (int k = 0; k < NIN; ++k) {
        x[k] = valid ? __bfloat162float(X[(size_t)row * NIN + k]) : 0.f;
        XS[t * NIN + k] = x[k];
    }
    float h1[NH], h2[NH];
    for (int o = 0; o < NH; ++o) {
        float z = W[OFF_B1 + o];
        for (int k = 0; k < NIN; ++k) z += W[OFF_W1 + o * NIN + k] * x[k];
        Z1[t * NH + o] = z;
        h1[o] = bf16r(gelu(z));  // inference feeds BF16 activations to the next layer
    }
    for (int o = 0; o < NH; ++o) {
        float z = W[OFF_B2 + o];
        for (int k = 0; k < NH; ++k) z += W[OFF_W2 + o * NH + k] * h1[k];
        Z2[t * NH + o] = z;
        h2[o] = bf16r(gelu(z));
    }
    float out = W[OFF_B4];
    for (int o = 0; o < NH; ++o) {
        float z = W[OFF_B3 + o];
        for (int k = 0; k < NH; ++k) z += W[OFF_W3 + o * NH + k] * h2[k];
        Z3[t * NH + o] = z;
        out += gelu(z) * W[OFF_W4 + o];
    }
    float dy = valid ? (out - y[row]) : 0.f;  // d(0.5 (out - y)^2) / d out
    // per-sample deltas
    float d3[NH];
    for (int o = 0; o < NH; ++o) d3[o] = dy * W[OFF_W4 + o] * gelu_grad(Z3[t * NH + o]);
    for (int o = 0; o < NH; ++o) G[t * NH + o] = d3[o];
    __syncthreads();
    // head and layer-3 weight gradients: dW3[o][k] = sum_t d3[t][o] h2[t][k]; h2 recomputed from Z2
    // (each thread owns 32 of the 4096 + 64 + 64 + 1 entries)
    for (int e = t; e < NH * NH; e += TB) {
        int o = e / NH, k = e % NH;
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH + o] * bf16r(gelu(Z2[s * NH + k]));
        atomicAdd(&grad[OFF_W3 + e], acc);
    }
    if (t < NH) {
        float accb = 0;
        for (int s = 0; s < TB; ++s) {
            accb += G[s * NH + t];
        }
        atomicAdd(&grad[OFF_B3 + t], accb);
    }
    // head: dW4[o] = sum dy gelu(Z3), dB4 = sum dy
    __syncthreads();
    G[t * NH + 0] = dy;  // reuse column 0 for dy (d3 already consumed)
    __syncthreads();
    if (t < NH) {
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH] * gelu(Z3[s * NH + t]);
        atomicAdd(&grad[OFF_W4 + t], acc);
    }
    if (t == 0) {
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH];
        atomicAdd(&grad[OFF_B4], acc);
    }
    __syncthreads();
    // back to layer 2
    float d2[NH];
    for (int k = 0; k < NH; ++k) {
        float acc = 0;
        for (int o = 0; o < NH; ++o) acc += d3[o] * W[OFF_W3 + o * NH + k];
        d2[k] = acc * gelu_grad(Z2[t * NH + k]);
    }
    for (int o = 0; o < NH; ++o) G[t * NH + o] = d2[o];
    __syncthreads();
    for (int e = t; e < NH * NH; e += TB) {
        int o = e / NH, k = e % NH;
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH + o] * bf16r(gelu(Z1[s * NH + k]));
        atomicAdd(&grad[OFF_W2 + e], acc);
    }
    if (t < NH) {
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH + t];
        atomicAdd(&grad[OFF_B2 + t], acc);
    }
    __syncthreads();
    float d1[NH];
    for (int k = 0; k < NH; ++k) {
        float acc = 0;
        for (int o = 0; o < NH; ++o) acc += d2[o] * W[OFF_W2 + o * NH + k];
        d1[k] = acc * gelu_grad(Z1[t * NH + k]);
    }
    for (int o = 0; o < NH; ++o) G[t * NH + o] = d1[o];
    __syncthreads();
    for (int e = t; e < NH * NIN; e += TB) {
        int o = e / NIN, k = e % NIN;
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH + o] * XS[s * NIN + k];
        atomicAdd(&grad[OFF_W1 + e], acc);
    }
    if (t < NH) {
        float acc = 0;
        for (int s = 0; s < TB; ++s) acc += G[s * NH + t];
        atomicAdd(&grad[OFF_B1 + t], acc);
    }
    if (loss) {
        float l = 0.5f * dy * dy;
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((t & 31) == 0) atomicAdd(loss, l);
    }
}

__global__ void mlp_adam(float* __restrict__ params, const float* __restrict__ grad, float* __restrict__ m,
                         float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float scale, int step)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NPARAM) return;
    float g = grad[q] * scale;
    float mq = b1 * m[q] + (1 - b1) * g;
    float vq = b2 * v[q] + (1 - b2) * g * g;
    m[q] = mq;
    v[q] = vq;
    float mh = mq / (1 - powf(b1, (float)step));
    float vh = vq / (1 - powf(b2, (float)step));
    params[q] -= lr * mh / (sqrtf(vh) + eps);
    (void)n;
}

size_t train_smem() { return sizeof(float) * (NPARAM + 3 + 4 * TB * NH + TB * NIN); }

// skip[p] = 1 when the predicted distance |chord| + sigma yhat exceeds sigma (1 + margin); nothing is skipped while
// *disable is set (the audit found a dropped pair)
__global__ void screen_decide(int n, const int* __restrict__ nDev, const float* __restrict__ chord,
                              const float* __restrict__ yhat, double margin, unsigned char* __restrict__ skip,
                              const int* __restrict__ disable)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (nDev) n = min(n, *nDev);
    if (p >= n) return;
    const bool off = disable && *disable;
    skip[p] = (!off && (double)chord[p] + (double)yhat[p] > 1.0 + margin) ? 1 : 0;
}

size_t infer_smem() { return sizeof(InferSmem) + 128; }

// resident CTAs per SM for the persistent grid, from the kernel's registers and the SM's shared memory (each CTA
// also holds 64 of the 512 tensor-memory columns, so at most 8)
int infer_ctas_per_sm(int dev)
{
    cudaFuncAttributes fa;
    int smemSM = 0, regsSM = 0;
    if (cudaFuncGetAttributes(&fa, mlp_infer_tc) != cudaSuccess ||
        cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess)
        return 4;
    const int byRegs = regsSM / std::max(1, fa.numRegs * 128);
    const int bySmem = (int)(smemSM / (infer_smem() + fa.sharedSizeBytes + 1024));  // 1 KB reserved per CTA
    return std::max(1, std::min(std::min(byRegs, bySmem), 8));
}

// devices on which mlp_infer_tc's dynamic shared-memory limit has been raised
std::atomic<unsigned long long> g_inferSmemSet{0};

}  // namespace

void cssg_launch_screen(const SysDesc* sys, const int* sysOf, int maxPairs, const int* nPairsDev, const int* pi,
                        const int* pj, const int* face, const double* pos, void* X, float* chord, const float* params,
                        float* yhat, unsigned char* skip, double margin, int* errFlag, int sms, cudaStream_t s,
                        const int* disable)
{
    if (maxPairs <= 0) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cssg_raise_smem_once(g_inferSmemSet, mlp_infer_tc, (int)infer_smem(), dev);
    cudaFuncSetAttribute(mlp_infer_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    screen_features<<<(maxPairs + 127) / 128, 128, 0, s>>>(sys, sysOf, maxPairs, nPairsDev, pi, pj, face, pos,
                                                            (__nv_bfloat16*)X, chord);
    int tiles = (maxPairs + TILE_M - 1) / TILE_M;
    mlp_infer_tc<<<std::min(tiles, sms * infer_ctas_per_sm(dev)), 128, infer_smem(), s>>>(
        (const __nv_bfloat16*)X, maxPairs, nPairsDev, params, yhat, errFlag);
    screen_decide<<<(maxPairs + 255) / 256, 256, 0, s>>>(maxPairs, nPairsDev, chord, yhat, margin, skip, disable);
}

// ======================================================================================================================
// C ABI
// ======================================================================================================================
extern "C" int cssg_mlp_param_count(void) { return NPARAM; }

extern "C" int cssg_screen_features(cssg_ctx* ctx, const cssg_mesh* mesh, double sigma, int nPairs, const int* pi,
                                    const int* pj, const int* face, const double* pos, void* X_bf16,
                                    float* chord_over_sigma)
{
    if (!ctx || !mesh || nPairs < 0 || (nPairs > 0 && (!pi || !pj || !face || !pos || !X_bf16))) {
        cssg_set_error("cssg_screen_features: bad arguments");
        return CSSG_ERR_ARG;
    }
    if (nPairs == 0) return CSSG_OK;
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    SysDesc hd;
    memset(&hd, 0, sizeof(hd));
    hd.mesh = mesh->d;
    hd.sigma = sigma;
    SysDesc* dsys = nullptr;
    CSSG_CUDA(cudaMallocAsync((void**)&dsys, sizeof(SysDesc), ctx->stream));
    CSSG_CUDA(cudaMemcpyAsync(dsys, &hd, sizeof(SysDesc), cudaMemcpyHostToDevice, ctx->stream));
    screen_features<<<(nPairs + 127) / 128, 128, 0, ctx->stream>>>(dsys, nullptr, nPairs, nullptr, pi, pj, face, pos,
                                                                   (__nv_bfloat16*)X_bf16, chord_over_sigma);
    CSSG_CUDA(cudaGetLastError());
    CSSG_CUDA(cudaFreeAsync(dsys, ctx->stream));
    return CSSG_OK;
}

extern "C" int cssg_mlp_infer(cssg_ctx* ctx, const void* X_bf16, int n, const float* params, float* y, int* err_flag)
{
    if (!ctx || n < 0 || (n > 0 && (!X_bf16 || !params || !y))) {
        cssg_set_error("cssg_mlp_infer: bad arguments");
        return CSSG_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(X_bf16) % 16 != 0) {  // rows are read as 16-byte words
        cssg_set_error("cssg_mlp_infer: X must be 16-byte aligned");
        return CSSG_ERR_ARG;
    }
    if (n == 0) return CSSG_OK;
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    size_t smem = infer_smem();
    CSSG_CUDA(cssg_raise_smem_once(g_inferSmemSet, mlp_infer_tc, (int)smem, ctx->device));
    CSSG_CUDA(cudaFuncSetAttribute(mlp_infer_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    int tiles = (n + TILE_M - 1) / TILE_M;
    int blocks = std::min(tiles, sms * infer_ctas_per_sm(ctx->device));
    mlp_infer_tc<<<blocks, 128, smem, ctx->stream>>>((const __nv_bfloat16*)X_bf16, n, nullptr, params, y, err_flag);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

// gradient of 0.5 * sum (f(x) - y)^2 over the n samples, accumulated into grad[NPARAM] (zeroed first here);
// loss (nullable) receives the same sum
extern "C" int cssg_mlp_grad(cssg_ctx* ctx, const void* X_bf16, const float* y, int n, const float* params, float* grad,
                             float* loss)
{
    if (!ctx || n <= 0 || !X_bf16 || !y || !params || !grad) {
        cssg_set_error("cssg_mlp_grad: bad arguments");
        return CSSG_ERR_ARG;
    }
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    size_t smem = train_smem();
    static std::atomic<unsigned long long> configured{0};
    CSSG_CUDA(cssg_raise_smem_once(configured, mlp_train_fwd_bwd, (int)smem, ctx->device));
    CSSG_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * NPARAM, ctx->stream));
    if (loss) CSSG_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), ctx->stream));
    mlp_train_fwd_bwd<<<(n + TB - 1) / TB, TB, smem, ctx->stream>>>((const __nv_bfloat16*)X_bf16, y, n, params, grad,
                                                                    loss);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

// one Adam step on the mean-squared loss of the batch: state = m[NPARAM], v[NPARAM] (zero-initialised by caller)
extern "C" int cssg_mlp_adam(cssg_ctx* ctx, float* params, const float* grad, float* m, float* v, int batch, float lr,
                             int step)
{
    if (!ctx || !params || !grad || !m || !v || batch <= 0 || step <= 0) {
        cssg_set_error("cssg_mlp_adam: bad arguments");
        return CSSG_ERR_ARG;
    }
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    mlp_adam<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(params, grad, m, v, NPARAM, lr, 0.9f, 0.999f, 1e-8f,
                                                            1.0f / batch, step);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}
