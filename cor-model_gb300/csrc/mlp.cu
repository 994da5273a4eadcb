// mlp.cu -- the learned rigidity window's network (include/cor_window.h): a
// BF16 MLP whose every matrix product runs on the 5th-generation tensor cores.
//
// One GEMM kernel serves the forward and backward passes:
//   C[M][N] = A[M][K] . B[N][K]^T      (A, B BF16 and K-major, C FP32 in TMEM)
// with M a multiple of 128 (one 128-row tile per CTA), N a multiple of 16 up
// to 256 (the whole N in one tcgen05.mma), K a multiple of 64 (one 64-deep
// shared-memory stage = four K=16 MMAs).  Operand tiles sit in shared memory
// in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core
// matrix; LBO = 128 B between core matrices along K, SBO = 1024 B between
// 8-row groups).  One thread issues the MMAs and commits them to an mbarrier;
// the four warps then read the accumulator out of TMEM (warp w owns lanes
// 32w..32w+31, i.e. rows) and apply the epilogue of the pass:
//   FWD_SILU  z = acc + b -> Z (FP32), H = silu(z) and H^T (BF16)
//   LINEAR    y = acc (+ b) -> C (FP32)
//   BWD_SILU  dz = acc * silu'(Z) -> dZ and dZ^T (BF16), db += column sums
// The transposed copies make every backward product K-major again:
//   dH = dZ . W       uses W^T [in][out]   as B
//   dW = dZ^T . X^T   uses dZ^T [out][batch] as A and X^T [in][batch] as B.
// Waits on the mbarrier are bounded (about 2 s of SM clock); a wait that
// runs out sets the error word, skips the rest and still frees the TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cor_trace.h"
#include "cor_window.h"

namespace mlp {

typedef __nv_bfloat16 bf16;

constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr int kThreads = 128;
constexpr int kInPad = 64;      // 19 input features, zero-padded to one K stage
constexpr int kOutPad = 16;     // 2 outputs, padded to the smallest N
constexpr int kH = COR_MLP_HIDDEN;
constexpr int kLayers = COR_MLP_LAYERS + 1;   // 5 weight matrices
constexpr size_t kSmemBytes = 96 * 1024;     // also caps residency at 2 CTAs/SM (2 x 256 TMEM columns)
constexpr long long kWaitCycles = 4000000000ll;

enum Mode { FWD_SILU = 0, LINEAR = 1, BWD_SILU = 2 };

struct GemmArgs {
    const bf16* A;
    int lda;
    const bf16* B;
    int ldb;
    int M, N, K;
    int mode;
    const float* bias;  // LINEAR / FWD_SILU, may be null for LINEAR
    float* C;           // FP32 out (Z for FWD_SILU, C for LINEAR)
    int ldc;
    bf16* H;            // BF16 out, row-major (H or dZ)
    int ldh;
    bf16* Ht;           // BF16 out, transposed [N][M]
    int ldht;
    const float* Zin;   // BWD_SILU: the pre-activation of the layer
    int ldz;
    float* dbias;       // BWD_SILU: column sums accumulate here
    int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (tcgen05 "matrix descriptor"): start
// address, leading and stride byte offsets in 16-byte units, version 1,
// no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > kWaitCycles) return false;
    }
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.f / (1.f + expf(-z));
    return s * (1.f + z * (1.f - s));
}

// Copies rows [r0, r0+rows) x K columns [k0, k0+64) of a row-major BF16 matrix
// into the core-matrix layout at `dst`.
__device__ __forceinline__ void load_tile(uint8_t* dst, const bf16* src, int ld, int r0, int rows, int k0) {
    for (int v = threadIdx.x; v < rows * 8; v += kThreads) {
        const int r = v >> 3, c = v & 7;
        const uint4 x = *reinterpret_cast<const uint4*>(src + (size_t)(r0 + r) * ld + k0 + c * 8);
        *reinterpret_cast<uint4*>(dst + (r >> 3) * 1024 + c * 128 + (r & 7) * 16) = x;
    }
}

__global__ void __launch_bounds__(kThreads) gemm_kernel(const GemmArgs g) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sa = smem;                       // 128 x 64 BF16 = 16 KB
    uint8_t* sb = smem + 16 * 1024;           // N x 64 BF16 <= 32 KB
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 48 * 1024);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 48 * 1024 + 64);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM;
    uint32_t ncols = 32;
    while ((int)ncols < g.N) ncols <<= 1;

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = instr_desc(kBM, g.N);

    bool ok = true;
    const int kb_n = g.K / kBK;
    for (int kb = 0; kb < kb_n && ok; kb++) {
        load_tile(sa, g.A, g.lda, m0, kBM, kb * kBK);
        load_tile(sb, g.B, g.ldb, 0, g.N, kb * kBK);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
            for (int s = 0; s < kBK / 16; s++) {
                const uint64_t ad = smem_desc(a0 + s * 256, 128, 1024);
                const uint64_t bd = smem_desc(b0 + s * 256, 128, 1024);
                const uint32_t acc = (kb > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(bar))
                         : "memory");
        }
        ok = mbar_wait(bar, (uint32_t)(kb & 1));
        if (!ok) atomicExch(g.err, 1);
        // the MMAs of this stage are complete: the tiles may be overwritten
        __syncthreads();
        ok = __syncthreads_and(ok);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (ok) {
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < g.N; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float v[16];
#pragma unroll
            for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
            if (g.mode == FWD_SILU) {
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int c = c0 + i;
                    const float z = v[i] + g.bias[c];
                    g.C[(size_t)row * g.ldc + c] = z;
                    const bf16 h = __float2bfloat16(silu(z));
                    g.H[(size_t)row * g.ldh + c] = h;
                    g.Ht[(size_t)c * g.ldht + row] = h;
                }
            } else if (g.mode == LINEAR) {
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int c = c0 + i;
                    g.C[(size_t)row * g.ldc + c] = v[i] + (g.bias ? g.bias[c] : 0.f);
                }
            } else {
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int c = c0 + i;
                    const float d = v[i] * silu_grad(g.Zin[(size_t)row * g.ldz + c]);
                    const bf16 h = __float2bfloat16(d);
                    g.H[(size_t)row * g.ldh + c] = h;
                    g.Ht[(size_t)c * g.ldht + row] = h;
                    float s = d;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                    if (lane == 0) atomicAdd(g.dbias + c, s);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---- element-wise kernels -------------------------------------------------------
// features (n x 19 FP32) -> X0 (Bt x 64 BF16, zero-padded rows and columns)
// and X0^T (64 x Bt)
__global__ void input_kernel(const float* __restrict__ x, int n, int bt, bf16* __restrict__ x0,
                             bf16* __restrict__ x0t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bt * kInPad) return;
    const int r = i / kInPad, c = i % kInPad;
    const float v = (r < n && c < COR_MLP_IN) ? x[(size_t)r * COR_MLP_IN + c] : 0.f;
    const bf16 b = __float2bfloat16(v);
    x0[i] = b;
    x0t[(size_t)c * bt + r] = b;
}

// mean squared error over the n valid rows and COR_MLP_OUT outputs, its
// gradient dY (Bt x 64, zero outside), dY^T (16 x Bt) and db5
__global__ void loss_kernel(const float* __restrict__ y, const float* __restrict__ t, int n, int bt,
                            bf16* __restrict__ dy, bf16* __restrict__ dyt, float* __restrict__ db5,
                            float* __restrict__ loss) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= bt) return;
    const float scale = 2.f / (float)(n * COR_MLP_OUT);
    float l = 0.f;
    for (int c = 0; c < kInPad; c++) {
        float d = 0.f;
        if (r < n && c < COR_MLP_OUT) {
            const float e = y[(size_t)r * kOutPad + c] - t[(size_t)r * COR_MLP_OUT + c];
            l += e * e;
            d = scale * e;
            atomicAdd(db5 + c, d);
        }
        dy[(size_t)r * kInPad + c] = __float2bfloat16(d);
        if (c < kOutPad) dyt[(size_t)c * bt + r] = __float2bfloat16(d);
    }
    if (r < n) atomicAdd(loss, l / (float)(n * COR_MLP_OUT));
}

__global__ void copy_out_kernel(const float* __restrict__ y, int n, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * COR_MLP_OUT) return;
    out[i] = y[(size_t)(i / COR_MLP_OUT) * kOutPad + i % COR_MLP_OUT];
}

// One weight matrix or bias vector: FP32 master, moments, gradient source and
// the BF16 copies the GEMMs read.
struct ParamView {
    float* w;          // master [rows][cols]
    float* m;
    float* v;
    const float* g;    // gradient
    int g_transposed;  // gradient stored [cols][g_ld] (layer 5)
    int g_ld;
    int rows, cols;
    bf16* wb;          // [rows][wb_ld] zero-padded   (null for biases)
    int wb_ld;
    bf16* wt;          // [cols][wt_ld] zero-padded   (null for biases)
    int wt_ld;
    float* gout;       // packed gradient export (may be null)
    float decay;
};

__global__ void adamw_kernel(ParamView p, float lr, float b1c, float b2c, int update) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.rows * p.cols) return;
    const int r = i / p.cols, c = i % p.cols;
    const float g = p.g_transposed ? p.g[(size_t)c * p.g_ld + r] : p.g[(size_t)r * p.g_ld + c];
    if (p.gout) p.gout[i] = g;
    if (!update) return;
    const float m = 0.9f * p.m[i] + 0.1f * g;
    const float v = 0.999f * p.v[i] + 0.001f * g * g;
    p.m[i] = m;
    p.v[i] = v;
    float w = p.w[i];
    w -= lr * ((m / b1c) / (sqrtf(v / b2c) + 1e-8f) + p.decay * w);
    p.w[i] = w;
    if (p.wb) p.wb[(size_t)r * p.wb_ld + c] = __float2bfloat16(w);
    if (p.wt) p.wt[(size_t)c * p.wt_ld + r] = __float2bfloat16(w);
}

__global__ void cast_kernel(ParamView p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.rows * p.cols) return;
    const int r = i / p.cols, c = i % p.cols;
    if (p.wb) p.wb[(size_t)r * p.wb_ld + c] = __float2bfloat16(p.w[i]);
    if (p.wt) p.wt[(size_t)c * p.wt_ld + r] = __float2bfloat16(p.w[i]);
}

}  // namespace mlp

using namespace mlp;

struct cor_mlp {
    int device = 0;
    int max_bt = 0;
    char err[256] = {0};
    int step = 0;
    void* block = nullptr;      // one allocation holds every buffer
    float *w[kLayers], *b[kLayers], *mw[kLayers], *vw[kLayers], *mb[kLayers], *vb[kLayers];
    float *gw[kLayers], *gb[kLayers];
    bf16 *wb[kLayers], *wt[kLayers];
    bf16 *x0, *x0t, *h[COR_MLP_LAYERS], *ht[COR_MLP_LAYERS], *dz, *dzt, *dz2, *dz2t, *dy, *dyt;
    float *z[COR_MLP_LAYERS], *y;
    int* dev_err = nullptr;
};

static const int kIn[kLayers] = {COR_MLP_IN, kH, kH, kH, kH};
static const int kOut[kLayers] = {kH, kH, kH, kH, COR_MLP_OUT};
static const int kInP[kLayers] = {kInPad, kH, kH, kH, kH};
static const int kOutP[kLayers] = {kH, kH, kH, kH, kOutPad};

static int mfail(cor_mlp* m, int code, const char* fmt, ...) {
    if (m) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(m->err, sizeof m->err, fmt, ap);
        va_end(ap);
    }
    return code;
}

#define MTRY(m, call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return mfail((m), COR_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

static int gemm(cor_mlp* m, GemmArgs g, cudaStream_t s) {
    if (g.M % kBM || g.N % 16 || g.N < 16 || g.N > 256 || g.K % kBK || g.K <= 0 || g.lda % 8 || g.ldb % 8)
        return mfail(m, COR_ERR_INVALID, "gemm shape %d x %d x %d not supported", g.M, g.N, g.K);
    g.err = m->dev_err;
    gemm_kernel<<<g.M / kBM, kThreads, kSmemBytes, s>>>(g);
    MTRY(m, cudaGetLastError());
    return COR_OK;
}

static int forward(cor_mlp* m, const float* x, int n, int bt, cudaStream_t s) {
    const int th = 256;
    input_kernel<<<(bt * kInPad + th - 1) / th, th, 0, s>>>(x, n, bt, m->x0, m->x0t);
    MTRY(m, cudaGetLastError());
    const bf16* in = m->x0;
    int in_ld = kInPad;
    for (int l = 0; l < COR_MLP_LAYERS; l++) {
        GemmArgs g = {};
        g.A = in;
        g.lda = in_ld;
        g.B = m->wb[l];
        g.ldb = kInP[l];
        g.M = bt;
        g.N = kH;
        g.K = kInP[l];
        g.mode = FWD_SILU;
        g.bias = m->b[l];
        g.C = m->z[l];
        g.ldc = kH;
        g.H = m->h[l];
        g.ldh = kH;
        g.Ht = m->ht[l];
        g.ldht = bt;
        int rc = gemm(m, g, s);
        if (rc != COR_OK) return rc;
        in = m->h[l];
        in_ld = kH;
    }
    GemmArgs g = {};
    g.A = in;
    g.lda = kH;
    g.B = m->wb[4];
    g.ldb = kH;
    g.M = bt;
    g.N = kOutPad;
    g.K = kH;
    g.mode = LINEAR;
    g.bias = m->b[4];
    g.C = m->y;
    g.ldc = kOutPad;
    return gemm(m, g, s);
}

static int backward(cor_mlp* m, const float* t, int n, int bt, float* loss, cudaStream_t s) {
    for (int l = 0; l < kLayers; l++) MTRY(m, cudaMemsetAsync(m->gb[l], 0, sizeof(float) * kOut[l], s));
    MTRY(m, cudaMemsetAsync(loss, 0, sizeof(float), s));
    loss_kernel<<<(bt + 127) / 128, 128, 0, s>>>(m->y, t, n, bt, m->dy, m->dyt, m->gb[4], loss);
    MTRY(m, cudaGetLastError());
    int rc;
    {   // dW5^T [256][16] = H4^T . dY^T
        GemmArgs g = {};
        g.A = m->ht[3]; g.lda = bt; g.B = m->dyt; g.ldb = bt;
        g.M = kH; g.N = kOutPad; g.K = bt; g.mode = LINEAR; g.C = m->gw[4]; g.ldc = kOutPad;
        if ((rc = gemm(m, g, s)) != COR_OK) return rc;
    }
    // dZ4 = (dY . W5) * silu'(Z4); W5^T is [256][64] (zero beyond the 2 outputs)
    const bf16* up = m->dy;
    int up_ld = kInPad;
    int up_k = kInPad;
    bf16* dzb[2] = {m->dz, m->dz2};
    bf16* dztb[2] = {m->dzt, m->dz2t};
    for (int l = COR_MLP_LAYERS - 1; l >= 0; l--) {
        const int cur = l & 1;
        GemmArgs g = {};
        g.A = up; g.lda = up_ld; g.B = m->wt[l + 1]; g.ldb = up_k;
        g.M = bt; g.N = kH; g.K = up_k; g.mode = BWD_SILU;
        g.Zin = m->z[l]; g.ldz = kH; g.H = dzb[cur]; g.ldh = kH; g.Ht = dztb[cur]; g.ldht = bt;
        g.dbias = m->gb[l];
        if ((rc = gemm(m, g, s)) != COR_OK) return rc;
        // dW_l [256][in_pad] = dZ_l^T . X_{l-1}^T
        GemmArgs w = {};
        w.A = dztb[cur]; w.lda = bt; w.B = l == 0 ? m->x0t : m->ht[l - 1]; w.ldb = bt;
        w.M = kH; w.N = kInP[l]; w.K = bt; w.mode = LINEAR; w.C = m->gw[l]; w.ldc = kInP[l];
        if ((rc = gemm(m, w, s)) != COR_OK) return rc;
        up = dzb[cur];
        up_ld = kH;
        up_k = kH;
    }
    return COR_OK;
}

static ParamView view(cor_mlp* m, int l, bool bias, float* gout) {
    ParamView p = {};
    if (!bias) {
        p.w = m->w[l]; p.m = m->mw[l]; p.v = m->vw[l];
        p.g = m->gw[l];
        p.g_transposed = l == 4;
        p.g_ld = l == 4 ? kOutPad : kInP[l];
        p.rows = kOut[l]; p.cols = kIn[l];
        p.wb = m->wb[l]; p.wb_ld = kInP[l];
        p.wt = m->wt[l]; p.wt_ld = l == 4 ? kInPad : kOutP[l];
        p.decay = 1.f;
    } else {
        p.w = m->b[l]; p.m = m->mb[l]; p.v = m->vb[l];
        p.g = m->gb[l]; p.g_ld = 1;
        p.rows = kOut[l]; p.cols = 1;
        p.decay = 0.f;
    }
    p.gout = gout;
    return p;
}

// offsets of each tensor in the packed parameter layout
static void param_offsets(size_t* wo, size_t* bo) {
    size_t o = 0;
    for (int l = 0; l < kLayers; l++) {
        wo[l] = o;
        o += (size_t)kOut[l] * kIn[l];
        bo[l] = o;
        o += kOut[l];
    }
}

static int update(cor_mlp* m, float lr, float wd, float* grads, int do_update, cudaStream_t s) {
    size_t wo[kLayers], bo[kLayers];
    param_offsets(wo, bo);
    if (do_update) m->step++;
    const float b1c = 1.f - powf(0.9f, (float)(m->step > 0 ? m->step : 1));
    const float b2c = 1.f - powf(0.999f, (float)(m->step > 0 ? m->step : 1));
    for (int l = 0; l < kLayers; l++) {
        for (int bias = 0; bias < 2; bias++) {
            ParamView p = view(m, l, bias, grads ? grads + (bias ? bo[l] : wo[l]) : nullptr);
            if (!bias) p.decay = wd;
            const int n = p.rows * p.cols;
            adamw_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, lr, b1c, b2c, do_update);
            MTRY(m, cudaGetLastError());
        }
    }
    return COR_OK;
}

static int check_err(cor_mlp* m) {
    int e = 0;
    MTRY(m, cudaMemcpy(&e, m->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return mfail(m, COR_ERR_WATCHDOG, "a tensor-core wait ran out of time");
    return COR_OK;
}

extern "C" {

const char* cor_mlp_error(const cor_mlp* m) { return m ? m->err : "null network"; }

int cor_mlp_create(int device, int32_t max_batch, cor_mlp** out) {
    if (!out || max_batch < 1) return COR_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return COR_ERR_NODEV;
    }
    if (device < 0 || device >= ndev) return COR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return COR_ERR_CUDA;
    cor_mlp* m = new cor_mlp();
    m->device = device;
    m->max_bt = (max_batch + kBM - 1) / kBM * kBM;
    const size_t bt = (size_t)m->max_bt;
    // sizes in bytes, each rounded to 256
    size_t total = 0;
    auto take = [&](size_t bytes) {
        const size_t o = total;
        total += (bytes + 255) & ~(size_t)255;
        return o;
    };
    size_t ow[kLayers], ob[kLayers], omw[kLayers], ovw[kLayers], omb[kLayers], ovb[kLayers], ogw[kLayers],
        ogb[kLayers], owb[kLayers], owt[kLayers];
    for (int l = 0; l < kLayers; l++) {
        const size_t nw = (size_t)kOut[l] * kIn[l];
        ow[l] = take(4 * nw); omw[l] = take(4 * nw); ovw[l] = take(4 * nw);
        ob[l] = take(4 * kOut[l]); omb[l] = take(4 * kOut[l]); ovb[l] = take(4 * kOut[l]);
        ogw[l] = take(4 * (size_t)kOutP[l] * kInP[l] + 4 * (size_t)kH * kOutPad);
        ogb[l] = take(4 * (size_t)kOutP[l]);
        owb[l] = take(2 * (size_t)kOutP[l] * kInP[l]);
        owt[l] = take(2 * (size_t)kInP[l] * (l == 4 ? kInPad : kOutP[l]));
    }
    const size_t ox0 = take(2 * bt * kInPad), ox0t = take(2 * bt * kInPad);
    size_t oh[COR_MLP_LAYERS], oht[COR_MLP_LAYERS], oz[COR_MLP_LAYERS];
    for (int l = 0; l < COR_MLP_LAYERS; l++) {
        oh[l] = take(2 * bt * kH);
        oht[l] = take(2 * bt * kH);
        oz[l] = take(4 * bt * kH);
    }
    const size_t odz = take(2 * bt * kH), odzt = take(2 * bt * kH), odz2 = take(2 * bt * kH),
                 odz2t = take(2 * bt * kH);
    const size_t ody = take(2 * bt * kInPad), odyt = take(2 * bt * kOutPad), oy = take(4 * bt * kOutPad);
    const size_t oerr = take(sizeof(int));
    if (cudaMalloc(&m->block, total) != cudaSuccess) {
        delete m;
        return COR_ERR_NOMEM;
    }
    cudaMemset(m->block, 0, total);
    uint8_t* B = (uint8_t*)m->block;
    for (int l = 0; l < kLayers; l++) {
        m->w[l] = (float*)(B + ow[l]); m->mw[l] = (float*)(B + omw[l]); m->vw[l] = (float*)(B + ovw[l]);
        m->b[l] = (float*)(B + ob[l]); m->mb[l] = (float*)(B + omb[l]); m->vb[l] = (float*)(B + ovb[l]);
        m->gw[l] = (float*)(B + ogw[l]); m->gb[l] = (float*)(B + ogb[l]);
        m->wb[l] = (bf16*)(B + owb[l]); m->wt[l] = (bf16*)(B + owt[l]);
    }
    m->x0 = (bf16*)(B + ox0); m->x0t = (bf16*)(B + ox0t);
    for (int l = 0; l < COR_MLP_LAYERS; l++) {
        m->h[l] = (bf16*)(B + oh[l]); m->ht[l] = (bf16*)(B + oht[l]); m->z[l] = (float*)(B + oz[l]);
    }
    m->dz = (bf16*)(B + odz); m->dzt = (bf16*)(B + odzt); m->dz2 = (bf16*)(B + odz2); m->dz2t = (bf16*)(B + odz2t);
    m->dy = (bf16*)(B + ody); m->dyt = (bf16*)(B + odyt); m->y = (float*)(B + oy);
    m->dev_err = (int*)(B + oerr);
    if (cudaFuncSetAttribute(gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) !=
            cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {
        cudaFree(m->block);
        delete m;
        return COR_ERR_CUDA;
    }
    *out = m;
    return COR_OK;
}

int cor_mlp_destroy(cor_mlp* m) {
    if (!m) return COR_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    if (m->block) cudaFree(m->block);
    delete m;
    return COR_OK;
}

int cor_mlp_set_params(cor_mlp* m, const float* params) {
    if (!m || !params) return COR_ERR_INVALID;
    MTRY(m, cudaSetDevice(m->device));
    size_t wo[kLayers], bo[kLayers];
    param_offsets(wo, bo);
    for (int l = 0; l < kLayers; l++) {
        const size_t nw = (size_t)kOut[l] * kIn[l];
        MTRY(m, cudaMemcpy(m->w[l], params + wo[l], 4 * nw, cudaMemcpyHostToDevice));
        MTRY(m, cudaMemcpy(m->b[l], params + bo[l], 4 * (size_t)kOut[l], cudaMemcpyHostToDevice));
        MTRY(m, cudaMemset(m->mw[l], 0, 4 * nw));
        MTRY(m, cudaMemset(m->vw[l], 0, 4 * nw));
        MTRY(m, cudaMemset(m->mb[l], 0, 4 * (size_t)kOut[l]));
        MTRY(m, cudaMemset(m->vb[l], 0, 4 * (size_t)kOut[l]));
        ParamView p = view(m, l, false, nullptr);
        cast_kernel<<<(p.rows * p.cols + 255) / 256, 256>>>(p);
        MTRY(m, cudaGetLastError());
    }
    m->step = 0;
    MTRY(m, cudaDeviceSynchronize());
    return COR_OK;
}

int cor_mlp_get_params(cor_mlp* m, float* params) {
    if (!m || !params) return COR_ERR_INVALID;
    MTRY(m, cudaSetDevice(m->device));
    MTRY(m, cudaDeviceSynchronize());
    size_t wo[kLayers], bo[kLayers];
    param_offsets(wo, bo);
    for (int l = 0; l < kLayers; l++) {
        MTRY(m, cudaMemcpy(params + wo[l], m->w[l], 4 * (size_t)kOut[l] * kIn[l], cudaMemcpyDeviceToHost));
        MTRY(m, cudaMemcpy(params + bo[l], m->b[l], 4 * (size_t)kOut[l], cudaMemcpyDeviceToHost));
    }
    return COR_OK;
}

int cor_mlp_forward(cor_mlp* m, const float* x_dev, int32_t n, float* y_dev, void* stream) {
    if (!m) return COR_ERR_INVALID;
    if (n < 0 || n > m->max_bt || (n > 0 && (!x_dev || !y_dev)))
        return mfail(m, COR_ERR_INVALID, "batch of %d outside [0, %d]", n, m->max_bt);
    if (n == 0) return COR_OK;
    MTRY(m, cudaSetDevice(m->device));
    cudaStream_t s = (cudaStream_t)stream;
    const int bt = (n + kBM - 1) / kBM * kBM;
    int rc = forward(m, x_dev, n, bt, s);
    if (rc != COR_OK) return rc;
    copy_out_kernel<<<(n * COR_MLP_OUT + 255) / 256, 256, 0, s>>>(m->y, n, y_dev);
    MTRY(m, cudaGetLastError());
    MTRY(m, cudaStreamSynchronize(s));
    return check_err(m);
}

static int train(cor_mlp* m, const float* x, const float* t, int32_t n, float lr, float wd, float* loss,
                 float* grads, int do_update, void* stream) {
    if (!m) return COR_ERR_INVALID;
    if (n < 1 || n > m->max_bt || !x || !t || !loss)
        return mfail(m, COR_ERR_INVALID, "batch of %d outside [1, %d] or missing buffer", n, m->max_bt);
    MTRY(m, cudaSetDevice(m->device));
    cudaStream_t s = (cudaStream_t)stream;
    const int bt = (n + kBM - 1) / kBM * kBM;
    int rc = forward(m, x, n, bt, s);
    if (rc == COR_OK) rc = backward(m, t, n, bt, loss, s);
    if (rc == COR_OK) rc = update(m, lr, wd, grads, do_update, s);
    if (rc != COR_OK) return rc;
    MTRY(m, cudaStreamSynchronize(s));
    return check_err(m);
}

int cor_mlp_train_step(cor_mlp* m, const float* x_dev, const float* t_dev, int32_t n, float lr, float weight_decay,
                       float* loss_dev, float* grads_dev, void* stream) {
    return train(m, x_dev, t_dev, n, lr, weight_decay, loss_dev, grads_dev, 1, stream);
}

int cor_mlp_gradient(cor_mlp* m, const float* x_dev, const float* t_dev, int32_t n, float* loss_dev,
                     float* grads_dev, void* stream) {
    if (!grads_dev) return mfail(m, COR_ERR_INVALID, "no gradient buffer");
    return train(m, x_dev, t_dev, n, 0.f, 0.f, loss_dev, grads_dev, 0, stream);
}

}  // extern "C"
