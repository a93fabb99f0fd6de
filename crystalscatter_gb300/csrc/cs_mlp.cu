// cs_mlp.cu — the surrogate network: BF16 tensor-core training and inference
// kernels (FP32 accumulation) and the handle behind cs_mlp_* (include/crystalscatter.h).
//
// Network: n_in -> H -> H -> H -> n_out, GELU after each hidden layer, linear
// output (log10 intensity on a coarse detector grid). Weights W[l] are n_out x
// n_in row-major (K-major), kept as FP32 master copies for Adam and as BF16
// copies (plus transposed BF16 copies) that the GEMMs read. Activations
// entering a GEMM are BF16; every product is accumulated in FP32.
//
// One GEMM form covers forward and backward: C[M x N] = A[M x K] . B[N x K]^T
// with A and B K-major:
//   forward   Z = X . W^T            (A = X,    B = W)
//   input grad dX = dZ . W  = dZ . (W^T)^T       (A = dZ,   B = W^T copy)
//   weight grad dW = dZ^T . X                    (A = dZ^T, B = X^T: transposed
//                                                 copies written by the producers)
// Tensor-core instruction: mma.sync m16n8k16 BF16 x BF16 -> FP32; tiles
// 128 x 128 x 32 per block of 8 warps (64 x 32 per warp), operands staged in
// shared memory by cp.async (double buffered) and fed by ldmatrix.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/crystalscatter.h"

namespace {

constexpr int BM = 128, BN = 128, BK = 32, LDS = BK + 8;  // smem row: 40 bf16 = 80 B (16-B aligned rows)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
    const int n = valid ? 16 : 0;  // 0 source bytes: the 16 destination bytes are zero-filled
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(n));
}

__device__ __forceinline__ void ldsm_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

enum Epi { EPI_F32 = 0, EPI_BIAS_GELU = 1, EPI_BIAS = 2 };

// C = A . B^T; M % 128 == 0, K % 32 == 0, N % 32 == 0 (rows of B beyond N read
// as zero). Epilogue (per element (m, n), z = acc [+ bias[n]]):
//   EPI_F32        C32[m*ldc+n] = acc
//   EPI_BIAS       C32[m*ldc+n] = z
//   EPI_BIAS_GELU  Z32[m*ldc+n] = z; H[m*ldc+n] = bf16(gelu z); HT[n*ldt+m] = bf16(gelu z)
template <int EPI>
__global__ void __launch_bounds__(256) k_gemm_tn(const __nv_bfloat16 *__restrict__ A, int lda,
                                                 const __nv_bfloat16 *__restrict__ B, int ldb, int M, int N, int K,
                                                 const float *__restrict__ bias, float *__restrict__ C32, int ldc,
                                                 __nv_bfloat16 *__restrict__ H, __nv_bfloat16 *__restrict__ HT,
                                                 int ldt) {
    __shared__ __align__(16) __nv_bfloat16 As[2][BM][LDS];
    __shared__ __align__(16) __nv_bfloat16 Bs[2][BN][LDS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps: 64 x 32 each
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

    float acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[i][j][r] = 0.0f;

    auto load_tile = [&](int buf, int k0) {
#pragma unroll
        for (int c = tid; c < BM * (BK / 8); c += 256) {
            const int row = c >> 2, ch = c & 3;
            cp_async16(&As[buf][row][ch * 8], A + (size_t)(m0 + row) * lda + k0 + ch * 8, true);
            const bool vb = (n0 + row) < N;
            cp_async16(&Bs[buf][row][ch * 8], vb ? (const void *)(B + (size_t)(n0 + row) * ldb + k0 + ch * 8) : (const void *)B,
                       vb);
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };

    const int nk = K / BK;
    load_tile(0, 0);
    for (int kt = 0; kt < nk; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < nk) {
            load_tile(buf ^ 1, (kt + 1) * BK);
            asm volatile("cp.async.wait_group 1;\n" ::);
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::);
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t af[4][4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = wm * 64 + i * 16 + (lane & 15);
                const int c = ks + (lane >> 4) * 8;
                ldsm_x4(af[i][0], af[i][1], af[i][2], af[i][3], &As[buf][r][c]);
            }
            uint32_t bf[4][2];
#pragma unroll
            for (int j = 0; j < 4; j += 2) {
                const int r = wn * 32 + j * 8 + (lane & 7) + ((lane >> 4) << 3);
                const int c = ks + ((lane >> 3) & 1) * 8;
                ldsm_x4(bf[j][0], bf[j][1], bf[j + 1][0], bf[j + 1][1], &Bs[buf][r][c]);
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bf[j][0], bf[j][1]);
        }
        __syncthreads();
    }

    // epilogue: element (g, 2t..2t+1) and (g+8, 2t..2t+1) of each 16 x 8 tile
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int m = m0 + wm * 64 + i * 16 + g + h * 8;
                const int n = n0 + wn * 32 + j * 8 + 2 * t;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int nn = n + e;
                    if (nn >= N) continue;
                    const float a = acc[i][j][h * 2 + e];
                    if (EPI == EPI_F32) {
                        C32[(size_t)m * ldc + nn] = a;
                    } else {
                        const float z = a + bias[nn];
                        if (EPI == EPI_BIAS) {
                            C32[(size_t)m * ldc + nn] = z;
                        } else {
                            C32[(size_t)m * ldc + nn] = z;
                            const __nv_bfloat16 hv = __float2bfloat16_rn(gelu(z));
                            H[(size_t)m * ldc + nn] = hv;
                            HT[(size_t)nn * ldt + m] = hv;
                        }
                    }
                }
            }
}

// dZ = dH * gelu'(Z) (FP32 in), as BF16 row-major and transposed
__global__ void k_gelu_back(const float *__restrict__ dH, const float *__restrict__ Z, int rows, int cols,
                            __nv_bfloat16 *__restrict__ dZ, __nv_bfloat16 *__restrict__ dZT) {
    const long n = (long)rows * cols;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        const __nv_bfloat16 v = __float2bfloat16_rn(dH[i] * gelu_grad(Z[i]));
        dZ[i] = v;
        dZT[(size_t)c * rows + r] = v;
    }
}

// MSE over rows x cols (only rows < valid count): loss partial sums and
// dY = 2 (Y - T) / (valid * cols) as BF16 row-major and transposed
__global__ void k_mse(const float *__restrict__ Y, const float *__restrict__ T, int rows, int valid, int cols,
                      __nv_bfloat16 *__restrict__ dY, __nv_bfloat16 *__restrict__ dYT, float *__restrict__ loss) {
    __shared__ float red[256];
    const long n = (long)rows * cols;
    const float scale = 2.0f / ((float)valid * (float)cols);
    float s = 0.0f;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i % cols);
        const float d = r < valid ? Y[i] - T[i] : 0.0f;
        s += d * d;
        const __nv_bfloat16 v = __float2bfloat16_rn(scale * d);
        dY[i] = v;
        dYT[(size_t)c * rows + r] = v;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] / ((float)valid * (float)cols));
}

// db[c] = sum over rows of dZ[r][c] (from the transposed copy: contiguous rows)
__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ dZT, int rows, int cols, float *__restrict__ db) {
    const int c = blockIdx.x;
    __shared__ float red[256];
    float s = 0.0f;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) s += __bfloat162float(dZT[(size_t)c * rows + r]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = red[0];
}

// Adam (bias-corrected) on the FP32 master copy; refreshes the BF16 copies
// W (rows x cols) and WT (cols x rows) of weight matrices (WT null for biases)
__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ gr, long n, int cols, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16 *__restrict__ wb, __nv_bfloat16 *__restrict__ wt,
                       int rows) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = gr[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb) {
            const __nv_bfloat16 b = __float2bfloat16_rn(wi);
            wb[i] = b;
            if (wt) {
                const int r = (int)(i / cols), c = (int)(i % cols);
                wt[(size_t)c * rows + r] = b;
            }
        }
    }
}

// input rows (FP32, n_in values) -> BF16 [rows x kin_pad] and its transpose, zero padded
__global__ void k_pack_input(const float *__restrict__ x, int valid, int rows, int nin, int kpad,
                             __nv_bfloat16 *__restrict__ X, __nv_bfloat16 *__restrict__ XT) {
    const long n = (long)rows * kpad;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int r = (int)(i / kpad), c = (int)(i % kpad);
        const float val = (r < valid && c < nin) ? x[(size_t)r * nin + c] : 0.0f;
        const __nv_bfloat16 b = __float2bfloat16_rn(val);
        X[i] = b;
        XT[(size_t)c * rows + r] = b;
    }
}

// bilinear upsampling of row-major images (s x s per row of `in`) to f*s x f*s,
// sample centres aligned (half-pixel convention), clamped at the borders
__global__ void k_upsample(const float *__restrict__ in, int n, int s, int f, float *__restrict__ out) {
    const int S = s * f;
    const long tot = (long)n * S * S;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < tot; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i / ((long)S * S)), p = (int)(i % ((long)S * S));
        const int Y = p / S, X = p % S;
        float fy = (Y + 0.5f) / f - 0.5f, fx = (X + 0.5f) / f - 0.5f;
        fy = fminf(fmaxf(fy, 0.0f), (float)(s - 1));
        fx = fminf(fmaxf(fx, 0.0f), (float)(s - 1));
        const int y0 = (int)floorf(fy), x0 = (int)floorf(fx);
        const int y1 = min(y0 + 1, s - 1), x1 = min(x0 + 1, s - 1);
        const float wy = fy - y0, wx = fx - x0;
        const float *b = in + (size_t)k * s * s;
        out[i] = (1 - wy) * ((1 - wx) * b[y0 * s + x0] + wx * b[y0 * s + x1]) +
                 wy * ((1 - wx) * b[y1 * s + x0] + wx * b[y1 * s + x1]);
    }
}

int grid1d(long n) {
    long g = (n + 255) / 256;
    if (g > 152L * 16) g = 152L * 16;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

// ---------------------------------------------------------------- handle
struct cs_mlp {
    int nin = 0, kin = 0, hid = 0, nout = 0, rows_cap = 0;
    int layers = 4;
    int in_dim[4], out_dim[4];
    // parameters: FP32 master, Adam moments, BF16 copies and transposes, grads
    float *w[4] = {}, *b[4] = {}, *mw[4] = {}, *vw[4] = {}, *mb[4] = {}, *vb[4] = {}, *gw[4] = {}, *gb[4] = {};
    __nv_bfloat16 *wb[4] = {}, *wt[4] = {};
    // activations (rows_cap rows)
    __nv_bfloat16 *X = nullptr, *XT = nullptr;
    float *Z[3] = {};
    __nv_bfloat16 *Hh[3] = {}, *HT[3] = {};
    float *Y = nullptr, *T = nullptr, *dH = nullptr;
    __nv_bfloat16 *dZ = nullptr, *dZT = nullptr;
    float *d_loss = nullptr;
    long step = 0;
    std::string err;
    cudaStream_t stream = nullptr;
};

namespace {

int mlp_fail(cs_mlp *m, int code, const std::string &msg) {
    if (m) m->err = msg;
    return code;
}

template <class T>
cudaError_t dalloc(T *&p, size_t n) {
    return cudaMalloc(&p, sizeof(T) * (n ? n : 1));
}

void mlp_free_acts(cs_mlp *m) {
    cudaFree(m->X);
    cudaFree(m->XT);
    for (int l = 0; l < 3; l++) {
        cudaFree(m->Z[l]);
        cudaFree(m->Hh[l]);
        cudaFree(m->HT[l]);
        m->Z[l] = nullptr;
        m->Hh[l] = m->HT[l] = nullptr;
    }
    cudaFree(m->Y);
    cudaFree(m->T);
    cudaFree(m->dH);
    cudaFree(m->dZ);
    cudaFree(m->dZT);
    m->X = m->XT = m->dZ = m->dZT = nullptr;
    m->Y = m->T = m->dH = nullptr;
    m->rows_cap = 0;
}

int ensure_rows(cs_mlp *m, int rows) {
    if (rows <= m->rows_cap) return CS_OK;
    mlp_free_acts(m);
    const size_t r = (size_t)rows;
    const size_t wide = (size_t)std::max(m->hid, m->nout);
    cudaError_t e = cudaSuccess;
    if ((e = dalloc(m->X, r * m->kin)) || (e = dalloc(m->XT, r * m->kin))) goto fail;
    for (int l = 0; l < 3; l++)
        if ((e = dalloc(m->Z[l], r * m->hid)) || (e = dalloc(m->Hh[l], r * m->hid)) || (e = dalloc(m->HT[l], r * m->hid)))
            goto fail;
    if ((e = dalloc(m->Y, r * m->nout)) || (e = dalloc(m->T, r * m->nout)) || (e = dalloc(m->dH, r * wide)) ||
        (e = dalloc(m->dZ, r * wide)) || (e = dalloc(m->dZT, r * wide)))
        goto fail;
    m->rows_cap = rows;
    return CS_OK;
fail:
    mlp_free_acts(m);
    return mlp_fail(m, CS_ERR_CUDA, std::string("activation buffers: ") + cudaGetErrorString(e));
}

template <int EPI>
void gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K, const float *bias,
          float *C, int ldc, __nv_bfloat16 *H, __nv_bfloat16 *HT, int ldt, cudaStream_t s) {
    dim3 grid((N + BN - 1) / BN, M / BM);
    k_gemm_tn<EPI><<<grid, 256, 0, s>>>(A, lda, B, ldb, M, N, K, bias, C, ldc, H, HT, ldt);
}

// forward pass of `rows` rows (multiple of 128) from m->X; output in m->Y
void forward(cs_mlp *m, int rows, cudaStream_t s) {
    const __nv_bfloat16 *in = m->X;
    int k = m->kin;
    for (int l = 0; l < 3; l++) {
        gemm<EPI_BIAS_GELU>(in, k, m->wb[l], k, rows, m->hid, k, m->b[l], m->Z[l], m->hid, m->Hh[l], m->HT[l], rows,
                            s);
        in = m->Hh[l];
        k = m->hid;
    }
    gemm<EPI_BIAS>(in, k, m->wb[3], k, rows, m->nout, k, m->b[3], m->Y, m->nout, nullptr, nullptr, 0, s);
}

// backward pass from dY (BF16 in m->dZ/m->dZT, rows x nout): parameter grads
void backward(cs_mlp *m, int rows, cudaStream_t s) {
    // layer 4: dW4 = dY^T . H3, db4, dH3 = dY . W4
    for (int l = 3; l >= 0; l--) {
        const int nout = m->out_dim[l], nin = m->in_dim[l];
        const __nv_bfloat16 *actT = l == 0 ? m->XT : m->HT[l - 1];
        // dW[l] (nout x nin) = dZ^T (nout x rows) . act (rows x nin)  ->  A = dZT, B = actT (nin x rows)
        gemm<EPI_F32>(m->dZT, rows, actT, rows, nout, nin, rows, nullptr, m->gw[l], nin, nullptr, nullptr, 0, s);
        k_bias_grad<<<nout, 256, 0, s>>>(m->dZT, rows, nout, m->gb[l]);
        if (l == 0) break;
        // dH (rows x nin) = dZ (rows x nout) . W (nout x nin) -> A = dZ, B = W^T (nin x nout)
        gemm<EPI_F32>(m->dZ, nout, m->wt[l], nout, rows, nin, nout, nullptr, m->dH, nin, nullptr, nullptr, 0, s);
        k_gelu_back<<<grid1d((long)rows * nin), 256, 0, s>>>(m->dH, m->Z[l - 1], rows, nin, m->dZ, m->dZT);
    }
}

}  // namespace

extern "C" {

cs_mlp *cs_mlp_create(int n_in, int hidden, int n_out, unsigned long long seed) {
    if (n_in <= 0 || n_in > 256 || hidden <= 0 || hidden % 128 || n_out <= 0 || n_out % 128) return nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return nullptr;
    cs_mlp *m = new (std::nothrow) cs_mlp;
    if (!m) return nullptr;
    m->nin = n_in;
    m->kin = (n_in + 31) / 32 * 32;
    m->hid = hidden;
    m->nout = n_out;
    const int ins[4] = {m->kin, hidden, hidden, hidden}, outs[4] = {hidden, hidden, hidden, n_out};
    std::memcpy(m->in_dim, ins, sizeof ins);
    std::memcpy(m->out_dim, outs, sizeof outs);
    // a blocking stream: ordered with work on the legacy default stream (the
    // caller's inputs and reads of the outputs) when no stream is passed
    cudaStreamCreate(&m->stream);
    // He-style uniform initialisation from a 64-bit LCG (deterministic per seed);
    // padded input columns start (and stay, their gradient is 0) at zero
    uint64_t st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto next = [&]() {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(st >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < 4; l++) {
        const size_t n = (size_t)outs[l] * ins[l];
        std::vector<float> hw(n, 0.0f), hb(outs[l], 0.0f);
        const int fan_in = l == 0 ? n_in : ins[l];
        const double a = std::sqrt(6.0 / fan_in) * (l == 3 ? 0.5 : 1.0);
        for (int r = 0; r < outs[l]; r++)
            for (int c = 0; c < (l == 0 ? n_in : ins[l]); c++) hw[(size_t)r * ins[l] + c] = (float)((2 * next() - 1) * a);
        bool ok = dalloc(m->w[l], n) == cudaSuccess && dalloc(m->mw[l], n) == cudaSuccess &&
                  dalloc(m->vw[l], n) == cudaSuccess && dalloc(m->gw[l], n) == cudaSuccess &&
                  dalloc(m->wb[l], n) == cudaSuccess && dalloc(m->wt[l], n) == cudaSuccess &&
                  dalloc(m->b[l], outs[l]) == cudaSuccess && dalloc(m->mb[l], outs[l]) == cudaSuccess &&
                  dalloc(m->vb[l], outs[l]) == cudaSuccess && dalloc(m->gb[l], outs[l]) == cudaSuccess;
        if (!ok) {
            cs_mlp_destroy(m);
            return nullptr;
        }
        // synchronous copies and memsets, complete before the stream's kernel
        cudaMemcpy(m->w[l], hw.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(m->b[l], hb.data(), sizeof(float) * outs[l], cudaMemcpyHostToDevice);
        cudaMemset(m->mw[l], 0, sizeof(float) * n);
        cudaMemset(m->vw[l], 0, sizeof(float) * n);
        cudaMemset(m->mb[l], 0, sizeof(float) * outs[l]);
        cudaMemset(m->vb[l], 0, sizeof(float) * outs[l]);
        // BF16 copies (an Adam step with lr 0 and zero gradient only refreshes them)
        cudaMemset(m->gw[l], 0, sizeof(float) * n);
        cudaDeviceSynchronize();
        k_adam<<<grid1d((long)n), 256, 0, m->stream>>>(m->w[l], m->mw[l], m->vw[l], m->gw[l], (long)n, ins[l], 0.0f,
                                                         0.9f, 0.999f, 1e-8f, 1.0f, 1.0f, m->wb[l], m->wt[l], outs[l]);
    }
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) {
        cs_mlp_destroy(m);
        return nullptr;
    }
    return m;
}

void cs_mlp_destroy(cs_mlp *m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    mlp_free_acts(m);
    for (int l = 0; l < 4; l++) {
        cudaFree(m->w[l]);
        cudaFree(m->b[l]);
        cudaFree(m->mw[l]);
        cudaFree(m->vw[l]);
        cudaFree(m->mb[l]);
        cudaFree(m->vb[l]);
        cudaFree(m->gw[l]);
        cudaFree(m->gb[l]);
        cudaFree(m->wb[l]);
        cudaFree(m->wt[l]);
    }
    cudaFree(m->d_loss);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

const char *cs_mlp_last_error(cs_mlp *m) { return m ? m->err.c_str() : "null network"; }

int cs_mlp_forward(cs_mlp *m, const float *d_x, int n, float *d_y, void *stream) {
    if (!m || !d_x || !d_y || n <= 0) return CS_ERR_PARAM;
    const int rows = (n + 127) / 128 * 128;
    int rc = ensure_rows(m, rows);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
    k_pack_input<<<grid1d((long)rows * m->kin), 256, 0, s>>>(d_x, n, rows, m->nin, m->kin, m->X, m->XT);
    forward(m, rows, s);
    cudaMemcpyAsync(d_y, m->Y, sizeof(float) * (size_t)n * m->nout, cudaMemcpyDeviceToDevice, s);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : mlp_fail(m, CS_ERR_CUDA, cudaGetErrorString(e));
}

int cs_mlp_gradients(cs_mlp *m, const float *d_x, const float *d_t, int n, float *loss, void *stream) {
    if (!m || !d_x || !d_t || n <= 0) return CS_ERR_PARAM;
    const int rows = (n + 127) / 128 * 128;
    int rc = ensure_rows(m, rows);
    if (rc) return rc;
    if (!m->d_loss && dalloc(m->d_loss, 1) != cudaSuccess) return mlp_fail(m, CS_ERR_CUDA, "loss buffer");
    cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
    k_pack_input<<<grid1d((long)rows * m->kin), 256, 0, s>>>(d_x, n, rows, m->nin, m->kin, m->X, m->XT);
    forward(m, rows, s);
    cudaMemsetAsync(m->T, 0, sizeof(float) * (size_t)rows * m->nout, s);
    cudaMemcpyAsync(m->T, d_t, sizeof(float) * (size_t)n * m->nout, cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(m->d_loss, 0, sizeof(float), s);
    k_mse<<<grid1d((long)rows * m->nout), 256, 0, s>>>(m->Y, m->T, rows, n, m->nout, m->dZ, m->dZT, m->d_loss);
    backward(m, rows, s);
    if (loss) {
        cudaMemcpyAsync(loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : mlp_fail(m, CS_ERR_CUDA, cudaGetErrorString(e));
}

int cs_mlp_train_step(cs_mlp *m, const float *d_x, const float *d_t, int n, float lr, float *loss, void *stream) {
    int rc = cs_mlp_gradients(m, d_x, d_t, n, nullptr, stream);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
    m->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - (float)std::pow((double)b1, (double)m->step);
    const float c2 = 1.0f - (float)std::pow((double)b2, (double)m->step);
    for (int l = 0; l < 4; l++) {
        const long nw = (long)m->out_dim[l] * m->in_dim[l];
        k_adam<<<grid1d(nw), 256, 0, s>>>(m->w[l], m->mw[l], m->vw[l], m->gw[l], nw, m->in_dim[l], lr, b1, b2, 1e-8f,
                                          c1, c2, m->wb[l], m->wt[l], m->out_dim[l]);
        k_adam<<<grid1d(m->out_dim[l]), 256, 0, s>>>(m->b[l], m->mb[l], m->vb[l], m->gb[l], m->out_dim[l], 1, lr, b1,
                                                     b2, 1e-8f, c1, c2, nullptr, nullptr, 1);
    }
    if (loss) {
        cudaMemcpyAsync(loss, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : mlp_fail(m, CS_ERR_CUDA, cudaGetErrorString(e));
}

// layer l: weights (out x in_padded) and bias (out) to / from host FP32 arrays
int cs_mlp_layer_dims(cs_mlp *m, int l, int *rows, int *cols) {
    if (!m || l < 0 || l > 3) return CS_ERR_PARAM;
    if (rows) *rows = m->out_dim[l];
    if (cols) *cols = m->in_dim[l];
    return CS_OK;
}

int cs_mlp_get_layer(cs_mlp *m, int l, float *w, float *b, float *gw, float *gb) {
    if (!m || l < 0 || l > 3) return CS_ERR_PARAM;
    cudaStreamSynchronize(m->stream);
    const size_t n = (size_t)m->out_dim[l] * m->in_dim[l];
    if (w) cudaMemcpy(w, m->w[l], sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (b) cudaMemcpy(b, m->b[l], sizeof(float) * m->out_dim[l], cudaMemcpyDeviceToHost);
    if (gw) cudaMemcpy(gw, m->gw[l], sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (gb) cudaMemcpy(gb, m->gb[l], sizeof(float) * m->out_dim[l], cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : mlp_fail(m, CS_ERR_CUDA, cudaGetErrorString(e));
}

int cs_mlp_set_layer(cs_mlp *m, int l, const float *w, const float *b) {
    if (!m || l < 0 || l > 3 || !w || !b) return CS_ERR_PARAM;
    cudaStreamSynchronize(m->stream);
    const size_t n = (size_t)m->out_dim[l] * m->in_dim[l];
    cudaMemcpy(m->w[l], w, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(m->b[l], b, sizeof(float) * m->out_dim[l], cudaMemcpyHostToDevice);
    cudaMemset(m->gw[l], 0, sizeof(float) * n);
    cudaDeviceSynchronize();
    k_adam<<<grid1d((long)n), 256, 0, m->stream>>>(m->w[l], m->mw[l], m->vw[l], m->gw[l], (long)n, m->in_dim[l], 0.0f,
                                                     0.9f, 0.999f, 1e-8f, 1.0f, 1.0f, m->wb[l], m->wt[l],
                                                     m->out_dim[l]);
    const cudaError_t e = cudaStreamSynchronize(m->stream);
    return e == cudaSuccess ? CS_OK : mlp_fail(m, CS_ERR_CUDA, cudaGetErrorString(e));
}

int cs_upsample_bilinear(const float *d_in, int n, int s, int factor, float *d_out, void *stream) {
    if (!d_in || !d_out || n <= 0 || s <= 0 || factor <= 0) return CS_ERR_PARAM;
    k_upsample<<<grid1d((long)n * s * s * factor * factor), 256, 0, (cudaStream_t)stream>>>(d_in, n, s, factor, d_out);
    return cudaGetLastError() == cudaSuccess ? CS_OK : CS_ERR_CUDA;
}

}  // extern "C"
