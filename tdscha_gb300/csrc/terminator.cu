// Learned continued-fraction terminator: a 3-layer perceptron
//   h1 = tanh(x W1 + b1),  h2 = tanh(h1 W2 + b2),  y = h2 W3 + b3
// trained with mean-squared error and Adam, forward and backward on the GPU in
// float32 (inference optionally with bfloat16-rounded weights and layer
// inputs, float32 accumulation).  The network maps a window of normalised
// Lanczos coefficients to the next ones; the host side (terminator.py) builds
// the windows from runs of this engine and appends the prediction to the
// measured coefficients before the continued fraction.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

struct tdscha_mlp {
    int n_in = 0, n_h = 0, n_out = 0;
    // parameters, gradients, Adam moments: one flat float array each
    long n_par = 0;
    float *par = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    // activations / deltas for a batch of up to cap rows
    int cap = 0;
    float *x = nullptr, *t = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr;
    float *d2 = nullptr, *d1 = nullptr, *dy = nullptr, *loss = nullptr, *lossp = nullptr;
};

namespace tdscha {

// parameter offsets: W1 (n_in x n_h), b1, W2 (n_h x n_h), b2, W3 (n_h x n_out), b3
struct MlpOff {
    long w1, b1, w2, b2, w3, b3, n;
};
static MlpOff mlp_off(const tdscha_mlp *m) {
    MlpOff o;
    o.w1 = 0;
    o.b1 = o.w1 + (long)m->n_in * m->n_h;
    o.w2 = o.b1 + m->n_h;
    o.b2 = o.w2 + (long)m->n_h * m->n_h;
    o.w3 = o.b2 + m->n_h;
    o.b3 = o.w3 + (long)m->n_h * m->n_out;
    o.n = o.b3 + m->n_out;
    return o;
}

__device__ __forceinline__ float bf16_round(float v) {
    return __bfloat162float(__float2bfloat16_rn(v));
}

// C (rows x cols) = op(A) op(B) [+ bias] [tanh], A(i,k) = A[i*sai + k*sak],
// B(k,j) = B[k*sbk + j*sbj]; 32 x 32 tiles, 256 threads, 2 x 2 per thread.
// act: 0 none, 1 tanh.  bf16: round both operands to bfloat16 on load.
__global__ void k_mlp_gemm(const float *__restrict__ A, const float *__restrict__ B,
                           const float *__restrict__ bias, float *__restrict__ C, int rows,
                           int cols, int K, long sai, long sak, long sbk, long sbj, int act,
                           int bf16, int accumulate) {
    __shared__ float As[16][33], Bs[16][33];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 32; e += 256) {
            int kk = e % 16, ii = e / 16;
            int i = i0 + ii, k = k0 + kk;
            float a = (i < rows && k < K) ? A[i * sai + k * sak] : 0.f;
            int jj = e % 32, kb = e / 32;
            int j = j0 + jj, k2 = k0 + kb;
            float b = (j < cols && k2 < K) ? B[k2 * sbk + j * sbj] : 0.f;
            As[kk][ii] = bf16 ? bf16_round(a) : a;
            Bs[kb][jj] = bf16 ? bf16_round(b) : b;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float a0 = As[kk][ty], a1 = As[kk][ty + 16];
            float b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
            acc[0][0] = fmaf(a0, b0, acc[0][0]);
            acc[0][1] = fmaf(a0, b1, acc[0][1]);
            acc[1][0] = fmaf(a1, b0, acc[1][0]);
            acc[1][1] = fmaf(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
            if (i < rows && j < cols) {
                float v = acc[p][q];
                if (bias) v += bias[j];
                if (act == 1) v = tanhf(v);
                if (accumulate) v += C[(long)i * cols + j];
                C[(long)i * cols + j] = v;
            }
        }
}

// column sums: out[j] = sum_i D[i][j]
__global__ void k_mlp_colsum(const float *__restrict__ D, int rows, int cols, float *__restrict__ out) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.f;
    for (int i = 0; i < rows; ++i) s += D[(long)i * cols + j];
    out[j] = s;
}

// dy = 2 (y - t) / (rows * cols); loss partials per block
__global__ void k_mlp_mse(const float *__restrict__ y, const float *__restrict__ t, long n,
                          float scale, float *__restrict__ dy, float *__restrict__ part) {
    __shared__ float sh[32];
    float acc = 0.f;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        float r = y[e] - t[e];
        dy[e] = 2.f * r * scale;
        acc = fmaf(r, r, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
        part[blockIdx.x] = s;
    }
}

__global__ void k_mlp_sum(const float *__restrict__ part, int n, float scale, float *__restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < n; ++i) s += part[i];
        out[0] = (float)(s * scale);
    }
}

// d <- d * (1 - h^2)  (tanh derivative through the layer output h)
__global__ void k_mlp_dtanh(float *__restrict__ d, const float *__restrict__ h, long n) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
        d[e] *= 1.f - h[e] * h[e];
}

__global__ void k_mlp_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                           float *__restrict__ m2, long n, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        float gv = g[e];
        float a = b1 * m1[e] + (1.f - b1) * gv;
        float b = b2 * m2[e] + (1.f - b2) * gv * gv;
        m1[e] = a;
        m2[e] = b;
        p[e] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    }
}

static int mlp_reserve(tdscha_mlp *m, int rows) {
    if (rows <= m->cap) return TDSCHA_OK;
    float **bufs[] = {&m->x, &m->t, &m->h1, &m->h2, &m->y, &m->d2, &m->d1, &m->dy};
    for (float **b : bufs)
        if (*b) { cudaFree(*b); *b = nullptr; }
    m->cap = 0;
    size_t r = rows;
    TDS_CUDA(cudaMalloc(&m->x, sizeof(float) * r * m->n_in));
    TDS_CUDA(cudaMalloc(&m->t, sizeof(float) * r * m->n_out));
    TDS_CUDA(cudaMalloc(&m->h1, sizeof(float) * r * m->n_h));
    TDS_CUDA(cudaMalloc(&m->h2, sizeof(float) * r * m->n_h));
    TDS_CUDA(cudaMalloc(&m->y, sizeof(float) * r * m->n_out));
    TDS_CUDA(cudaMalloc(&m->d2, sizeof(float) * r * m->n_h));
    TDS_CUDA(cudaMalloc(&m->d1, sizeof(float) * r * m->n_h));
    TDS_CUDA(cudaMalloc(&m->dy, sizeof(float) * r * m->n_out));
    m->cap = rows;
    return TDSCHA_OK;
}

static dim3 gemm_grid(int rows, int cols) { return dim3(ceil_div(cols, 32), ceil_div(rows, 32)); }

// forward pass on m->x (rows x n_in) into m->h1, m->h2, m->y
static int mlp_forward(tdscha_mlp *m, int rows, int bf16, cudaStream_t st) {
    MlpOff o = mlp_off(m);
    const float *P = m->par;
    k_mlp_gemm<<<gemm_grid(rows, m->n_h), 256, 0, st>>>(m->x, P + o.w1, P + o.b1, m->h1, rows,
                                                         m->n_h, m->n_in, m->n_in, 1, m->n_h, 1, 1,
                                                         bf16, 0);
    k_mlp_gemm<<<gemm_grid(rows, m->n_h), 256, 0, st>>>(m->h1, P + o.w2, P + o.b2, m->h2, rows,
                                                         m->n_h, m->n_h, m->n_h, 1, m->n_h, 1, 1,
                                                         bf16, 0);
    k_mlp_gemm<<<gemm_grid(rows, m->n_out), 256, 0, st>>>(m->h2, P + o.w3, P + o.b3, m->y, rows,
                                                           m->n_out, m->n_h, m->n_h, 1, m->n_out, 1,
                                                           0, bf16, 0);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

// loss and gradients of the batch in m->x, m->t (forward must have run)
static int mlp_backward(tdscha_mlp *m, int rows, cudaStream_t st) {
    MlpOff o = mlp_off(m);
    const float *P = m->par;
    float *G = m->grad;
    const long ny = (long)rows * m->n_out;
    const int nbl = std::max(1, std::min(ceil_div(ny, 256), 256));
    k_mlp_mse<<<nbl, 256, 0, st>>>(m->y, m->t, ny, 1.f / (float)ny, m->dy, m->lossp);
    k_mlp_sum<<<1, 32, 0, st>>>(m->lossp, nbl, 1.0f / (float)ny, m->loss);
    // layer 3: dW3 = h2^T dy, db3 = colsum dy, d2 = dy W3^T
    k_mlp_gemm<<<gemm_grid(m->n_h, m->n_out), 256, 0, st>>>(m->h2, m->dy, nullptr, G + o.w3, m->n_h,
                                                             m->n_out, rows, 1, m->n_h, m->n_out, 1,
                                                             0, 0, 0);
    k_mlp_colsum<<<ceil_div(m->n_out, 128), 128, 0, st>>>(m->dy, rows, m->n_out, G + o.b3);
    k_mlp_gemm<<<gemm_grid(rows, m->n_h), 256, 0, st>>>(m->dy, P + o.w3, nullptr, m->d2, rows,
                                                         m->n_h, m->n_out, m->n_out, 1, 1, m->n_out,
                                                         0, 0, 0);
    k_mlp_dtanh<<<std::max(1, std::min(ceil_div((long)rows * m->n_h, 256), 1024)), 256, 0, st>>>(
        m->d2, m->h2, (long)rows * m->n_h);
    // layer 2
    k_mlp_gemm<<<gemm_grid(m->n_h, m->n_h), 256, 0, st>>>(m->h1, m->d2, nullptr, G + o.w2, m->n_h,
                                                           m->n_h, rows, 1, m->n_h, m->n_h, 1, 0, 0,
                                                           0);
    k_mlp_colsum<<<ceil_div(m->n_h, 128), 128, 0, st>>>(m->d2, rows, m->n_h, G + o.b2);
    k_mlp_gemm<<<gemm_grid(rows, m->n_h), 256, 0, st>>>(m->d2, P + o.w2, nullptr, m->d1, rows,
                                                         m->n_h, m->n_h, m->n_h, 1, 1, m->n_h, 0, 0,
                                                         0);
    k_mlp_dtanh<<<std::max(1, std::min(ceil_div((long)rows * m->n_h, 256), 1024)), 256, 0, st>>>(
        m->d1, m->h1, (long)rows * m->n_h);
    // layer 1
    k_mlp_gemm<<<gemm_grid(m->n_in, m->n_h), 256, 0, st>>>(m->x, m->d1, nullptr, G + o.w1, m->n_in,
                                                            m->n_h, rows, 1, m->n_in, m->n_h, 1, 0,
                                                            0, 0);
    k_mlp_colsum<<<ceil_div(m->n_h, 128), 128, 0, st>>>(m->d1, rows, m->n_h, G + o.b1);
    TDS_CHECK_LAUNCH();
    return TDSCHA_OK;
}

static int mlp_load_batch(tdscha_mlp *m, const float *x, const float *t, int rows, int device_ptrs,
                          cudaStream_t st) {
    TDS_TRY(mlp_reserve(m, rows));
    cudaMemcpyKind k = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    TDS_CUDA(cudaMemcpyAsync(m->x, x, sizeof(float) * rows * m->n_in, k, st));
    if (t) TDS_CUDA(cudaMemcpyAsync(m->t, t, sizeof(float) * rows * m->n_out, k, st));
    return TDSCHA_OK;
}

}  // namespace tdscha

using namespace tdscha;

extern "C" int tdscha_mlp_create(tdscha_mlp **out, int n_in, int n_hidden, int n_out) {
    set_error("");
    if (!out || n_in <= 0 || n_hidden <= 0 || n_out <= 0) { set_error("mlp_create: bad arguments"); return TDSCHA_ERR_ARG; }
    tdscha_mlp *m = new tdscha_mlp();
    m->n_in = n_in;
    m->n_h = n_hidden;
    m->n_out = n_out;
    m->n_par = mlp_off(m).n;
    bool ok = cudaMalloc(&m->par, sizeof(float) * m->n_par) == cudaSuccess &&
              cudaMalloc(&m->grad, sizeof(float) * m->n_par) == cudaSuccess &&
              cudaMalloc(&m->m1, sizeof(float) * m->n_par) == cudaSuccess &&
              cudaMalloc(&m->m2, sizeof(float) * m->n_par) == cudaSuccess &&
              cudaMalloc(&m->loss, sizeof(float)) == cudaSuccess &&
              cudaMalloc(&m->lossp, sizeof(float) * 256) == cudaSuccess &&
              cudaMemset(m->par, 0, sizeof(float) * m->n_par) == cudaSuccess &&
              cudaMemset(m->m1, 0, sizeof(float) * m->n_par) == cudaSuccess &&
              cudaMemset(m->m2, 0, sizeof(float) * m->n_par) == cudaSuccess;
    if (!ok) {
        set_error("mlp_create: %s", cudaGetErrorString(cudaGetLastError()));
        float *b[] = {m->par, m->grad, m->m1, m->m2, m->loss, m->lossp};
        for (float *p : b) if (p) cudaFree(p);
        delete m;
        return TDSCHA_ERR_CUDA;
    }
    *out = m;
    return TDSCHA_OK;
}

extern "C" int tdscha_mlp_destroy(tdscha_mlp *m) {
    if (!m) return TDSCHA_OK;
    cudaDeviceSynchronize();
    float *b[] = {m->par, m->grad, m->m1, m->m2, m->loss, m->lossp, m->x, m->t, m->h1, m->h2, m->y,
                  m->d2, m->d1, m->dy};
    for (float *p : b) if (p) cudaFree(p);
    delete m;
    return TDSCHA_OK;
}

extern "C" long tdscha_mlp_num_params(const tdscha_mlp *m) { return m ? m->n_par : -1; }

// params host <-> device (flat layout W1, b1, W2, b2, W3, b3, row-major weights);
// set also clears the Adam moments
extern "C" int tdscha_mlp_set_params(tdscha_mlp *m, const float *params) {
    set_error("");
    if (!m || !params) { set_error("mlp_set_params: null pointer"); return TDSCHA_ERR_ARG; }
    TDS_CUDA(cudaMemcpy(m->par, params, sizeof(float) * m->n_par, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemset(m->m1, 0, sizeof(float) * m->n_par));
    TDS_CUDA(cudaMemset(m->m2, 0, sizeof(float) * m->n_par));
    return TDSCHA_OK;
}

extern "C" int tdscha_mlp_get_params(tdscha_mlp *m, float *params) {
    set_error("");
    if (!m || !params) { set_error("mlp_get_params: null pointer"); return TDSCHA_ERR_ARG; }
    TDS_CUDA(cudaMemcpy(params, m->par, sizeof(float) * m->n_par, cudaMemcpyDeviceToHost));
    return TDSCHA_OK;
}

// y = net(x) for rows inputs (host buffers); bf16 != 0 rounds weights and
// layer inputs to bfloat16 (float32 accumulation)
extern "C" int tdscha_mlp_forward(tdscha_mlp *m, const float *x, int rows, int bf16, float *y) {
    set_error("");
    if (!m || !x || !y || rows <= 0) { set_error("mlp_forward: bad arguments"); return TDSCHA_ERR_ARG; }
    TDS_TRY(mlp_load_batch(m, x, nullptr, rows, 0, 0));
    TDS_TRY(mlp_forward(m, rows, bf16, 0));
    TDS_CUDA(cudaMemcpy(y, m->y, sizeof(float) * rows * m->n_out, cudaMemcpyDeviceToHost));
    return TDSCHA_OK;
}

// mean-squared-error loss of (x, t) and its gradient (host buffers)
extern "C" int tdscha_mlp_loss_grad(tdscha_mlp *m, const float *x, const float *t, int rows,
                                    float *loss, float *grad) {
    set_error("");
    if (!m || !x || !t || !loss || rows <= 0) { set_error("mlp_loss_grad: bad arguments"); return TDSCHA_ERR_ARG; }
    TDS_TRY(mlp_load_batch(m, x, t, rows, 0, 0));
    TDS_TRY(mlp_forward(m, rows, 0, 0));
    TDS_TRY(mlp_backward(m, rows, 0));
    TDS_CUDA(cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (grad) TDS_CUDA(cudaMemcpy(grad, m->grad, sizeof(float) * m->n_par, cudaMemcpyDeviceToHost));
    return TDSCHA_OK;
}

// one Adam step on the batch (x, t) given as device pointers; step counts from 1
extern "C" int tdscha_mlp_train_step(tdscha_mlp *m, const float *x, const float *t, int rows,
                                     float lr, float beta1, float beta2, float eps, int step,
                                     float *loss_out, void *stream) {
    set_error("");
    if (!m || !x || !t || rows <= 0 || step < 1) { set_error("mlp_train_step: bad arguments"); return TDSCHA_ERR_ARG; }
    cudaStream_t st = (cudaStream_t)stream;
    TDS_TRY(mlp_load_batch(m, x, t, rows, 1, st));
    TDS_TRY(mlp_forward(m, rows, 0, st));
    TDS_TRY(mlp_backward(m, rows, st));
    float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    k_mlp_adam<<<std::max(1, std::min(ceil_div(m->n_par, 256), 1024)), 256, 0, st>>>(
        m->par, m->grad, m->m1, m->m2, m->n_par, lr, beta1, beta2, eps, c1, c2);
    TDS_CHECK_LAUNCH();
    if (loss_out) {
        TDS_CUDA(cudaMemcpyAsync(loss_out, m->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
        TDS_CUDA(cudaStreamSynchronize(st));
    }
    return TDSCHA_OK;
}
