// learned.cu -- training and evaluation of the learned Newton starting pressure.
//
// Data: Riemann problems with density and pressure ratios log-uniform in
// [1e-4, 1e4] and velocity jumps uniform in [-5, 5] (normalised so that the
// geometric-mean density and pressure are 1), drawn from a counter-based hash
// (SplitMix64, S. Vigna) and labelled on the GPU by the FP64 exact solver
// (the reference's algorithm with a tight tolerance).  Problems that generate
// vacuum (no positive star pressure) are redrawn.
//
// Training: hand-written forward/backward kernels (FP32 arithmetic on
// BF16-rounded weights, inputs and hidden activations -- exactly what the
// tensor-core inference sees -- with straight-through gradients), per-block
// partial gradients reduced in a fixed order (deterministic), Adam on FP32
// master weights.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "hydro_device.cuh"
#include "learned.cuh"
#include "solver2d.h"

namespace hydro {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double uniform01(unsigned long long h) { return (double)(h >> 11) * 0x1p-53; }

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// One normalised training problem: rhoL = e^lr, rhoR = e^-lr, pL = e^lp, pR = e^-lp, uL = 0, uR = du.
struct Problem {
    double rL, uL, pL, rR, uR, pR, cL, cR;
};

__device__ Problem draw_problem(unsigned long long seed, long long i, double gamma)
{
    const double L4 = 4.605170185988091;  // log(1e4)/2: ratios in [1e-4, 1e4]
    Problem P;
    for (int attempt = 0; attempt < 32; ++attempt) {
        unsigned long long base = seed ^ ((unsigned long long)i * 0x632BE59BD9B4E019ull) ^ ((unsigned long long)attempt << 56);
        double lr = (2.0 * uniform01(splitmix64(base + 1)) - 1.0) * L4;
        double lp = (2.0 * uniform01(splitmix64(base + 2)) - 1.0) * L4;
        double du = (2.0 * uniform01(splitmix64(base + 3)) - 1.0) * 5.0;
        P.rL = exp(lr); P.rR = exp(-lr); P.pL = exp(lp); P.pR = exp(-lp);
        P.uL = 0.0; P.uR = du;
        P.cL = sqrt(gamma * P.pL / P.rL);
        P.cR = sqrt(gamma * P.pR / P.rR);
        // vacuum is generated when du >= 2 (cL + cR)/(gamma - 1); keep a margin
        if (du < 0.9 * 2.0 * (P.cL + P.cR) / (gamma - 1.0))
            return P;
    }
    P.uR = 0.0;
    return P;
}

__global__ void k_mlp_generate(long long n, unsigned long long seed, double gamma, float* __restrict__ X,
                               float* __restrict__ Y, double* __restrict__ raw)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Problem P = draw_problem(seed, i, gamma);
    float x[6];
    float pbar = mlp_features((float)P.rL, (float)P.uL, (float)P.pL, (float)P.cL, (float)P.rR, (float)P.uR,
                              (float)P.pR, (float)P.cR, x);
    Gas<double> G;
    G.g = gamma;
    G.gm1 = gamma - 1.0;
    G.zeta = (gamma - 1.0) / (gamma + 1.0);
    G.mu = (gamma - 1.0) / (2.0 * gamma);
    G.nu = (gamma + 1.0) / (2.0 * gamma);
    G.eps = 1e-12;
    double us, ps;
    StarInfo st;
    exact_riemann<double>(P.uL, P.uR, P.pL, P.pR, P.cL, P.cR, 1e-12, 200, G, us, ps, st);
    for (int k = 0; k < 6; ++k)
        X[i * 6 + k] = x[k];
    Y[i] = (float)log(ps / (double)pbar);
    if (raw) {
        double* r = raw + i * 6;
        r[0] = P.rL; r[1] = P.uL; r[2] = P.pL; r[3] = P.rR; r[4] = P.uR; r[5] = P.pR;
    }
}

// --- training -------------------------------------------------------------

constexpr int TB = 128;       // samples (= threads) per block
constexpr int HP = MLP_H + 1; // padded row of the per-sample activation arrays

struct TrainSmem {
    float W1[MLP_H * MLP_IN], b1[MLP_H], W2[MLP_H * MLP_H], b2[MLP_H], W3[MLP_H], b3;
    float H1[TB * HP];  // h1 (bf16-rounded), later dL/dz1
    float H2[TB * HP];  // h2 (bf16-rounded), later dL/dz2
    float Xs[TB * MLP_IN];
    float DY[TB];
    float L[TB];
};

// Loss sum and gradient (sum over the block's samples of d(e^2)/dw, scaled by
// `scale`) of one block of samples; written to part[block][MLP_NPARAM + 1].
__global__ void __launch_bounds__(TB) k_mlp_grad(const float* __restrict__ prm, const float* __restrict__ X,
                                                 const float* __restrict__ Y, long long n, long long offset,
                                                 float scale, float* __restrict__ part)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smraw);
    const int tid = threadIdx.x;
    for (int q = tid; q < MLP_H * MLP_IN; q += TB)
        S.W1[q] = bf16r(prm[MLP_W1 + q]);
    for (int q = tid; q < MLP_H * MLP_H; q += TB)
        S.W2[q] = bf16r(prm[MLP_W2 + q]);
    for (int q = tid; q < MLP_H; q += TB) {
        S.b1[q] = prm[MLP_B1 + q];
        S.b2[q] = prm[MLP_B2 + q];
        S.W3[q] = bf16r(prm[MLP_W3 + q]);
    }
    if (tid == 0)
        S.b3 = prm[MLP_B3];
    __syncthreads();

    const long long idx = offset + (long long)blockIdx.x * TB + tid;
    const bool valid = idx < n;
    float* h1 = S.H1 + tid * HP;
    float* h2 = S.H2 + tid * HP;
    float x[MLP_IN];
    for (int k = 0; k < MLP_IN; ++k) {
        x[k] = valid ? bf16r(X[idx * MLP_IN + k]) : 0.f;
        S.Xs[tid * MLP_IN + k] = x[k];
    }
    for (int i = 0; i < MLP_H; ++i) {
        float z = S.b1[i];
        for (int k = 0; k < MLP_IN; ++k)
            z += S.W1[i * MLP_IN + k] * x[k];
        h1[i] = bf16r(relu(z));
    }
    float y = S.b3;
    for (int o = 0; o < MLP_H; ++o) {
        float z = S.b2[o];
        for (int i = 0; i < MLP_H; ++i)
            z += S.W2[o * MLP_H + i] * h1[i];
        h2[o] = bf16r(relu(z));
        y += S.W3[o] * h2[o];
    }
    const float e = valid ? (y - Y[idx]) : 0.f;
    S.DY[tid] = 2.f * e * scale;
    S.L[tid] = e * e;
    __syncthreads();

    float* out = part + (size_t)blockIdx.x * (MLP_NPARAM + 1);
    // layer 3 and the loss
    if (tid < MLP_H) {
        float a = 0.f;
        for (int s = 0; s < TB; ++s)
            a += S.DY[s] * S.H2[s * HP + tid];
        out[MLP_W3 + tid] = a;
    } else if (tid == MLP_H) {
        float a = 0.f, l = 0.f;
        for (int s = 0; s < TB; ++s) {
            a += S.DY[s];
            l += S.L[s];
        }
        out[MLP_B3] = a;
        out[MLP_NPARAM] = l;
    }
    __syncthreads();
    // dL/dz2 in place of h2
    for (int o = 0; o < MLP_H; ++o)
        h2[o] = (h2[o] > 0.f) ? S.DY[tid] * S.W3[o] : 0.f;
    __syncthreads();
    // layer 2: each thread a 4 x 8 block of dW2, plus db2
    {
        const int o0 = (tid / 8) * 4, i0 = (tid % 8) * 8;
        float acc[4][8];
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 8; ++b)
                acc[a][b] = 0.f;
        for (int s = 0; s < TB; ++s) {
            float d[4], hv[8];
            for (int a = 0; a < 4; ++a)
                d[a] = S.H2[s * HP + o0 + a];
            for (int b = 0; b < 8; ++b)
                hv[b] = S.H1[s * HP + i0 + b];
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 8; ++b)
                    acc[a][b] += d[a] * hv[b];
        }
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 8; ++b)
                out[MLP_W2 + (o0 + a) * MLP_H + i0 + b] = acc[a][b];
        if (tid < MLP_H) {
            float a = 0.f;
            for (int s = 0; s < TB; ++s)
                a += S.H2[s * HP + tid];
            out[MLP_B2 + tid] = a;
        }
    }
    __syncthreads();
    // dL/dz1 in place of h1
    {
        float dz[MLP_H];
        for (int i = 0; i < MLP_H; ++i) {
            float a = 0.f;
            for (int o = 0; o < MLP_H; ++o)
                a += h2[o] * S.W2[o * MLP_H + i];
            dz[i] = (h1[i] > 0.f) ? a : 0.f;
        }
        __syncthreads();
        for (int i = 0; i < MLP_H; ++i)
            h1[i] = dz[i];
    }
    __syncthreads();
    // layer 1
    for (int q = tid; q < MLP_H * MLP_IN + MLP_H; q += TB) {
        float a = 0.f;
        if (q < MLP_H * MLP_IN) {
            const int i = q / MLP_IN, k = q % MLP_IN;
            for (int s = 0; s < TB; ++s)
                a += S.H1[s * HP + i] * S.Xs[s * MLP_IN + k];
            out[MLP_W1 + q] = a;
        } else {
            const int i = q - MLP_H * MLP_IN;
            for (int s = 0; s < TB; ++s)
                a += S.H1[s * HP + i];
            out[MLP_B1 + i] = a;
        }
    }
}

// grad[p] = sum over blocks of part[b][p] (fixed order: deterministic).
__global__ void k_mlp_reduce(const float* __restrict__ part, int nblocks, float* __restrict__ grad)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > MLP_NPARAM)
        return;
    float a = 0.f;
    for (int b = 0; b < nblocks; ++b)
        a += part[(size_t)b * (MLP_NPARAM + 1) + p];
    grad[p] = a;
}

__global__ void k_mlp_adam(float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m1,
                           float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= MLP_NPARAM)
        return;
    float g = grad[p];
    float a = b1 * m1[p] + (1.f - b1) * g;
    float v = b2 * m2[p] + (1.f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    prm[p] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

// Tensor-core inference over an array of feature rows (one warp per 32 rows).
__global__ void __launch_bounds__(256) k_mlp_predict(const uint32_t* __restrict__ frag, const float* __restrict__ prm,
                                                     const float* __restrict__ X, int n, float* __restrict__ Y)
{
    __shared__ MlpShared S;
    mlp_load_shared(S, frag, prm, threadIdx.x, blockDim.x);
    __syncthreads();
    const int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31;
    const int i = base + (threadIdx.x & 31);
    float x[6];
    for (int k = 0; k < 6; ++k)
        x[k] = (i < n) ? X[(size_t)i * 6 + k] : 0.f;
    if (base < n) {  // warp-uniform
        float y = warp_mlp(x, S);
        if (i < n)
            Y[i] = y;
    }
}

__global__ void k_features(const double* __restrict__ st, int n, double gamma, float* __restrict__ X)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const double* s = st + (size_t)i * 6;
    float cL = (float)sqrt(gamma * s[2] / s[0]), cR = (float)sqrt(gamma * s[5] / s[3]);
    float x[6];
    mlp_features((float)s[0], (float)s[1], (float)s[2], cL, (float)s[3], (float)s[4], (float)s[5], cR, x);
    for (int k = 0; k < 6; ++k)
        X[(size_t)i * 6 + k] = x[k];
}

}  // namespace hydro

using namespace hydro;

struct hydro_mlp {
    float* prm = nullptr;   // FP32 master weights
    float* m1 = nullptr;
    float* m2 = nullptr;
    float* grad = nullptr;
    float* part = nullptr;
    int part_blocks = 0;
    uint32_t* frag = nullptr;
    float* X = nullptr;
    float* Y = nullptr;
    long long n = 0;
    long long adam_t = 0;
};

static int mlp_smem_attr()
{
    static int done = 0;
    if (!done) {
        if (!cuda_ok(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(TrainSmem)),
                     "mlp smem"))
            return -1;
        done = 1;
    }
    return 0;
}

static int ensure_part(hydro_mlp* h, int blocks)
{
    if (blocks <= h->part_blocks)
        return 0;
    cudaFree(h->part);
    h->part = nullptr;
    if (!cuda_ok(cudaMalloc(&h->part, sizeof(float) * (size_t)blocks * (MLP_NPARAM + 1)), "mlp partials"))
        return -1;
    h->part_blocks = blocks;
    return 0;
}

static void refresh_frag(hydro_mlp* h)
{
    k_mlp_pack<<<(8 * 32 + 4 * 8 * 32 + 4 * 32 + 127) / 128, 128>>>(h->prm, h->frag);
    count_launch();
}

// loss and gradient of samples [off, off+cnt) of X/Y, mean over cnt
static int batch_grad(hydro_mlp* h, const float* X, const float* Y, long long n, long long off, int cnt, float* loss)
{
    int blocks = (cnt + TB - 1) / TB;
    if (ensure_part(h, blocks))
        return -1;
    long long end = off + cnt < n ? off + cnt : n;
    k_mlp_grad<<<blocks, TB, sizeof(TrainSmem)>>>(h->prm, X, Y, end, off, 1.0f / (float)cnt, h->part);
    k_mlp_reduce<<<(MLP_NPARAM + 1 + 255) / 256, 256>>>(h->part, blocks, h->grad);
    count_launch(2);
    if (loss) {
        float l = 0.f;
        if (!cuda_ok(cudaMemcpy(&l, h->grad + MLP_NPARAM, sizeof(float), cudaMemcpyDeviceToHost), "loss"))
            return -1;
        *loss = l / (float)cnt;
    }
    return cuda_ok(cudaGetLastError(), "mlp grad") ? 0 : -1;
}

extern "C" {

int hydro_mlp_create(hydro_mlp** out, unsigned long long seed)
{
    *out = nullptr;
    if (mlp_smem_attr())
        return -1;
    hydro_mlp* h = new hydro_mlp();
    if (!cuda_ok(cudaMalloc(&h->prm, sizeof(float) * MLP_NPARAM), "mlp") ||
        !cuda_ok(cudaMalloc(&h->m1, sizeof(float) * MLP_NPARAM), "mlp") ||
        !cuda_ok(cudaMalloc(&h->m2, sizeof(float) * MLP_NPARAM), "mlp") ||
        !cuda_ok(cudaMalloc(&h->grad, sizeof(float) * (MLP_NPARAM + 1)), "mlp") ||
        !cuda_ok(cudaMalloc(&h->frag, sizeof(uint32_t) * MLP_NFRAG), "mlp")) {
        delete h;
        return -1;
    }
    // He-uniform initialisation on the host from a SplitMix64 stream
    std::vector<float> p(MLP_NPARAM, 0.f);
    unsigned long long s = seed * 0x9E3779B97F4A7C15ull + 1;
    auto uni = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        unsigned long long z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * 0x1p-53 * 2.0 - 1.0;
    };
    for (int q = 0; q < MLP_H * MLP_IN; ++q)
        p[MLP_W1 + q] = (float)(uni() * sqrt(6.0 / MLP_IN));
    for (int q = 0; q < MLP_H * MLP_H; ++q)
        p[MLP_W2 + q] = (float)(uni() * sqrt(6.0 / MLP_H));
    for (int q = 0; q < MLP_H; ++q)
        p[MLP_W3 + q] = (float)(uni() * sqrt(3.0 / MLP_H));
    cudaMemcpy(h->prm, p.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice);
    cudaMemset(h->m1, 0, sizeof(float) * MLP_NPARAM);
    cudaMemset(h->m2, 0, sizeof(float) * MLP_NPARAM);
    refresh_frag(h);
    *out = h;
    return cuda_ok(cudaDeviceSynchronize(), "mlp init") ? 0 : -1;
}

void hydro_mlp_destroy(hydro_mlp* h)
{
    if (!h)
        return;
    cudaFree(h->prm);
    cudaFree(h->m1);
    cudaFree(h->m2);
    cudaFree(h->grad);
    cudaFree(h->part);
    cudaFree(h->frag);
    cudaFree(h->X);
    cudaFree(h->Y);
    delete h;
}

int hydro_mlp_get_params(hydro_mlp* h, float* params)
{
    return cuda_ok(cudaMemcpy(params, h->prm, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost), "get params") ? 0
                                                                                                                : -1;
}

int hydro_mlp_set_params(hydro_mlp* h, const float* params)
{
    if (!cuda_ok(cudaMemcpy(h->prm, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice), "set params"))
        return -1;
    cudaMemset(h->m1, 0, sizeof(float) * MLP_NPARAM);
    cudaMemset(h->m2, 0, sizeof(float) * MLP_NPARAM);
    h->adam_t = 0;
    refresh_frag(h);
    return cuda_ok(cudaDeviceSynchronize(), "set params") ? 0 : -1;
}

int hydro_mlp_generate(hydro_mlp* h, long long n, unsigned long long seed, double gamma, double* raw_host)
{
    cudaFree(h->X);
    cudaFree(h->Y);
    h->X = h->Y = nullptr;
    h->n = 0;
    double* raw = nullptr;
    if (!cuda_ok(cudaMalloc(&h->X, sizeof(float) * 6 * (size_t)n), "mlp data") ||
        !cuda_ok(cudaMalloc(&h->Y, sizeof(float) * (size_t)n), "mlp data"))
        return -1;
    if (raw_host && !cuda_ok(cudaMalloc(&raw, sizeof(double) * 6 * (size_t)n), "mlp raw"))
        return -1;
    k_mlp_generate<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, gamma, h->X, h->Y, raw);
    count_launch();
    if (!cuda_ok(cudaDeviceSynchronize(), "mlp generate"))
        return -1;
    if (raw_host) {
        cudaMemcpy(raw_host, raw, sizeof(double) * 6 * (size_t)n, cudaMemcpyDeviceToHost);
        cudaFree(raw);
    }
    h->n = n;
    return 0;
}

int hydro_mlp_get_data(hydro_mlp* h, float* X, float* Y, long long n)
{
    if (n > h->n)
        n = h->n;
    if (X && !cuda_ok(cudaMemcpy(X, h->X, sizeof(float) * 6 * (size_t)n, cudaMemcpyDeviceToHost), "get data"))
        return -1;
    if (Y && !cuda_ok(cudaMemcpy(Y, h->Y, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost), "get data"))
        return -1;
    return 0;
}

// Trains on the generated set; loss_per_epoch[e] = mean squared error of epoch e
// (mean of the batch losses).  The last `holdout` samples are not trained on.
int hydro_mlp_train(hydro_mlp* h, int epochs, int batch, float lr, long long holdout, float* loss_per_epoch)
{
    if (!h->n) {
        set_error("hydro_mlp_train: no data (call hydro_mlp_generate)");
        return -1;
    }
    long long ntrain = h->n - holdout;
    if (ntrain < batch)
        ntrain = h->n;
    int nb = (int)(ntrain / batch);
    for (int e = 0; e < epochs; ++e) {
        float lr_e = lr * (0.5f * (1.0f + cosf(3.14159265f * (float)e / (float)epochs)));  // cosine schedule
        double lsum = 0.0;
        for (int b = 0; b < nb; ++b) {
            float l = 0.f;
            // loss readback only at a few batches per epoch (it synchronises)
            if (batch_grad(h, h->X, h->Y, ntrain, (long long)b * batch, batch, (b % 64 == 0) ? &l : nullptr))
                return -1;
            if (b % 64 == 0)
                lsum += l;
            h->adam_t++;
            float c1 = 1.f - powf(0.9f, (float)h->adam_t), c2 = 1.f - powf(0.999f, (float)h->adam_t);
            k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256>>>(h->prm, h->grad, h->m1, h->m2, lr_e, 0.9f, 0.999f, 1e-8f,
                                                           c1, c2);
            count_launch();
        }
        if (loss_per_epoch)
            loss_per_epoch[e] = (float)(lsum / ((nb + 63) / 64));
    }
    refresh_frag(h);
    return cuda_ok(cudaDeviceSynchronize(), "mlp train") ? 0 : -1;
}

// Mean loss and gradient of n given samples (host arrays) with the current weights.
int hydro_mlp_gradient(hydro_mlp* h, const float* X, const float* Y, int n, float* grad, float* loss)
{
    float *dX = nullptr, *dY = nullptr;
    if (!cuda_ok(cudaMalloc(&dX, sizeof(float) * 6 * n), "grad data") ||
        !cuda_ok(cudaMalloc(&dY, sizeof(float) * n), "grad data"))
        return -1;
    cudaMemcpy(dX, X, sizeof(float) * 6 * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dY, Y, sizeof(float) * n, cudaMemcpyHostToDevice);
    int rc = batch_grad(h, dX, dY, n, 0, n, loss);
    if (!rc && !cuda_ok(cudaMemcpy(grad, h->grad, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost), "grad"))
        rc = -1;
    cudaFree(dX);
    cudaFree(dY);
    return rc;
}

// Tensor-core inference on host feature rows.
int hydro_mlp_predict(hydro_mlp* h, const float* X, int n, float* Y)
{
    float *dX = nullptr, *dY = nullptr;
    if (!cuda_ok(cudaMalloc(&dX, sizeof(float) * 6 * (size_t)n), "predict") ||
        !cuda_ok(cudaMalloc(&dY, sizeof(float) * (size_t)n), "predict"))
        return -1;
    cudaMemcpy(dX, X, sizeof(float) * 6 * (size_t)n, cudaMemcpyHostToDevice);
    k_mlp_predict<<<(n + 255) / 256, 256>>>(h->frag, h->prm, dX, n, dY);
    count_launch();
    int rc = cuda_ok(cudaMemcpy(Y, dY, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost), "predict") ? 0 : -1;
    cudaFree(dX);
    cudaFree(dY);
    return rc;
}

// The device feature map on host states (rhoL,uL,pL,rhoR,uR,pR per row).
int hydro_mlp_features(const double* states, int n, double gamma, float* X)
{
    double* dS = nullptr;
    float* dX = nullptr;
    if (!cuda_ok(cudaMalloc(&dS, sizeof(double) * 6 * (size_t)n), "features") ||
        !cuda_ok(cudaMalloc(&dX, sizeof(float) * 6 * (size_t)n), "features"))
        return -1;
    cudaMemcpy(dS, states, sizeof(double) * 6 * (size_t)n, cudaMemcpyHostToDevice);
    k_features<<<(n + 255) / 256, 256>>>(dS, n, gamma, dX);
    count_launch();
    int rc = cuda_ok(cudaMemcpy(X, dX, sizeof(float) * 6 * (size_t)n, cudaMemcpyDeviceToHost), "features") ? 0 : -1;
    cudaFree(dS);
    cudaFree(dX);
    return rc;
}

// Device pointers of the packed network (for the solver kernels).
const unsigned int* hydro_mlp_device_fragments(hydro_mlp* h) { return h->frag; }
const float* hydro_mlp_device_params(hydro_mlp* h) { return h->prm; }

}  // extern "C"
