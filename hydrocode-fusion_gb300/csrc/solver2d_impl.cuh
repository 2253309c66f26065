// solver2d_impl.cuh -- host side of the 2D solver, instantiated per precision.
//
// Memory: one cudaMalloc per solver holding 26 planes of m x ld elements
// (two 13-plane states: rho,u,v,p,E + 4 x-slopes + 4 y-slopes), plus the -1
// boundary table and the control block.  ld is n rounded up to 32 elements so
// every x-station starts on a 128-byte boundary.  At 4096^2 that is 3.5 GB in
// FP64 and 1.75 GB in FP32: far below HBM capacity, so nothing is ever paged.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <stdlib.h>

#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "solver2d.h"
#include "step2d.cuh"
#include "strip2d.cuh"

namespace hydro {

// Compiled configurations of the unsplit step kernel (tile TJ x TI cells,
// NT threads, at least MINB resident CTAs per SM requested from ptxas).  The
// autotuner (Solver2D::autotune) times them on the actual problem.
// tma = 1 or 2: the persistent TMA-staged kernel (k_step_tma) with that many
// shared-memory stages, launched with occ CTAs per SM; tma = 0: one CTA per
// tile (k_step_unsplit).  strip = 1: the FP32 strip kernel (k_step_strip,
// strip2d.cuh), persistent with occ CTAs per SM, TJ = rows per work unit,
// TI = columns a strip updates.
// The smallest shared-memory carve-out (per cent of the largest, 228 KB) that
// holds `ctas` CTAs of `bytes` shared memory each (the hardware keeps 1 KB per
// CTA besides), so that the rest of the unified L1/shared storage is L1 for the
// tile code's spills and the exact path's stack.  The percentage is rounded
// down: the driver takes the smallest configuration at or above it.
inline int carve_for(size_t bytes, int ctas)
{
    static const int cfg_kb[] = {0, 8, 16, 32, 64, 100, 132, 164, 196, 228};
    const size_t need = (size_t)ctas * (bytes + 1024);
    for (int kb : cfg_kb)
        if ((size_t)kb * 1024 >= need)
            return kb * 100 / 228;
    return 100;
}

template <typename R>
struct StepVariant {
    int TJ, TI, NT, MINB;
    size_t smem;
    const void* kern;
    int tma = 0;
    int occ = 0;
    StepMaps maps[2];  // tma: descriptors of the two state buffers
    int strip = 0;
    int carve = 100;   // shared-memory carve-out of the L1/shared storage, per cent
    int mlp_min = STRIP_MLP_MIN;  // strip kernel, learned form: smallest flush the network runs on
    int mlp_global = 0;           // strip kernel, learned form: network image read from global memory
};

template <typename R, int TJ, int TI, int NT, int MINB, bool LEARNED = false, int RS = 0>
StepVariant<R> step_variant()
{
    return StepVariant<R>{TJ, TI, NT, MINB, UnsplitSmem<R, TJ, TI>::bytes,
                          (const void*)k_step_unsplit<R, TJ, TI, NT, MINB, LEARNED, RS>, 0, 0, {}};
}

template <typename R, int TJ, int TI, int NT, int MINB, bool LEARNED = false, int STAGES = 2, int RS = 0>
StepVariant<R> tma_variant()
{
    return StepVariant<R>{TJ, TI, NT, MINB, TmaSmem<R, TJ, TI, LEARNED, STAGES>::launch_bytes,
                          (const void*)k_step_tma<R, TJ, TI, NT, MINB, LEARNED, STAGES, RS>, STAGES, 0, {}};
}

template <int NW, int MINB, bool LEARNED>
StepVariant<float> strip_variant(int seg, int carve, int mlp_min = STRIP_MLP_MIN, int mlp_global = 0)
{
    // a learned variant that reads the network image from global memory needs no shared copy of it
    StepVariant<float> v{seg, STRIP_W, NW * 32, MINB,
                         (LEARNED && !mlp_global) ? StripSmem<NW, true>::bytes : StripSmem<NW, false>::bytes,
                         (const void*)k_step_strip<NW, MINB, LEARNED>, 0, 0, {}};
    v.strip = 1;
    v.carve = carve;
    v.mlp_min = mlp_min;
    v.mlp_global = mlp_global;
    return v;
}

// The compiled configurations, each list instantiated in its own translation
// unit so the kernels compile in parallel (f32_gathered.cu, f32_tma.cu,
// f32_learned.cu, f64_variants.cu, g2d_f32.cu, g2d_f64.cu).  The lists keep
// the configurations that the autotuner picks on some workload;
// HYDRO_STEP_VARIANT* index into them.  The *_g2d lists are the unsplit step
// with the genuinely-2D interface solver (HYDRO_SOLVER_G2D).
void variants_f32_gathered(std::vector<StepVariant<float>>& v);
void variants_f32_tma(std::vector<StepVariant<float>>& v);
void variants_f32_learned(std::vector<StepVariant<float>>& v);
void variants_f32_strip(std::vector<StepVariant<float>>& v, bool learned);
void variants_f64(std::vector<StepVariant<double>>& v);
void variants_f32_g2d(std::vector<StepVariant<float>>& v);
void variants_f64_g2d(std::vector<StepVariant<double>>& v);

template <typename R> struct Variants;
template <> struct Variants<double> {
    static std::vector<StepVariant<double>> all(bool, int rs)
    {
        std::vector<StepVariant<double>> v;
        if (rs == HYDRO_SOLVER_G2D)
            variants_f64_g2d(v);
        else
            variants_f64(v);
        return v;
    }
    static constexpr int SJ = 16, SI = 32, SNT = 256;  // split sweeps
};
template <> struct Variants<float> {
    static std::vector<StepVariant<float>> all(bool learned, int rs)
    {
        std::vector<StepVariant<float>> v;
        if (rs == HYDRO_SOLVER_G2D) {
            variants_f32_g2d(v);
        } else if (learned) {
            // the strip kernels first: index 0 is the default when nothing is tuned
            variants_f32_strip(v, true);
            variants_f32_learned(v);
        } else {
            variants_f32_strip(v, false);
            variants_f32_tma(v);
            variants_f32_gathered(v);
        }
        return v;
    }
    static constexpr int SJ = 16, SI = 32, SNT = 256;
};

// ---------------------------------------------------------------------------
// helper kernels
// ---------------------------------------------------------------------------

// Copy an x-major FP64 host-layout plane (staged on the device) into a pitched plane.
template <typename R>
__global__ void k_pack_plane(const double* __restrict__ in, R* __restrict__ out, int m, int n, int ld)
{
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)m * n;
    for (; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(idx / n), i = (int)(idx - (size_t)j * n);
        out[(size_t)j * ld + i] = (R)in[idx];
    }
}

template <typename R>
__global__ void k_unpack_plane(const R* __restrict__ in, double* __restrict__ out, int m, int n, int ld)
{
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t total = (size_t)m * n;
    for (; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(idx / n), i = (int)(idx - (size_t)j * n);
        out[idx] = (double)in[(size_t)j * ld + i];
    }
}

// Gather of one field from the caller's row arrays in host memory (read by
// the GPU through coherent pageable-memory access): row j at rows[j].
template <typename R>
__global__ void k_gather_rows(const double* const* __restrict__ rows, R* __restrict__ out, int m, int n, int ld)
{
    const int j = blockIdx.y;
    const double* __restrict__ r = rows[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[(size_t)j * ld + i] = (R)r[i];
}

template <typename R>
__global__ void k_scatter_rows(const R* __restrict__ in, double* const* __restrict__ rows, int m, int n, int ld)
{
    const int j = blockIdx.y;
    double* __restrict__ r = rows[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        r[i] = (double)in[(size_t)j * ld + i];
}

// E = 0.5 u^2 + p/(gamma-1)/rho; E += 0.5 v^2 (the driver's formula,
// src/hydrocode_2D/hydrocode.c:252-253), evaluated in FP64.
static __global__ void k_energy(const double* rho, const double* u, const double* v, const double* p, double* E, size_t total,
                         double gamma)
{
    size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        double e = 0.5 * u[idx] * u[idx] + p[idx] / (gamma - 1.0) / rho[idx];
        e += 0.5 * v[idx] * v[idx];
        E[idx] = e;
    }
}

// Edge values of the initial state for the fixed (-1) boundary code:
// [4][n] left (j=0), [4][n] right (j=m-1), [4][m] down (i=0), [4][m] up (i=n-1).
template <typename R>
__global__ void k_ghost0(const R* __restrict__ w, size_t plane, int m, int n, int ld, R* __restrict__ g)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        for (int k = 0; k < 4; ++k) {
            g[k * n + t] = w[k * plane + t];
            g[4 * n + k * n + t] = w[k * plane + (size_t)(m - 1) * ld + t];
        }
    }
    if (t < m) {
        for (int k = 0; k < 4; ++k) {
            g[8 * n + k * m + t] = w[k * plane + (size_t)t * ld];
            g[8 * n + 4 * m + k * m + t] = w[k * plane + (size_t)t * ld + (n - 1)];
        }
    }
}

// CFL: h_S_max = min over cells of min(h_x,h_y)/(|c|+|u|+|v|), c = sqrt(gamma p/rho),
// in FP64 (grp_solver_2D_EUL_source.c:180-188).  fmin is exact, so the
// warp-shuffle/atomic reduction order cannot change the result.  The minimum
// of non-negative doubles is taken on their bit patterns (same order).
template <typename R>
__global__ void k_cfl_min(const R* __restrict__ w, size_t plane, int m, int n, int ld, double gamma, double hmin,
                          unsigned long long* __restrict__ out)
{
    double best = INFINITY;
    size_t total = (size_t)m * n;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(idx / n), i = (int)(idx - (size_t)j * n);
        size_t o = (size_t)j * ld + i;
        double rho = (double)w[o], u = (double)w[plane + o], v = (double)w[2 * plane + o], p = (double)w[3 * plane + o];
        double c = sqrt(gamma * p / rho);
        double sigma = fabs(c) + fabs(u) + fabs(v);
        best = fmin(best, hmin / sigma);
    }
    for (int off = 16; off; off >>= 1)
        best = fmin(best, __shfl_xor_sync(0xffffffffu, best, off));
    __shared__ double red[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        red[wid] = best;
    __syncthreads();
    if (wid == 0) {
        best = (lane < (int)(blockDim.x >> 5)) ? red[lane] : INFINITY;
        for (int off = 16; off; off >>= 1)
            best = fmin(best, __shfl_xor_sync(0xffffffffu, best, off));
        if (lane == 0 && !(best != best))
            atomicMin(out, (unsigned long long)__double_as_longlong(best));
    }
}

// True when h is a power of two (then d/h == d*(1/h) exactly).
// The strip kernel's strong-jump threshold of the learned start
// (LEARNED_JUMP2_MIN unless HYDRO_LEARNED_JUMP2 gives another), read once.
inline float learned_jump2()
{
    static const float v = [] {
        const char* e = getenv("HYDRO_LEARNED_JUMP2");
        const float x = e ? (float)atof(e) : LEARNED_JUMP2_MIN;
        return x >= 0.f ? x : LEARNED_JUMP2_MIN;
    }();
    return v;
}

inline bool h_is_pow2(double h)
{
    int e;
    double f = frexp(h, &e);
    return h > 0.0 && f == 0.5;
}

// Gas constants of the step kernels, derived once in FP64 on the host.
template <typename R>
void fill_gas_params(Gas<R>& G, double g, double eps)
{
    gas_fill(G, g, eps);
}

// Conservation sums in FP64: mass, x/y momentum and total energy,
// sum over cells of rho, rho u, rho v, rho E (times the cell area on the
// host).  Deterministic: block b owns the fixed rows b, b + grid, ..., each
// block reduces in a fixed tree, and one warp adds the block partials in
// order, so the result does not depend on scheduling.
template <typename R>
__global__ void k_conserve_partial(const R* __restrict__ w, size_t plane, int m, int n, int ld,
                                   double* __restrict__ partial)
{
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int j = blockIdx.x; j < m; j += gridDim.x)
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const size_t o = (size_t)j * ld + i;
            const double rho = (double)w[o];
            s0 += rho;
            s1 += rho * (double)w[plane + o];
            s2 += rho * (double)w[2 * plane + o];
            s3 += rho * (double)w[4 * plane + o];
        }
    __shared__ double red[4][32];
    for (int off = 16; off; off >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, off);
        s1 += __shfl_down_sync(0xffffffffu, s1, off);
        s2 += __shfl_down_sync(0xffffffffu, s2, off);
        s3 += __shfl_down_sync(0xffffffffu, s3, off);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        red[0][wid] = s0;
        red[1][wid] = s1;
        red[2][wid] = s2;
        red[3][wid] = s3;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int q = 0; q < nw; ++q)
            t += red[threadIdx.x][q];
        partial[(size_t)blockIdx.x * 4 + threadIdx.x] = t;
    }
}

static __global__ void k_conserve_final(const double* __restrict__ partial, int nblocks, double* __restrict__ out)
{
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int b = 0; b < nblocks; ++b)
            t += partial[(size_t)b * 4 + threadIdx.x];
        out[threadIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// the solver
// ---------------------------------------------------------------------------
template <typename R>
class Solver2D : public Solver2DBase {
public:
    int ld = 0;
    size_t plane = 0;
    R* mem = nullptr;
    R* ghost0 = nullptr;
    Ctl* ctl = nullptr;
    double* stage = nullptr;   // FP64 staging, 5 planes of m*n
    unsigned long long* red = nullptr;
    unsigned int* work = nullptr;  // per-launch work counters of the strip kernel
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sms = 148;

    R* W(int b) { return mem + (size_t)b * 13 * plane; }

    // The split scheme's sweep kernel along x (ydir 0) or y (1) for this solver's interface solver.
    using SweepFn = void (*)(const StepArgs<R>);
    SweepFn sweep_kernel(int ydir) const
    {
        using TS = Variants<R>;
        if (rs == HYDRO_SOLVER_G2D)
            return ydir ? k_sweep<R, 1, TS::SJ, TS::SI, TS::SNT, 1> : k_sweep<R, 0, TS::SJ, TS::SI, TS::SNT, 1>;
        return ydir ? k_sweep<R, 1, TS::SJ, TS::SI, TS::SNT, 0> : k_sweep<R, 0, TS::SJ, TS::SI, TS::SNT, 0>;
    }
    R* Sx(int b) { return W(b) + 5 * plane; }
    R* Ty(int b) { return W(b) + 9 * plane; }

    // Tensor map over `planes` consecutive pitched planes starting at base
    // (dims n x m x planes, innermost n), box bw x bh x planes.
    bool encode_planes(CUtensorMap* map, R* base, int planes, int bw, int bh)
    {
        static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
        if (!encode) {
            cudaDriverEntryPointQueryResult q;
            void* fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                    cudaSuccess ||
                q != cudaDriverEntryPointSuccess || !fn) {
                set_error("cuTensorMapEncodeTiled is not available");
                return false;
            }
            encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        }
        const cuuint64_t dims[3] = {(cuuint64_t)n, (cuuint64_t)m, (cuuint64_t)planes};
        const cuuint64_t strides[2] = {(cuuint64_t)ld * sizeof(R), (cuuint64_t)plane * sizeof(R)};
        const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, (cuuint32_t)planes};
        const cuuint32_t estr[3] = {1, 1, 1};
        const CUresult r = encode(map, sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                                  3, (void*)base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
            return false;
        }
        return true;
    }

    int init(int m_, int n_, int form_, int rs_)
    {
        m = m_;
        n = n_;
        form = form_;
        rs = rs_;
        if (rs != HYDRO_SOLVER_Q1D && rs != HYDRO_SOLVER_G2D) {
            set_error("unknown interface solver");
            return -1;
        }
        if (rs == HYDRO_SOLVER_G2D && form == HYDRO_FORM_FP32_LEARNED) {
            set_error("the learned start is built for the quasi-1D interface solver");
            return -1;
        }
        ld = (n + 31) / 32 * 32;
        plane = (size_t)m * ld;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (!cuda_ok(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream")) return -1;
        if (!cuda_ok(cudaEventCreate(&ev0), "event")) return -1;
        if (!cuda_ok(cudaEventCreate(&ev1), "event")) return -1;
        if (!cuda_ok(cudaMalloc(&mem, sizeof(R) * 26 * plane), "state buffers")) return -1;
        if (!cuda_ok(cudaMemset(mem, 0, sizeof(R) * 26 * plane), "state clear")) return -1;
        if (!cuda_ok(cudaMalloc(&ghost0, sizeof(R) * (8 * (size_t)n + 8 * (size_t)m)), "ghost table")) return -1;
        if (!cuda_ok(cudaMalloc(&ctl, sizeof(Ctl)), "control block")) return -1;
        if (!cuda_ok(cudaMalloc(&red, sizeof(unsigned long long)), "reduction")) return -1;
        if (!cuda_ok(cudaMalloc(&work, 3 * sizeof(unsigned int)), "work counters")) return -1;
        using TS = Variants<R>;
        variants = TS::all(form == HYDRO_FORM_FP32_LEARNED, rs);
        if (form == HYDRO_FORM_FP32_LEARNED) {
            if (!cuda_ok(cudaMalloc(&mlp_frag, sizeof(uint32_t) * MLP_NFRAG), "network") ||
                !cuda_ok(cudaMalloc(&mlp_prm, sizeof(float) * MLP_NPARAM), "network") ||
                !cuda_ok(cudaMalloc(&mlp_img, sizeof(MlpShared)), "network"))
                return -1;
        }
        int smem_optin = 0;
        cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        for (auto& v : variants) {
            // the dynamic shared memory a CTA may have next to the kernel's static variables
            cudaFuncAttributes fa;
            if (!cuda_ok(cudaFuncGetAttributes(&fa, v.kern), "kernel attributes"))
                return -1;
            const int avail = smem_optin - (int)fa.sharedSizeBytes;
            if ((int)v.smem > avail) {  // too large for this device: dropped below
                v.tma = 1;
                v.occ = 0;
                continue;
            }
            // variants of one kernel may differ in their shared memory: allow the largest
            size_t smax = v.smem;
            for (const auto& w : variants)
                if (w.kern == v.kern && (int)w.smem <= avail && w.smem > smax)
                    smax = w.smem;
            if (!cuda_ok(cudaFuncSetAttribute(v.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax),
                         "smem attr"))
                return -1;
            // the unified L1/shared storage: the shared memory the variant's CTAs need, the
            // rest L1 (the gathered tiles: MINB CTAs per SM; the strip kernel: its own split;
            // the persistent TMA kernels: all of it)
            if (!v.strip && !v.tma)
                v.carve = carve_for(v.smem + fa.sharedSizeBytes, v.MINB);
            if (!cuda_ok(cudaFuncSetAttribute(v.kern, cudaFuncAttributePreferredSharedMemoryCarveout, v.carve),
                         "carveout attr"))
                return -1;
            if (v.strip) {
                if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v.occ, v.kern, v.NT, v.smem),
                             "occupancy"))
                    return -1;
                continue;  // (occ < 1: dropped below)
            }
            if (v.tma) {
                if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v.occ, v.kern, v.NT, v.smem),
                             "occupancy"))
                    return -1;
                if (v.occ < 1)
                    continue;  // does not fit on an SM: dropped below
                // descriptors of both state buffers: box of 5 value planes x (TJ+4) rows, 8 slope
                // planes x (TJ+2) rows, TI + 2X columns
                const int bw = v.TI + 2 * (16 / (int)sizeof(R));
                for (int b = 0; b < 2; ++b)
                    if (!encode_planes(&v.maps[b].vals, W(b), 5, bw, v.TJ + 4) ||
                        !encode_planes(&v.maps[b].slopes, W(b) + 5 * plane, 8, bw, v.TJ + 2))
                        return -1;
            }
        }
        {
            std::vector<StepVariant<R>> keep;
            for (auto& v : variants)
                if ((!v.tma && !v.strip) || v.occ >= 1)
                    keep.push_back(v);
            variants.swap(keep);
        }
        size_t smem_x = SweepSmem<R, TS::SJ, TS::SI>::bytes(TS::SJ, TS::SI);
        size_t smem_y = SweepSmem<R, TS::SJ, TS::SI>::bytes(TS::SI, TS::SJ);
        if (!cuda_ok(cudaFuncSetAttribute(sweep_kernel(0), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x),
                     "smem attr"))
            return -1;
        if (!cuda_ok(cudaFuncSetAttribute(sweep_kernel(1), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_y),
                     "smem attr"))
            return -1;
        // variant override for profiling: HYDRO_STEP_VARIANT_FP64 / _FP32 / _FP32_LEARNED,
        // else HYDRO_STEP_VARIANT for every form
        const char* fenv = form == HYDRO_FORM_FP64 ? "HYDRO_STEP_VARIANT_FP64"
                           : form == HYDRO_FORM_FP32 ? "HYDRO_STEP_VARIANT_FP32"
                                                     : "HYDRO_STEP_VARIANT_FP32_LEARNED";
        const char* e = getenv(fenv);
        if (!e)
            e = getenv("HYDRO_STEP_VARIANT");
        if (e) {
            int v = atoi(e);
            if (v >= 0 && v < (int)variants.size())
                variant = v;
        }
        return 0;
    }

    uint32_t* mlp_frag = nullptr;
    float* mlp_prm = nullptr;
    MlpShared* mlp_img = nullptr;  // the shared-memory image in global memory
    bool mlp_set = false;

    int set_mlp(const float* params) override
    {
        if (form != HYDRO_FORM_FP32_LEARNED) {
            set_error("set_mlp: the solver is not in the learned form");
            return -1;
        }
        if (!cuda_ok(cudaMemcpyAsync(mlp_prm, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, stream),
                     "network upload"))
            return -1;
        k_mlp_pack<<<(8 * 32 + 4 * 8 * 32 + 4 * 32 + 127) / 128, 128, 0, stream>>>(mlp_prm, mlp_frag);
        k_mlp_image<<<1, 256, 0, stream>>>(mlp_frag, mlp_prm, mlp_img);
        count_launch(2);
        mlp_set = true;
        return cuda_ok(cudaStreamSynchronize(stream), "network pack") ? 0 : -1;
    }

    ~Solver2D() override
    {
        if (stream) cudaStreamSynchronize(stream);
        cudaFree(mlp_frag);
        cudaFree(mlp_prm);
        cudaFree(mlp_img);
        cudaFree(mem);
        cudaFree(ghost0);
        cudaFree(ctl);
        cudaFree(stage);
        cudaFree(red);
        cudaFree(work);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    int grid1d(size_t total) const
    {
        size_t b = (total + 255) / 256;
        size_t cap = (size_t)sms * 8;
        return (int)(b < cap ? (b ? b : 1) : cap);
    }

    // FP64 staging of 5 planes for the host-plane API (upload/download and
    // plot snapshots), allocated on first use: the scheme entry points copy
    // rows through host buffers without it.
    bool ensure_stage()
    {
        return stage || cuda_ok(cudaMalloc(&stage, sizeof(double) * 5 * (size_t)m * n), "staging");
    }

    int upload(const double* rho, const double* u, const double* v, const double* p, const double* E,
               double gamma) override
    {
        if (!ensure_stage())
            return -1;
        size_t mn = (size_t)m * n;
        const double* src[4] = {rho, u, v, p};
        for (int k = 0; k < 4; ++k)
            if (!cuda_ok(cudaMemcpyAsync(stage + k * mn, src[k], sizeof(double) * mn, cudaMemcpyHostToDevice, stream),
                         "upload"))
                return -1;
        if (E) {
            if (!cuda_ok(cudaMemcpyAsync(stage + 4 * mn, E, sizeof(double) * mn, cudaMemcpyHostToDevice, stream), "upload"))
                return -1;
        } else {
            k_energy<<<grid1d(mn), 256, 0, stream>>>(stage, stage + mn, stage + 2 * mn, stage + 3 * mn, stage + 4 * mn,
                                                       mn, gamma);
            count_launch();
        }
        for (int k = 0; k < 5; ++k) {
            k_pack_plane<R><<<grid1d(mn), 256, 0, stream>>>(stage + k * mn, W(0) + k * plane, m, n, ld);
            count_launch();
        }
        // slopes start at zero (the first limiting uses minmod2 and ignores them)
        if (!cuda_ok(cudaMemsetAsync(Sx(0), 0, sizeof(R) * 8 * plane, stream), "clear")) return -1;
        if (!cuda_ok(cudaMemsetAsync(Sx(1), 0, sizeof(R) * 8 * plane, stream), "clear")) return -1;
        cur_w = cur_s = cur_t = 0;
        return cuda_ok(cudaStreamSynchronize(stream), "upload sync") ? 0 : -1;
    }

    // State buffer b into x-major FP64 planes (dst[k] may be null), through
    // the host staging pair like the scheme entry points' rows.
    int download_planes(int b, double* const dst[5])
    {
        std::vector<double*> ptr(5 * (size_t)m);
        double* const* rows[5];
        for (int k = 0; k < 5; ++k) {
            rows[k] = nullptr;
            if (!dst[k])
                continue;
            for (int j = 0; j < m; ++j)
                ptr[(size_t)k * m + j] = dst[k] + (size_t)j * n;
            rows[k] = &ptr[(size_t)k * m];
        }
        return download_rows_staged_from(b, rows);
    }

    int download(double* rho, double* u, double* v, double* p, double* E) override
    {
        double* dst[5] = {rho, u, v, p, E};
        return download_planes(cur_w, dst);
    }

    // A host value in the state's precision, rounded as the FP32 forms' device
    // conversion rounds it (to nearest, a subnormal float result flushed to a
    // zero of its sign: those kernels are compiled with --use_fast_math).
    // (a select, not a branch, so that the packing loops vectorise)
    static R to_state(double x)
    {
        if constexpr (sizeof(R) == 4) {
            const float f = (float)x;
            return fabsf(f) < 1.17549435e-38f ? copysignf(0.f, f) : f;
        } else {
            return x;
        }
    }

    int upload_rows_staged(const double* const* const rows[5]) override
    {
        HostPair* hp = host_pair();
        if (!hp)
            return -1;
        std::lock_guard<std::mutex> guard(hp->lock);
        const size_t row_bytes = sizeof(R) * (size_t)n;
        const int CH = (int)(hp->bytes / row_bytes > 0 ? (hp->bytes / row_bytes < (size_t)m ? hp->bytes / row_bytes : m) : 1);
        bool used[2] = {false, false};
        int b = 0;
        for (int k = 0; k < 5; ++k)
            for (int j0 = 0; j0 < m; j0 += CH) {
                const int j1 = j0 + CH < m ? j0 + CH : m;
                // the copy that last read this buffer is done before it is refilled
                if (used[b] && !cuda_ok(cudaEventSynchronize(hp->ev[b]), "staging wait"))
                    return -1;
                R* dst = static_cast<R*>(hp->buf[b]);
                const double* const* src = rows[k];
                parallel_range(j1 - j0, (size_t)(j1 - j0) * n * (8 + sizeof(R)), [&](int r0, int r1) {
                    for (int r = r0; r < r1; ++r) {
                        const double* sr = src[j0 + r];
                        R* dr = dst + (size_t)r * n;
                        if constexpr (sizeof(R) == 8) {
                            memcpy(dr, sr, row_bytes);
                        } else {
                            for (int i = 0; i < n; ++i)
                                dr[i] = to_state(sr[i]);
                        }
                    }
                });
                if (!cuda_ok(cudaMemcpy2DAsync(W(0) + k * plane + (size_t)j0 * ld, sizeof(R) * ld, dst, row_bytes,
                                               row_bytes, j1 - j0, cudaMemcpyHostToDevice, stream),
                             "upload") ||
                    !cuda_ok(cudaEventRecord(hp->ev[b], stream), "staging event"))
                    return -1;
                used[b] = true;
                b ^= 1;
            }
        // slopes start at zero (the first limiting uses minmod2 and ignores them)
        if (!cuda_ok(cudaMemsetAsync(Sx(0), 0, sizeof(R) * 8 * plane, stream), "clear")) return -1;
        if (!cuda_ok(cudaMemsetAsync(Sx(1), 0, sizeof(R) * 8 * plane, stream), "clear")) return -1;
        cur_w = cur_s = cur_t = 0;
        return cuda_ok(cudaStreamSynchronize(stream), "upload sync") ? 0 : -1;
    }

    int download_rows_staged(double* const* const rows[5]) override { return download_rows_staged_from(cur_w, rows); }

    // State buffer b into the caller's rows (rows[k] may be null: plane k is skipped).
    int download_rows_staged_from(int b, double* const* const rows[5])
    {
        HostPair* hp = host_pair();
        if (!hp)
            return -1;
        std::lock_guard<std::mutex> guard(hp->lock);
        const size_t row_bytes = sizeof(R) * (size_t)n;
        const int CH = (int)(hp->bytes / row_bytes > 0 ? (hp->bytes / row_bytes < (size_t)m ? hp->bytes / row_bytes : m) : 1);
        // the chunks to copy: (plane, first row), planes the caller asked for
        std::vector<std::pair<int, int>> ch;
        for (int k = 0; k < 5; ++k)
            if (rows[k])
                for (int j0 = 0; j0 < m; j0 += CH)
                    ch.push_back({k, j0});
        const int nchunk = (int)ch.size();
        auto issue = [&](int c) -> bool {
            const int k = ch[c].first, j0 = ch[c].second, j1 = j0 + CH < m ? j0 + CH : m, bb = c & 1;
            return cuda_ok(cudaMemcpy2DAsync(hp->buf[bb], row_bytes, W(b) + k * plane + (size_t)j0 * ld,
                                             sizeof(R) * ld, row_bytes, j1 - j0, cudaMemcpyDeviceToHost, stream),
                           "download") &&
                   cuda_ok(cudaEventRecord(hp->ev[bb], stream), "staging event");
        };
        if (nchunk == 0)
            return 0;
        if (!issue(0))
            return -1;
        for (int c = 0; c < nchunk; ++c) {
            // the next block's copy runs while this one is unpacked (its buffer was emptied last turn)
            if (c + 1 < nchunk && !issue(c + 1))
                return -1;
            if (!cuda_ok(cudaEventSynchronize(hp->ev[c & 1]), "download wait"))
                return -1;
            const int k = ch[c].first, j0 = ch[c].second, j1 = j0 + CH < m ? j0 + CH : m;
            const R* srcb = static_cast<const R*>(hp->buf[c & 1]);
            double* const* dst = rows[k];
            parallel_range(j1 - j0, (size_t)(j1 - j0) * n * (8 + sizeof(R)), [&](int r0, int r1) {
                for (int r = r0; r < r1; ++r) {
                    const R* sr = srcb + (size_t)r * n;
                    double* dr = dst[j0 + r];
                    if constexpr (sizeof(R) == 8) {
                        memcpy(dr, sr, row_bytes);
                    } else {
                        for (int i = 0; i < n; ++i)
                            dr[i] = (double)sr[i];
                    }
                }
            });
        }
        return 0;
    }

    int upload_rows(const double* const* const rows[5]) override
    {
        // one element per thread: host-memory latency is hidden by having every load in flight
        const dim3 grid((n + 255) / 256, m);
        for (int k = 0; k < 5; ++k) {
            k_gather_rows<R><<<grid, 256, 0, stream>>>(rows[k], W(0) + k * plane, m, n, ld);
            count_launch();
        }
        if (!cuda_ok(cudaMemsetAsync(Sx(0), 0, sizeof(R) * 8 * plane, stream), "clear")) return -1;
        if (!cuda_ok(cudaMemsetAsync(Sx(1), 0, sizeof(R) * 8 * plane, stream), "clear")) return -1;
        cur_w = cur_s = cur_t = 0;
        return cuda_ok(cudaStreamSynchronize(stream), "row upload") ? 0 : -1;
    }

    int download_rows(double* const* const rows[5]) override
    {
        const dim3 grid((n + 255) / 256, m);
        for (int k = 0; k < 5; ++k) {
            k_scatter_rows<R><<<grid, 256, 0, stream>>>(W(cur_w) + k * plane, rows[k], m, n, ld);
            count_launch();
        }
        return cuda_ok(cudaStreamSynchronize(stream), "row download") ? 0 : -1;
    }

    int conservation(double hx, double hy, double* out4) override
    {
        constexpr int NB = 512;  // fixed block count: the summation order depends only on the grid
        double* buf = nullptr;
        if (!cuda_ok(cudaMalloc(&buf, sizeof(double) * (4 * NB + 4)), "conservation buffer"))
            return -1;
        k_conserve_partial<R><<<NB, 256, 0, stream>>>(W(cur_w), plane, m, n, ld, buf);
        k_conserve_final<<<1, 32, 0, stream>>>(buf, NB, buf + 4 * NB);
        count_launch(2);
        double h[4];
        cudaMemcpyAsync(h, buf + 4 * NB, sizeof(h), cudaMemcpyDeviceToHost, stream);
        const bool ok = cuda_ok(cudaStreamSynchronize(stream), "conservation sums");
        cudaFree(buf);
        if (!ok)
            return -1;
        for (int k = 0; k < 4; ++k)
            out4[k] = h[k] * hx * hy;
        return 0;
    }

    double cfl_hsmax(double gamma, double hmin)
    {
        unsigned long long init = 0x7ff0000000000000ull;  // +inf
        cudaMemcpyAsync(red, &init, sizeof(init), cudaMemcpyHostToDevice, stream);
        k_cfl_min<R><<<grid1d((size_t)m * n), 256, 0, stream>>>(W(cur_w), plane, m, n, ld, gamma, hmin, red);
        count_launch();
        unsigned long long bits = 0;
        cudaMemcpyAsync(&bits, red, sizeof(bits), cudaMemcpyDeviceToHost, stream);
        cudaStreamSynchronize(stream);
        double r;
        memcpy(&r, &bits, sizeof(r));
        return r;
    }

    int cur_w = 0, cur_s = 0, cur_t = 0;
    std::vector<StepVariant<R>> variants;
    int variant = 0;

    int num_variants() const override { return (int)variants.size(); }
    int set_variant(int v) override
    {
        if (v < 0 || v >= (int)variants.size()) {
            set_error("no such kernel variant");
            return -1;
        }
        variant = v;
        return 0;
    }
    int get_variant() const override { return variant; }
    void variant_shape(int v, int* shape) const override
    {
        const StepVariant<R>& s = variants[v];
        shape[0] = s.TJ;
        shape[1] = s.TI;
        shape[2] = s.NT;
        shape[3] = s.MINB;
        shape[4] = s.strip ? 3 : s.tma;
    }

    // Times every variant on `steps` steps of the uploaded state (restored
    // afterwards) and keeps the fastest.  Returns its index.
    int autotune(const RunConfig& rc, int steps, float* times_ms) override
    {
        size_t bytes = sizeof(R) * 5 * plane;
        R* backup = nullptr;
        if (!cuda_ok(cudaMalloc(&backup, bytes), "autotune backup")) return -1;
        int w0 = cur_w;
        cudaMemcpyAsync(backup, W(w0), bytes, cudaMemcpyDeviceToDevice, stream);
        RunConfig r2 = rc;
        r2.N = steps;
        r2.t_all = INFINITY;
        double tp[2] = {0.0, INFINITY};
        int best = 0;
        float best_ms = 1e30f;
        for (int v = 0; v < (int)variants.size(); ++v) {
            variant = v;
            cudaMemcpyAsync(W(w0), backup, bytes, cudaMemcpyDeviceToDevice, stream);
            cur_w = w0;
            hydro_run_info info;
            int nt;
            // a variant that fails to run is timed as infinitely slow (and its launch error is
            // cleared, so that it is not reported by the next variant's run)
            const bool failed = run(r2, 0, 0, tp, 2, 2, nullptr, &info, &nt) != 0;
            if (failed)
                cudaGetLastError();
            float ms = failed ? 3e38f : (float)info.gpu_ms;
            if (times_ms)
                times_ms[v] = ms;
            if (ms < best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        cudaMemcpyAsync(W(w0), backup, bytes, cudaMemcpyDeviceToDevice, stream);
        cur_w = w0;
        cudaStreamSynchronize(stream);
        cudaFree(backup);
        variant = best;
        return best;
    }

    void fill_gas(Gas<R>& G, double g, double eps) { fill_gas_params(G, g, eps); }

    static bool is_pow2(double h) { return h_is_pow2(h); }

    int run(const RunConfig& rc, int split, int stats, const double* time_plot, int N_plot, int N_T,
            double** snap_out, hydro_run_info* info, int* final_nt) override
    {
        memset(info, 0, sizeof(*info));
        // ghost table for the fixed boundary, from the initial state
        {
            int t = (m > n ? m : n);
            k_ghost0<R><<<(t + 255) / 256, 256, 0, stream>>>(W(cur_w), plane, m, n, ld, ghost0);
            count_launch();
        }
        double hs = cfl_hsmax(rc.gamma, fmin(rc.hx, rc.hy));
        RunPlan plan = plan_run(rc, hs, split, time_plot, N_plot, N_T);
        if (!cuda_ok(cudaMemsetAsync(ctl, 0, sizeof(Ctl), stream), "ctl clear")) return -1;
        if (!cuda_ok(cudaMemsetAsync(work, 0, 3 * sizeof(unsigned int), stream), "work counters")) return -1;

        StepArgs<R> a;
        memset(&a, 0, sizeof(a));
        a.m = m;
        a.n = n;
        a.ld = ld;
        a.plane = plane;
        a.ghost0 = ghost0;
        fill_gas(a.G, rc.gamma, rc.eps);
        a.hx = (R)rc.hx;
        a.hy = (R)rc.hy;
        a.hhx = (R)(0.5 * rc.hx);
        a.hhy = (R)(0.5 * rc.hy);
        a.pow2_x = is_pow2(rc.hx);
        a.pow2_y = is_pow2(rc.hy);
        a.inv_hx = (R)(1.0 / rc.hx);
        a.inv_hy = (R)(1.0 / rc.hy);
        a.alpha = (R)rc.alpha;
        a.bx = rc.bx;
        a.by = rc.by;
        a.ctl = ctl;
        a.stats = stats;
        if (form == HYDRO_FORM_FP32_LEARNED) {
            if (!mlp_set) {
                set_error("learned form: no network weights installed (hydro2d_set_mlp)");
                return -1;
            }
            a.mlp_frag = mlp_frag;
            a.mlp_prm = mlp_prm;
            a.mlp_img = mlp_img;
        }

        using TS = Variants<R>;
        const StepVariant<R>& V = variants[variant];
        dim3 gu((n + V.TI - 1) / V.TI, (m + V.TJ - 1) / V.TJ);
        dim3 gs((n + TS::SI - 1) / TS::SI, (m + TS::SJ - 1) / TS::SJ);
        size_t smem_x = SweepSmem<R, TS::SJ, TS::SI>::bytes(TS::SJ, TS::SI);
        size_t smem_y = SweepSmem<R, TS::SJ, TS::SI>::bytes(TS::SI, TS::SJ);

        // snapshots: pinned staging per requested snapshot
        std::vector<double*> snap_dev;
        size_t mn = (size_t)m * n;
        size_t snap_next = 0;
        int wbuf_at_seq0 = cur_w;
        std::vector<int> wbuf_before(plan.sweeps.size() + 1);

        cudaEventRecord(ev0, stream);
        // slopes are scratch between runs (the first limiting of a run ignores
        // them), so they restart in the state's own buffer, as the TMA boxes expect
        int w = cur_w, s = cur_w, t = cur_w;
        const int ntiles_u = ((n + V.TI - 1) / V.TI) * ((m + V.TJ - 1) / V.TJ);
        const int grid_tma = V.tma ? (ntiles_u < sms * V.occ ? ntiles_u : sms * V.occ) : 0;
        for (size_t q = 0; q < plan.sweeps.size(); ++q) {
            const SweepRec& r = plan.sweeps[q];
            int seq = (int)q + 1;
            while (snap_next < plan.snaps.size() && plan.snaps[snap_next].seq == seq) {
                // record the state in front of this launch
                if (snap_out && snap_out[plan.snaps[snap_next].nt]) {
                    double* dst[5];
                    for (int k = 0; k < 5; ++k)
                        dst[k] = snap_out[plan.snaps[snap_next].nt] + k * mn;
                    // ordered on the stream: the state is exactly the one before launch seq
                    if (download_planes(w, dst)) return -1;
                }
                snap_next++;
            }
            wbuf_before[q] = w;
            a.seq = seq;
            a.find_x = r.find_x;
            a.find_y = r.find_y;
            a.tau = (R)r.tau_face;
            a.htau = (R)(0.5 * r.tau_face);
            a.nu = (R)r.fac_x;
            a.mu = (R)r.fac_y;
            a.src_w = W(w);
            a.dst_w = W(w ^ 1);
            if (r.dir == 0) {
                a.src_s = Sx(s); a.dst_s = Sx(s ^ 1);
                a.src_t = Ty(t); a.dst_t = Ty(t ^ 1);
                if (V.strip) {
                    StripArgs sa;
                    sa.work = work;
                    sa.seg = V.TJ;
                    sa.mlp_min = V.mlp_min;
                    sa.mlp_jump2 = learned_jump2();
                    sa.mlp_global = V.mlp_global;
                    void* args[] = {(void*)&a, (void*)&sa};
                    // variants of one kernel differ in their L1/shared split: set per launch
                    cudaLaunchConfig_t lc;
                    memset(&lc, 0, sizeof(lc));
                    lc.gridDim = dim3(sms * V.occ);
                    lc.blockDim = dim3(V.NT);
                    lc.dynamicSmemBytes = V.smem;
                    lc.stream = stream;
                    cudaLaunchAttribute at[1];
                    at[0].id = cudaLaunchAttributePreferredSharedMemoryCarveout;
                    at[0].val.sharedMemCarveout = (unsigned)V.carve;
                    lc.attrs = at;
                    lc.numAttrs = 1;
                    if (!cuda_ok(cudaLaunchKernelExC(&lc, V.kern, args), "step launch"))
                        return -1;
                } else if (V.tma) {
                    // the boxes read the state buffer w, whose slope planes are s = t = w here
                    StepMaps mp = V.maps[w];
                    void* args[] = {(void*)&a, (void*)&mp};
                    if (!cuda_ok(cudaLaunchKernel(V.kern, dim3(grid_tma), dim3(V.NT), args, V.smem, stream),
                                 "step launch"))
                        return -1;
                } else {
                    void* args[] = {(void*)&a};
                    if (!cuda_ok(cudaLaunchKernel(V.kern, gu, dim3(V.NT), args, V.smem, stream), "step launch"))
                        return -1;
                }
                s ^= 1;
                t ^= 1;
            } else if (r.dir == 1) {
                a.src_s = Sx(s); a.dst_s = Sx(s ^ 1);
                a.src_t = Ty(t); a.dst_t = Ty(t);
                sweep_kernel(0)<<<gs, TS::SNT, smem_x, stream>>>(a);
                s ^= 1;
            } else {
                a.src_s = Sx(s); a.dst_s = Sx(s);
                a.src_t = Ty(t); a.dst_t = Ty(t ^ 1);
                sweep_kernel(1)<<<gs, TS::SNT, smem_y, stream>>>(a);
                t ^= 1;
            }
            count_launch();
            w ^= 1;
            if (!cuda_ok(cudaGetLastError(), "step launch")) return -1;
        }
        wbuf_before[plan.sweeps.size()] = w;
        cudaEventRecord(ev1, stream);
        Ctl hc;
        if (!cuda_ok(cudaMemcpyAsync(&hc, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream), "ctl read")) return -1;
        if (!cuda_ok(cudaStreamSynchronize(stream), "time loop")) return -1;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        (void)wbuf_at_seq0;
        if (hc.wait_err) {
            set_error(hc.wait_err == 2 ? "the step kernel's TMA descriptor check failed; the run is invalid"
                                       : "a bounded TMA wait in the step kernel gave up; the run is invalid");
            return -1;
        }

        // resolve the outcome
        int nsw = (int)plan.sweeps.size();
        int halt_q = 0, kind = 0;  // 1-based launch that halted the run
        if (hc.halted_seq) {
            halt_q = hc.halted_seq;
            kind = hc.halt_kind;
        } else if (nsw > 0) {
            int ls = nsw % 3;
            int d = halt_decision(hc.key[ls][0], hc.key[ls][1], hc.upd_bad[ls]);
            if (d) {
                halt_q = nsw;
                kind = d;
            }
        }
        int final_w;
        if (halt_q) {
            const SweepRec& r = plan.sweeps[halt_q - 1];
            int hs3 = halt_q % 3;
            info->error_code_x = (int)(hc.key[hs3][0] & 3ull);
            info->error_code_y = (int)(hc.key[hs3][1] & 3ull);
            info->halted = kind;
            info->k_out = r.k;
            info->time = (kind == 1) ? r.time_before : r.time_after;
            info->tau = r.tau_face;
            final_w = (kind == 1) ? wbuf_before[halt_q - 1] : wbuf_before[halt_q];
            *final_nt = r.nt;
            info->sweeps_launched = nsw;
            int kept = (kind == 1) ? halt_q - 1 : halt_q;
            info->steps_done = kept;
        } else {
            info->k_out = plan.end_k;
            info->time = plan.end_time;
            info->tau = plan.end_tau;
            final_w = wbuf_before[nsw];
            *final_nt = plan.end_nt;
            info->sweeps_launched = nsw;
            info->steps_done = nsw;
        }
        info->gpu_ms = ms;
        info->newton_faces = hc.newton_faces;
        info->newton_iters = hc.newton_iters;
        info->newton_fallbacks = hc.newton_fallbacks;
        cur_w = final_w;
        // slopes are scratch after the run (the reference frees them)
        cur_s = s;
        cur_t = t;
        return 0;
    }
};

}  // namespace hydro
