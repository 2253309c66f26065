// batch.cu -- many independent 2D problems of uneven grid size advanced together.
//
// Every problem keeps its own two states (13 pitched planes each), boundary
// table, time step and halting control block.  The planes are pooled: plane k
// of state s of every problem lies in one array of `pool` elements, problem p
// at offset off[p], so the stride between a problem's planes is the same for
// all problems.  All work units of all problems form one flat list; a unit is
// a tile running exactly the per-tile code of the one-problem FP32 step
// (unsplit_tile), or, for the strip shapes, a (strip, run of rows) running the
// one-problem strip kernel's per-unit march (strip_unit).  Each problem's
// result is therefore a one-problem FP32 run of the same data (to the last bit
// where the same compiled instance runs; separately compiled kernels may
// contract multiply-adds differently under fast math, a difference at FP32
// rounding).  There is no reference counterpart: the reference advances one grid
// per process (grp_solver_2D_EUL_source.c:146-286).
//
// Schedules (picked by hydro_batch_autotune from timings on the real batch):
//   0  persistent, static round robin over the problem-major tile order
//   1  persistent, static round robin over a largest-problem-first order
//   2  persistent, dynamic (one atomic work counter per step), problem-major
//   3  persistent, dynamic, largest-first
//   4  a CUDA graph of one launch per step, one CTA per tile (strip shapes:
//      the CTAs that fit at once, taking units from the step's counter)
// "Persistent" is ONE cooperative kernel for all steps with a grid barrier
// between steps; its wait is bounded by the global timer (the barrier gives
// up, flags an error and every CTA returns).  The launch is captured in a
// CUDA graph.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "solver2d_impl.cuh"

namespace hydro {

// Step arguments of a problem come in BATCH_VERSIONS ready-made versions, so a
// tile only copies them: (step & 1) * 3 + step % 3 for steps >= 2 (buffer
// parity and error-key slot), and 6 for step 1 (first limiting: minmod2).
constexpr int BATCH_VERSIONS = 7;
__host__ __device__ inline int batch_version(int step) { return step == 1 ? 6 : (step & 1) * 3 + step % 3; }

struct BatchDev {
    const StepArgs<float>* args;  // [nprob][BATCH_VERSIONS]
    Ctl* ctl;                     // [nprob]
    const int* tile_prob;         // [ntiles] problem of each flat tile
    const int* tile_local;        // [ntiles] tile index within its problem (y-tiles fastest)
    const int* order;             // [ntiles] processing order of the flat tiles
    const int* tiles_y;           // [nprob] tiles along y (the contiguous axis)
    const int4* rec;              // [ntiles] per processing position k: problem, tile within it,
                                  // tiles along y of the problem (one load per tile)
    int ntiles, nprob, steps, dynamic, stats;
    unsigned int* work;           // [2] per-step work counters (dynamic schedules)
    unsigned int* bar_count;      // grid barrier: arrivals
    unsigned int* bar_gen;        // grid barrier: generation
    int* bar_err;                 // set when a barrier wait gave up
    unsigned long long wait_ns;   // barrier wait limit
    Gas<float> G;                 // gas constants (one gas for the whole batch): read from the
                                  // kernel's parameter space, not from the per-tile copy
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier of a cooperative launch (all CTAs co-resident).  Returns
// false if some CTA's wait ran out of time; the caller then leaves the loop.
__device__ __forceinline__ bool grid_barrier(const BatchDev& B)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = B.bar_gen;
        const unsigned int g = *gen;
        __threadfence();
        if (atomicAdd(B.bar_count, 1u) == gridDim.x - 1) {
            *B.bar_count = 0u;
            __threadfence();
            atomicAdd(B.bar_gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            // the timer is read every 1024 polls, every poll under a limit of 100 us
            const unsigned int mask = B.wait_ns < 100000ull ? 0u : 1023u;
            unsigned int polls = 0;
            while (*gen == g) {
                __nanosleep(100);
                // the poll count also ends the wait should the timer not advance
                if ((++polls & mask) == 0u && (global_ns() - t0 > B.wait_ns || polls > (1u << 30))) {
                    atomicExch(B.bar_err, 1);
                    break;
                }
                if (*((volatile int*)B.bar_err))
                    break;
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *((volatile int*)B.bar_err) == 0;
}

// Loads the step arguments of the tile at processing position k into shared
// memory and applies the one-problem kernel's halting protocol (halt_prologue)
// for its problem.  Returns false (uniformly over the block) when the problem
// has halted.  One thread reads the control block and decides; the block
// copies the arguments word by word meanwhile (also for a halted problem: its
// arguments exist, and the copy is not used) and one barrier publishes both.
__device__ __forceinline__ bool batch_tile_args(const BatchDev& B, int k, int step, StepArgs<float>& sa, int& lt,
                                                int& nty)
{
    __shared__ int s_ok;
    const int4 r = B.rec[k];
    const int p = r.x;
    lt = r.y;
    nty = r.z;
    if (threadIdx.x == 0) {
        volatile Ctl* c = B.ctl + p;
        bool ok = c->halted_seq == 0;
        if (ok && step > 1) {
            const int ps = (step - 1) % 3;
            const int d = halt_decision(c->key[ps][0], c->key[ps][1], c->upd_bad[ps]);
            if (d) {
                ok = false;
                if (lt == 0) {
                    c->halt_kind = d;
                    c->halted_seq = step - 1;
                }
            }
        }
        if (ok && lt == 0) {
            const int ns = (step + 1) % 3;
            c->key[ns][0] = 0ull;
            c->key[ns][1] = 0ull;
            c->upd_bad[ns] = 0u;
        }
        s_ok = ok ? 1 : 0;
    }
    constexpr int WORDS = (int)(sizeof(StepArgs<float>) / 4);
    static_assert(sizeof(StepArgs<float>) % 4 == 0, "word copy");
    const int* src = reinterpret_cast<const int*>(B.args + (size_t)p * BATCH_VERSIONS + batch_version(step));
    int* dst = reinterpret_cast<int*>(&sa);
    for (int w = threadIdx.x; w < WORDS; w += blockDim.x)
        dst[w] = src[w];
    __syncthreads();
    const bool ok = s_ok != 0;
    // a skipped tile: every thread has read s_ok before the next tile's decision
    // overwrites it (a computed tile's own barriers do this)
    if (!ok)
        __syncthreads();
    return ok;
}

// The tile at processing position k.
template <int TJ, int TI, int NT>
__device__ __forceinline__ void batch_tile(const BatchDev& B, int k, int step, StepArgs<float>& sa, unsigned char* smem,
                                           const MlpShared& M, bool last_tile = false)
{
    int lt, nty;
    if (batch_tile_args(B, k, step, sa, lt, nty))
        unsplit_tile<float, TJ, TI, NT, false>(sa, B.G, (lt % nty) * TI, (lt / nty) * TJ, smem, M, last_tile);
}

// ONE cooperative kernel for all steps of all problems.  The schedule only
// decides which tile comes next; the tile code has a single call site, so
// both schedules run the same compiled instructions.
template <int TJ, int TI, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_batch_persistent(const __grid_constant__ BatchDev B)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ StepArgs<float> sa;
    __shared__ int s_k;
    const MlpShared& M = *reinterpret_cast<const MlpShared*>(smem_raw);  // not read by the plain form
    for (int step = 1; step <= B.steps; ++step) {
        unsigned int* ctr = B.work + (step & 1);
        // next flat tile: the CTA's own stride (static) or the step's shared counter (dynamic)
        auto next = [&](int k) -> int {
            if (!B.dynamic)
                return k + (int)gridDim.x;
            if (threadIdx.x == 0)
                s_k = (int)atomicAdd(ctr, 1u);
            __syncthreads();
            const int r = s_k;
            __syncthreads();
            return r;
        };
        for (int k = B.dynamic ? next(0) : (int)blockIdx.x; k < B.ntiles; k = next(k))
            batch_tile<TJ, TI, NT>(B, k, step, sa, smem_raw, M);
        // the counter of the next step was last used two steps ago: reset it
        if (B.dynamic && blockIdx.x == 0 && threadIdx.x == 0)
            B.work[(step + 1) & 1] = 0u;
        if (!grid_barrier(B))
            return;
    }
}

// One step of all problems, one CTA per tile (the per-step graph schedule).
template <int TJ, int TI, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_batch_step(const __grid_constant__ BatchDev B, int step)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ StepArgs<float> sa;
    const MlpShared& M = *reinterpret_cast<const MlpShared*>(smem_raw);
    batch_tile<TJ, TI, NT>(B, blockIdx.x, step, sa, smem_raw, M, true);
}

// ---------------------------------------------------------------------------
// strip shapes: the one-grid strip kernel's per-unit march (strip_unit), a
// unit being (problem, strip of 60 columns, SEG rows)
// ---------------------------------------------------------------------------
// Per problem, what a strip unit needs beyond the batch's common arguments
// (56 B, so that the arguments of BATCH_STRIP_MAX problems fit the kernel's
// parameter space, from which a warp-uniform problem index reads them).
constexpr int BATCH_STRIP_MAX = 576;
struct BatchStripProb {
    unsigned off64;  // element offset of the problem's planes within each plane of the pool, / 64
    unsigned spare;
    unsigned goff;   // element offset of its boundary table
    int m, n, ld;
    float tau, hx, hy, inv_hx, inv_hy, nu, mu;
    int pow2;  // bit 0: h_x is a power of two, bit 1: h_y
};
static_assert(sizeof(BatchStripProb) == 56, "per-problem strip arguments");

struct BatchStripDev {
    BatchDev B;
    float* mem;          // plane k of state s of every problem starts at mem + (13 s + k) pool
    size_t pool;
    const float* ghost;
    float alpha;
    int bx, by;
    BatchStripProb P[BATCH_STRIP_MAX];
};
static_assert(sizeof(BatchStripDev) <= 32764, "kernel parameter space");

// The members of StepArgs<float> that strip_unit reads, for one problem and step.
struct BatchStripView {
    int m, n, ld;
    size_t plane;
    const float* src_w;
    float* dst_w;
    const float* src_s;
    float* dst_s;
    const float* src_t;
    float* dst_t;
    const float* ghost0;
    float tau, htau, hx, hy, hhx, hhy, inv_hx, inv_hy;
    int pow2_x, pow2_y;
    float nu, mu, alpha;
    int bx, by, find_x, find_y;
    Ctl* ctl;
    int seq, stats;
};

// One unit e of the flat unit list at step `step` (warp-collective): the
// problem's halting protocol (as batch_tile_args), then strip_unit.
template <int SEG>
__device__ __forceinline__ void batch_strip_unit(const BatchStripDev& D, int e, int step, float* q, int* stats3)
{
    const BatchDev& B = D.B;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // the unit's problem and local index, warp-uniform by construction
    const int p = (int)__reduce_max_sync(FULL, (unsigned)B.tile_prob[e]);
    const int lt = (int)__reduce_max_sync(FULL, (unsigned)B.tile_local[e]);
    volatile Ctl* c = B.ctl + p;
    bool ok = c->halted_seq == 0;
    if (ok && step > 1) {
        const int ps = (step - 1) % 3;
        const int d = halt_decision(c->key[ps][0], c->key[ps][1], c->upd_bad[ps]);
        if (d) {
            ok = false;
            if (lt == 0 && lane == 0) {
                c->halt_kind = d;
                c->halted_seq = step - 1;
            }
        }
    }
    if (!ok)
        return;
    if (lt == 0 && lane == 0) {
        const int ns = (step + 1) % 3;
        c->key[ns][0] = 0ull;
        c->key[ns][1] = 0ull;
        c->upd_bad[ns] = 0u;
    }
    const BatchStripProb& P = D.P[p];
    BatchStripView a;
    a.m = P.m;
    a.n = P.n;
    a.ld = P.ld;
    a.plane = D.pool;
    // odd steps read state 0 and write state 1, even steps the reverse
    const size_t o = (size_t)P.off64 * 64;
    float* W0 = D.mem + ((step & 1) ? 0 : 13 * D.pool) + o;
    float* W1 = D.mem + ((step & 1) ? 13 * D.pool : 0) + o;
    a.src_w = W0;
    a.dst_w = W1;
    a.src_s = W0 + 5 * a.plane;
    a.dst_s = W1 + 5 * a.plane;
    a.src_t = W0 + 9 * a.plane;
    a.dst_t = W1 + 9 * a.plane;
    a.ghost0 = D.ghost + P.goff;
    a.tau = P.tau;
    a.htau = 0.5f * P.tau;
    a.hx = P.hx;
    a.hy = P.hy;
    a.hhx = 0.5f * P.hx;
    a.hhy = 0.5f * P.hy;
    a.inv_hx = P.inv_hx;
    a.inv_hy = P.inv_hy;
    a.pow2_x = P.pow2 & 1;
    a.pow2_y = (P.pow2 >> 1) & 1;
    a.nu = P.nu;
    a.mu = P.mu;
    a.alpha = D.alpha;
    a.bx = D.bx;
    a.by = D.by;
    a.find_x = a.find_y = (step > 1);
    a.ctl = B.ctl + p;
    a.seq = step;
    a.stats = B.stats;
    const int nstrip = (a.n + STRIP_W - 1) / STRIP_W;
    const int seg = lt / nstrip, strip = lt - seg * nstrip;
    const int r0 = seg * SEG;
    unsigned bad = 0;
    strip_unit<false>(a, &B.G, strip * STRIP_W, r0, (r0 + SEG < a.m) ? r0 + SEG : a.m, q, nullptr, STRIP_MLP_MIN,
                      LEARNED_JUMP2_MIN, stats3, bad);
    strip_report(a.ctl, step % 3, B.stats, stats3, bad);
}

// ONE cooperative kernel for all steps of all problems, strip units; warps
// take units by a static stride or from the step's counter (one call site of
// the unit code for both).
template <int NW, int SEG>
__global__ void __launch_bounds__(NW * 32, 1) k_batch_strip_persistent(const __grid_constant__ BatchStripDev D)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const BatchDev& B = D.B;
    const unsigned FULL = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* q = reinterpret_cast<float*>(smem_raw + warp * StripSmem<NW, false>::q_bytes);
    int stats3[3] = {0, 0, 0};
    const int gw = blockIdx.x * NW + warp, nw = gridDim.x * NW;
    for (int step = 1; step <= B.steps; ++step) {
        unsigned int* ctr = B.work + (step & 1);
        int k = gw;
        for (;;) {
            if (B.dynamic) {
                int t = 0;
                if (lane == 0)
                    t = (int)atomicAdd(ctr, 1u);
                k = __shfl_sync(FULL, t, 0);
            }
            if (k >= B.ntiles)
                break;
            batch_strip_unit<SEG>(D, B.order[k], step, q, stats3);
            k += nw;
        }
        // the counter of the next step was last used two steps ago: reset it
        if (B.dynamic && blockIdx.x == 0 && threadIdx.x == 0)
            B.work[(step + 1) & 1] = 0u;
        if (!grid_barrier(B))
            return;
    }
}

// One step of all problems, strip units from the step's counter (the per-step
// graph schedule; a grid of the CTAs that fit at once).
template <int NW, int SEG>
__global__ void __launch_bounds__(NW * 32, 1) k_batch_strip_step(const __grid_constant__ BatchStripDev D, int step)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const BatchDev& B = D.B;
    const unsigned FULL = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* q = reinterpret_cast<float*>(smem_raw + warp * StripSmem<NW, false>::q_bytes);
    int stats3[3] = {0, 0, 0};
    unsigned int* ctr = B.work + (step & 1);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        B.work[(step + 1) & 1] = 0u;  // the next launch's counter (this one's was cleared by the previous launch)
    for (;;) {
        int k = 0;
        if (lane == 0)
            k = (int)atomicAdd(ctr, 1u);
        k = __shfl_sync(FULL, k, 0);
        if (k >= B.ntiles)
            break;
        batch_strip_unit<SEG>(D, B.order[k], step, q, stats3);
    }
}

struct BatchShape {
    int TJ, TI, NT, MINB;  // strip shapes: TJ rows per unit, TI = STRIP_W columns
    size_t smem;
    const void* persistent;
    const void* step;
    int strip;  // 1: strip units (BatchStripDev arguments)
    int carve;  // shared-memory carveout, percent
};

template <int TJ, int TI, int NT, int MINB>
BatchShape batch_shape()
{
    return BatchShape{TJ, TI, NT, MINB, UnsplitSmem<float, TJ, TI>::bytes,
                      (const void*)k_batch_persistent<TJ, TI, NT, MINB>, (const void*)k_batch_step<TJ, TI, NT, MINB>,
                      0, 100};
}

template <int NW, int SEG>
BatchShape batch_strip_shape()
{
    // the smallest shared-memory configuration that holds two CTAs (64 KB);
    // the rest of the unified storage is L1 for the strip code's spills
    return BatchShape{SEG, STRIP_W, NW * 32, 1, StripSmem<NW, false>::bytes,
                      (const void*)k_batch_strip_persistent<NW, SEG>, (const void*)k_batch_strip_step<NW, SEG>, 1, 28};
}

static const std::vector<BatchShape>& batch_shapes()
{
    static const std::vector<BatchShape> s = {batch_shape<32, 32, 512, 1>(), batch_shape<8, 32, 256, 3>(),
                                              batch_shape<16, 16, 256, 4>(), batch_strip_shape<4, 16>(),
                                              batch_strip_shape<4, 32>()};
    return s;
}

constexpr int BATCH_SCHEDULES = 5;

}  // namespace hydro

using namespace hydro;

struct hydro_batch {
    int nprob = 0;
    std::vector<int> m, n, ld;
    std::vector<size_t> off, goff;  // element offsets of each problem's state and boundary table
    float* mem = nullptr;
    float* ghost = nullptr;
    Ctl* ctl = nullptr;
    StepArgs<float>* args = nullptr;
    int* tables = nullptr;
    size_t tables_cap = 0;
    int4* rec = nullptr;
    size_t rec_cap = 0;
    unsigned int* sync = nullptr;  // work[2], bar_count, bar_gen, bar_err
    double* stage = nullptr;
    unsigned long long* red = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int shape = 0, schedule = 0, sms = 148;
    double wait_s = 5.0;
    std::vector<double> tau;
    std::vector<int> final_buf, halted_kind, halted_step;
    std::vector<BatchStripProb> sprob;  // per-problem arguments of the strip shapes

    size_t pool = 0;  // elements of one plane of all problems: plane k of state s of problem p
                      // starts at mem + (13 s + k) pool + off[p]
    float* W(int p, int buf) { return mem + (size_t)buf * 13 * pool + off[p]; }
    size_t plane(int) const { return pool; }  // the stride between a problem's planes
    int grid1d(size_t total) const
    {
        size_t b = (total + 255) / 256, cap = (size_t)sms * 8;
        return (int)(b < cap ? (b ? b : 1) : cap);
    }
    ~hydro_batch()
    {
        if (stream)
            cudaStreamSynchronize(stream);
        cudaFree(mem);
        cudaFree(ghost);
        cudaFree(ctl);
        cudaFree(args);
        cudaFree(tables);
        cudaFree(rec);
        cudaFree(sync);
        cudaFree(stage);
        cudaFree(red);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
    }
};

// Host side of one run: per-problem plans, step arguments and tile tables.
static int batch_prepare(hydro_batch* b, const double* cfg, int ncfg, int steps, int stats, const BatchShape& S,
                         int schedule, int* ntiles)
{
    const int np = b->nprob;
    RunConfig rc = run_config_from(cfg, ncfg);
    rc.N = steps;
    rc.t_all = INFINITY;  // fixed step count
    std::vector<StepArgs<float>> args(BATCH_VERSIONS * (size_t)np);
    b->tau.assign(np, 0.0);
    b->sprob.assign(np, BatchStripProb{});
    for (int p = 0; p < np; ++p) {
        const int m = b->m[p], n = b->n[p], ld = b->ld[p];
        const size_t plane = b->plane(p);
        RunConfig r = rc;
        r.hx = 1.0 / m;
        r.hy = 1.0 / n;
        float* g0 = b->ghost + b->goff[p];
        k_ghost0<float><<<(std::max(m, n) + 255) / 256, 256, 0, b->stream>>>(b->W(p, 0), plane, m, n, ld, g0);
        count_launch();
        unsigned long long init = 0x7ff0000000000000ull, bits = 0;
        cudaMemcpyAsync(b->red, &init, sizeof(init), cudaMemcpyHostToDevice, b->stream);
        k_cfl_min<float><<<b->grid1d((size_t)m * n), 256, 0, b->stream>>>(b->W(p, 0), plane, m, n, ld, r.gamma,
                                                                          fmin(r.hx, r.hy), b->red);
        count_launch();
        cudaMemcpyAsync(&bits, b->red, sizeof(bits), cudaMemcpyDeviceToHost, b->stream);
        if (!cuda_ok(cudaStreamSynchronize(b->stream), "batch CFL reduction"))
            return -1;
        double hs;
        memcpy(&hs, &bits, sizeof(hs));
        const double tp[2] = {0.0, INFINITY};
        RunPlan plan = plan_run(r, hs, 0, tp, 2, 2);
        if ((int)plan.sweeps.size() != steps) {
            set_error("batch: a problem's time step is below eps or not finite");
            return -1;
        }
        const SweepRec& r0 = plan.sweeps[0];
        for (const SweepRec& q : plan.sweeps)
            if (q.tau_face != r0.tau_face || q.fac_x != r0.fac_x || q.fac_y != r0.fac_y) {
                set_error("batch: the time step must be the same on every step");
                return -1;
            }
        b->tau[p] = r0.tau_face;
        {
            // the same values as the step arguments below
            BatchStripProb& sp = b->sprob[p];
            sp.off64 = (unsigned)(b->off[p] / 64);
            sp.goff = (unsigned)b->goff[p];
            sp.m = m;
            sp.n = n;
            sp.ld = ld;
            sp.tau = (float)r0.tau_face;
            sp.hx = (float)r.hx;
            sp.hy = (float)r.hy;
            sp.inv_hx = (float)(1.0 / r.hx);
            sp.inv_hy = (float)(1.0 / r.hy);
            sp.nu = (float)r0.fac_x;
            sp.mu = (float)r0.fac_y;
            sp.pow2 = (h_is_pow2(r.hx) ? 1 : 0) | (h_is_pow2(r.hy) ? 2 : 0);
        }
        for (int ver = 0; ver < BATCH_VERSIONS; ++ver) {
            // a representative step of this version (same parity, slot and first-step flag)
            int step = 1;
            while (batch_version(step) != ver)
                ++step;
            const int par = step & 1;
            StepArgs<float>& a = args[(size_t)p * BATCH_VERSIONS + ver];
            memset(&a, 0, sizeof(a));
            a.seq = step;
            a.find_x = a.find_y = (step > 1);
            a.stats = stats;
            a.m = m;
            a.n = n;
            a.ld = ld;
            a.plane = plane;
            a.ghost0 = g0;
            fill_gas_params(a.G, r.gamma, r.eps);
            a.hx = (float)r.hx;
            a.hy = (float)r.hy;
            a.hhx = (float)(0.5 * r.hx);
            a.hhy = (float)(0.5 * r.hy);
            a.pow2_x = h_is_pow2(r.hx);
            a.pow2_y = h_is_pow2(r.hy);
            a.inv_hx = (float)(1.0 / r.hx);
            a.inv_hy = (float)(1.0 / r.hy);
            a.alpha = (float)r.alpha;
            a.bx = r.bx;
            a.by = r.by;
            a.ctl = b->ctl + p;
            a.tau = (float)r0.tau_face;
            a.htau = (float)(0.5 * r0.tau_face);
            a.nu = (float)r0.fac_x;
            a.mu = (float)r0.fac_y;
            // odd steps read buffer 0 and write buffer 1, even steps the reverse
            const int src = (par == 1) ? 0 : 1;
            float* W0 = b->W(p, src);
            float* W1 = b->W(p, src ^ 1);
            a.src_w = W0;
            a.dst_w = W1;
            a.src_s = W0 + 5 * plane;
            a.dst_s = W1 + 5 * plane;
            a.src_t = W0 + 9 * plane;
            a.dst_t = W1 + 9 * plane;
        }
    }
    // flat tile list and processing order
    std::vector<int> tprob, tlocal, ty(np), first(np + 1);
    for (int p = 0; p < np; ++p) {
        const int nty = (b->n[p] + S.TI - 1) / S.TI, ntx = (b->m[p] + S.TJ - 1) / S.TJ;
        ty[p] = nty;
        first[p] = (int)tprob.size();
        for (int q = 0; q < ntx * nty; ++q) {
            tprob.push_back(p);
            tlocal.push_back(q);
        }
    }
    const int nt = (int)tprob.size();
    first[np] = nt;
    std::vector<int> order(nt);
    std::iota(order.begin(), order.end(), 0);
    if (schedule == 1 || schedule == 3) {
        std::vector<int> pidx(np);
        std::iota(pidx.begin(), pidx.end(), 0);
        std::stable_sort(pidx.begin(), pidx.end(), [&](int x, int y) {
            return (size_t)b->m[x] * b->n[x] > (size_t)b->m[y] * b->n[y];
        });
        order.clear();
        for (int p : pidx)
            for (int q = first[p]; q < first[p + 1]; ++q)
                order.push_back(q);
    }
    const size_t need = 3 * (size_t)nt + np;
    if (need > b->tables_cap) {
        cudaFree(b->tables);
        b->tables = nullptr;
        b->tables_cap = 0;
        if (!cuda_ok(cudaMalloc(&b->tables, sizeof(int) * need), "batch tile tables"))
            return -1;
        b->tables_cap = need;
    }
    cudaMemcpyAsync(b->tables, tprob.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->tables + nt, tlocal.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->tables + 2 * (size_t)nt, order.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->tables + 3 * (size_t)nt, ty.data(), sizeof(int) * np, cudaMemcpyHostToDevice, b->stream);
    // per processing position: the tile's problem, its index there, the problem's tiles along y
    std::vector<int4> rec(nt);
    for (int k = 0; k < nt; ++k) {
        const int t = order[k];
        rec[k] = make_int4(tprob[t], tlocal[t], ty[tprob[t]], 0);
    }
    if ((size_t)nt > b->rec_cap) {
        cudaFree(b->rec);
        b->rec = nullptr;
        b->rec_cap = 0;
        if (!cuda_ok(cudaMalloc(&b->rec, sizeof(int4) * nt), "batch tile records"))
            return -1;
        b->rec_cap = nt;
    }
    cudaMemcpyAsync(b->rec, rec.data(), sizeof(int4) * nt, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(b->args, args.data(), sizeof(StepArgs<float>) * BATCH_VERSIONS * np, cudaMemcpyHostToDevice,
                    b->stream);
    *ntiles = nt;
    return cuda_ok(cudaStreamSynchronize(b->stream), "batch prepare") ? 0 : -1;
}

// Records the time loop of the current schedule on the (capturing) stream.
// kp: the kernels' argument, a BatchDev or (strip shapes) a BatchStripDev.
static int batch_enqueue(hydro_batch* b, const BatchShape& S, const BatchDev& B, void* kp, int steps)
{
    if (b->schedule == 4 && !S.strip) {
        for (int s = 1; s <= steps; ++s) {
            void* kargs[] = {kp, (void*)&s};
            if (!cuda_ok(cudaLaunchKernel(S.step, dim3(B.ntiles), dim3(S.NT), kargs, S.smem, b->stream),
                         "batch step launch"))
                return -1;
        }
        count_launch(steps);
        return 0;
    }
    const int nwarps = S.NT / 32;
    if (b->schedule == 4) {  // strip units: per step, the CTAs that fit at once take units from a counter
        int per_sm = 0;
        if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, S.step, S.NT, S.smem), "occupancy"))
            return -1;
        if (per_sm < 1) {
            set_error("batch: the step kernel does not fit on an SM");
            return -1;
        }
        const int grid = std::max(1, std::min(per_sm * b->sms, (B.ntiles + nwarps - 1) / nwarps));
        for (int s = 1; s <= steps; ++s) {
            void* kargs[] = {kp, (void*)&s};
            if (!cuda_ok(cudaLaunchKernel(S.step, dim3(grid), dim3(S.NT), kargs, S.smem, b->stream),
                         "batch step launch"))
                return -1;
        }
        count_launch(steps);
        return 0;
    }
    int per_sm = 0;
    if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, S.persistent, S.NT, S.smem), "occupancy"))
        return -1;
    if (per_sm < 1) {
        set_error("batch: the persistent kernel does not fit on an SM");
        return -1;
    }
    const int work_ctas = S.strip ? (B.ntiles + nwarps - 1) / nwarps : B.ntiles;
    const int grid = std::max(1, std::min(per_sm * b->sms, work_ctas));
    cudaLaunchConfig_t lc;
    memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(S.NT);
    lc.dynamicSmemBytes = S.smem;
    lc.stream = b->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    void* kargs[] = {kp};
    if (!cuda_ok(cudaLaunchKernelExC(&lc, S.persistent, kargs), "batch persistent launch"))
        return -1;
    count_launch();
    return 0;
}

extern "C" {

int hydro_batch_create(hydro_batch** out, int nprob, const int* m, const int* n)
{
    *out = nullptr;
    if (nprob < 1) {
        set_error("batch: no problems");
        return -1;
    }
    hydro_batch* b = new hydro_batch();
    b->nprob = nprob;
    b->m.assign(m, m + nprob);
    b->n.assign(n, n + nprob);
    b->ld.resize(nprob);
    b->off.assign(nprob + 1, 0);
    b->goff.assign(nprob + 1, 0);
    size_t maxmn = 0;
    for (int p = 0; p < nprob; ++p) {
        if (m[p] < 2 || n[p] < 2) {
            set_error("batch: every grid must be at least 2 x 2");
            delete b;
            return -1;
        }
        b->ld[p] = (n[p] + 31) / 32 * 32;
        // 256-byte aligned starts keep every problem's stations 128-byte aligned
        b->off[p + 1] = b->off[p] + ((size_t)m[p] * b->ld[p] + 63) / 64 * 64;
        b->goff[p + 1] = b->goff[p] + 8 * ((size_t)m[p] + n[p]);
        maxmn = std::max(maxmn, (size_t)m[p] * n[p]);
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    b->pool = b->off[nprob];
    if (!cuda_ok(cudaMalloc(&b->mem, sizeof(float) * 26 * b->pool), "batch states") ||
        !cuda_ok(cudaMemset(b->mem, 0, sizeof(float) * 26 * b->pool), "batch clear") ||
        !cuda_ok(cudaMalloc(&b->ghost, sizeof(float) * b->goff[nprob]), "batch boundary tables") ||
        !cuda_ok(cudaMalloc(&b->ctl, sizeof(Ctl) * nprob), "batch control blocks") ||
        !cuda_ok(cudaMalloc(&b->args, sizeof(StepArgs<float>) * BATCH_VERSIONS * nprob), "batch step arguments") ||
        !cuda_ok(cudaMalloc(&b->sync, sizeof(unsigned int) * 8), "batch barrier") ||
        !cuda_ok(cudaMalloc(&b->stage, sizeof(double) * 5 * maxmn), "batch staging") ||
        !cuda_ok(cudaMalloc(&b->red, sizeof(unsigned long long)), "batch reduction") ||
        !cuda_ok(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "batch stream") ||
        !cuda_ok(cudaEventCreate(&b->e0), "event") || !cuda_ok(cudaEventCreate(&b->e1), "event")) {
        delete b;
        return -1;
    }
    for (const BatchShape& s : batch_shapes())
        for (const void* k : {s.persistent, s.step}) {
            // tile shapes: the shared memory their MINB CTAs per SM need, the rest L1
            int carve = s.carve;
            cudaFuncAttributes fa;
            if (!s.strip && cudaFuncGetAttributes(&fa, k) == cudaSuccess)
                carve = carve_for(s.smem + fa.sharedSizeBytes, s.MINB);
            if (!cuda_ok(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem),
                         "smem attr") ||
                !cuda_ok(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, carve),
                         "carveout attr")) {
                delete b;
                return -1;
            }
        }
    *out = b;
    return 0;
}

void hydro_batch_destroy(hydro_batch* b) { delete b; }

int hydro_batch_upload(hydro_batch* b, int p, const double* rho, const double* u, const double* v, const double* pr,
                       const double* E, double gamma)
{
    if (p < 0 || p >= b->nprob) {
        set_error("batch: no such problem");
        return -1;
    }
    const int m = b->m[p], n = b->n[p], ld = b->ld[p];
    const size_t mn = (size_t)m * n, plane = b->plane(p);
    double* st = b->stage;
    const double* src[4] = {rho, u, v, pr};
    for (int k = 0; k < 4; ++k)
        if (!cuda_ok(cudaMemcpyAsync(st + k * mn, src[k], sizeof(double) * mn, cudaMemcpyHostToDevice, b->stream),
                     "batch upload"))
            return -1;
    if (E) {
        if (!cuda_ok(cudaMemcpyAsync(st + 4 * mn, E, sizeof(double) * mn, cudaMemcpyHostToDevice, b->stream),
                     "batch upload"))
            return -1;
    } else {
        k_energy<<<b->grid1d(mn), 256, 0, b->stream>>>(st, st + mn, st + 2 * mn, st + 3 * mn, st + 4 * mn, mn, gamma);
        count_launch();
    }
    for (int k = 0; k < 5; ++k) {
        k_pack_plane<float><<<b->grid1d(mn), 256, 0, b->stream>>>(st + k * mn, b->W(p, 0) + k * plane, m, n, ld);
        count_launch();
    }
    // the 8 slope planes of both states: rows of m ld elements, pool elements apart
    const size_t row = sizeof(float) * m * ld;
    if (!cuda_ok(cudaMemset2DAsync(b->W(p, 0) + 5 * plane, sizeof(float) * plane, 0, row, 8, b->stream),
                 "batch clear") ||
        !cuda_ok(cudaMemset2DAsync(b->W(p, 1) + 5 * plane, sizeof(float) * plane, 0, row, 8, b->stream),
                 "batch clear"))
        return -1;
    if (!b->final_buf.empty())
        b->final_buf[p] = 0;
    return cuda_ok(cudaStreamSynchronize(b->stream), "batch upload") ? 0 : -1;
}

int hydro_batch_download(hydro_batch* b, int p, double* rho, double* u, double* v, double* pr, double* E)
{
    if (p < 0 || p >= b->nprob) {
        set_error("batch: no such problem");
        return -1;
    }
    const int m = b->m[p], n = b->n[p], ld = b->ld[p];
    const size_t mn = (size_t)m * n, plane = b->plane(p);
    const int buf = b->final_buf.empty() ? 0 : b->final_buf[p];
    double* dst[5] = {rho, u, v, pr, E};
    for (int k = 0; k < 5; ++k) {
        if (!dst[k])
            continue;
        k_unpack_plane<float><<<b->grid1d(mn), 256, 0, b->stream>>>(b->W(p, buf) + k * plane, b->stage + k * mn, m,
                                                                    n, ld);
        count_launch();
        if (!cuda_ok(cudaMemcpyAsync(dst[k], b->stage + k * mn, sizeof(double) * mn, cudaMemcpyDeviceToHost,
                                     b->stream),
                     "batch download"))
            return -1;
    }
    return cuda_ok(cudaStreamSynchronize(b->stream), "batch download") ? 0 : -1;
}

int hydro_batch_num_shapes(void) { return (int)batch_shapes().size(); }
int hydro_batch_shape_kind(int shape)
{
    if (shape < 0 || shape >= (int)batch_shapes().size()) {
        set_error("batch: no such tile shape");
        return -1;
    }
    return batch_shapes()[shape].strip;
}
int hydro_batch_num_schedules(void) { return BATCH_SCHEDULES; }

int hydro_batch_shape(int shape, int* out4)
{
    if (shape < 0 || shape >= (int)batch_shapes().size()) {
        set_error("batch: no such tile shape");
        return -1;
    }
    const BatchShape& s = batch_shapes()[shape];
    out4[0] = s.TI;
    out4[1] = s.TJ;
    out4[2] = s.NT;
    out4[3] = s.MINB;
    return 0;
}

int hydro_batch_set_schedule(hydro_batch* b, int shape, int schedule)
{
    if (shape < 0 || shape >= (int)batch_shapes().size() || schedule < 0 || schedule >= BATCH_SCHEDULES) {
        set_error("batch: no such tile shape or schedule");
        return -1;
    }
    b->shape = shape;
    b->schedule = schedule;
    return 0;
}

int hydro_batch_set_wait_limit(hydro_batch* b, double seconds)
{
    if (!(seconds > 0.0)) {
        set_error("batch: the barrier wait limit must be positive");
        return -1;
    }
    b->wait_s = seconds;
    return 0;
}

int hydro_batch_run(hydro_batch* b, const double* cfg, int ncfg, int steps, int stats, hydro_batch_info* info)
{
    if (steps < 1) {
        set_error("batch: at least one step");
        return -1;
    }
    if (ncfg > 301 && isfinite(cfg[301]) && (int)cfg[301] != HYDRO_SOLVER_Q1D) {
        set_error("batch: built for the quasi-1D interface solver (config[301])");
        return -1;
    }
    const BatchShape& S = batch_shapes()[b->shape];
    if (S.strip && (b->nprob > BATCH_STRIP_MAX || b->pool / 64 > 0xffffffffull || b->goff[b->nprob] > 0xffffffffull)) {
        set_error("batch: the strip shapes take at most 576 problems of at most 2^38 state elements");
        return -1;
    }
    int nt = 0;
    if (batch_prepare(b, cfg, ncfg, steps, stats, S, b->schedule, &nt))
        return -1;
    BatchDev B;
    memset(&B, 0, sizeof(B));
    B.args = b->args;
    B.ctl = b->ctl;
    B.tile_prob = b->tables;
    B.tile_local = b->tables + nt;
    B.order = b->tables + 2 * (size_t)nt;
    B.tiles_y = b->tables + 3 * (size_t)nt;
    B.rec = b->rec;
    B.ntiles = nt;
    B.nprob = b->nprob;
    B.steps = steps;
    B.dynamic = (b->schedule == 2 || b->schedule == 3);
    B.stats = stats;
    B.work = b->sync;
    B.bar_count = b->sync + 2;
    B.bar_gen = b->sync + 3;
    B.bar_err = (int*)(b->sync + 4);
    B.wait_ns = (unsigned long long)(b->wait_s * 1e9);
    const RunConfig rcfg = run_config_from(cfg, ncfg);
    fill_gas_params(B.G, rcfg.gamma, rcfg.eps);
    // the strip shapes' arguments: the batch's common ones and every problem's
    std::unique_ptr<BatchStripDev> D;
    void* kp = &B;
    if (S.strip) {
        D.reset(new BatchStripDev());
        memset(D.get(), 0, sizeof(BatchStripDev));
        D->B = B;
        D->mem = b->mem;
        D->pool = b->pool;
        D->ghost = b->ghost;
        D->alpha = (float)rcfg.alpha;
        D->bx = rcfg.bx;
        D->by = rcfg.by;
        std::copy(b->sprob.begin(), b->sprob.end(), D->P);
        kp = D.get();
    }
    if (!cuda_ok(cudaMemsetAsync(b->ctl, 0, sizeof(Ctl) * b->nprob, b->stream), "batch control clear") ||
        !cuda_ok(cudaMemsetAsync(b->sync, 0, sizeof(unsigned int) * 8, b->stream), "batch barrier clear"))
        return -1;

    // the whole time loop as one CUDA graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graphed = 0;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc = batch_enqueue(b, S, B, kp, steps);
        const cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
        if (rc == 0 && ce == cudaSuccess && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
            graphed = 1;
    }
    if (!graphed) {
        // this launch form could not be captured: clear the error and launch directly
        cudaGetLastError();
        set_error("");
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    cudaEventRecord(b->e0, b->stream);
    int rc = 0;
    if (graphed)
        rc = cuda_ok(cudaGraphLaunch(exec, b->stream), "batch graph launch") ? 0 : -1;
    else
        rc = batch_enqueue(b, S, B, kp, steps);
    cudaEventRecord(b->e1, b->stream);
    std::vector<Ctl> hc(b->nprob);
    unsigned int hs[8] = {0};
    cudaMemcpyAsync(hc.data(), b->ctl, sizeof(Ctl) * b->nprob, cudaMemcpyDeviceToHost, b->stream);
    cudaMemcpyAsync(hs, b->sync, sizeof(hs), cudaMemcpyDeviceToHost, b->stream);
    const bool ok = cuda_ok(cudaStreamSynchronize(b->stream), "batch run");
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (!ok || rc)
        return -1;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->e0, b->e1);
    if (hs[4]) {
        set_error("batch: a grid barrier wait ran out of time");
        return -2;
    }
    b->final_buf.assign(b->nprob, steps & 1);
    b->halted_kind.assign(b->nprob, 0);
    b->halted_step.assign(b->nprob, 0);
    int halted = 0;
    unsigned long long nf = 0, ni = 0, nfb = 0;
    for (int p = 0; p < b->nprob; ++p) {
        int q = 0, kind = 0;
        if (hc[p].halted_seq) {
            q = hc[p].halted_seq;
            kind = hc[p].halt_kind;
        } else {
            const int ls = steps % 3;
            const int d = halt_decision(hc[p].key[ls][0], hc[p].key[ls][1], hc[p].upd_bad[ls]);
            if (d) {
                q = steps;
                kind = d;
            }
        }
        if (q) {
            halted++;
            b->halted_kind[p] = kind;
            b->halted_step[p] = q;
            // abort discards launch q (its input buffer is kept), stop keeps it
            b->final_buf[p] = (kind == 1) ? ((q - 1) & 1) : (q & 1);
        }
        nf += hc[p].newton_faces;
        ni += hc[p].newton_iters;
        nfb += hc[p].newton_fallbacks;
    }
    if (info) {
        memset(info, 0, sizeof(*info));
        info->gpu_ms = ms;
        info->shape = b->shape;
        info->schedule = b->schedule;
        info->graphed = graphed;
        info->steps = steps;
        info->tiles = nt;
        info->halted_problems = halted;
        info->newton_faces = nf;
        info->newton_iters = ni;
        info->newton_fallbacks = nfb;
    }
    return 0;
}

int hydro_batch_autotune(hydro_batch* b, const double* cfg, int ncfg, int steps, float* times_ms)
{
    const size_t total = 26 * b->pool;
    float* backup = nullptr;
    if (!cuda_ok(cudaMalloc(&backup, sizeof(float) * total), "autotune backup"))
        return -1;
    std::vector<int> fb = b->final_buf;
    cudaMemcpyAsync(backup, b->mem, sizeof(float) * total, cudaMemcpyDeviceToDevice, b->stream);
    int best = -1;
    float best_ms = 3e38f;
    const int nshape = (int)batch_shapes().size();
    for (int sh = 0; sh < nshape; ++sh)
        for (int sc = 0; sc < BATCH_SCHEDULES; ++sc) {
            // The strip shapes are not candidates: timed over the first steps of a run they come
            // within ~20% of the tiles, but their warps solve the exact faces of a discontinuity
            // along the march one or two at a time, and as a run develops more of those faces they
            // fall far behind (5 against 8.6 G cell-updates/s over 300 steps of 512 problems).
            if (batch_shapes()[sh].strip) {
                if (times_ms)
                    times_ms[sh * BATCH_SCHEDULES + sc] = 3e38f;
                continue;
            }
            cudaMemcpyAsync(b->mem, backup, sizeof(float) * total, cudaMemcpyDeviceToDevice, b->stream);
            b->shape = sh;
            b->schedule = sc;
            hydro_batch_info info;
            const int rc = hydro_batch_run(b, cfg, ncfg, steps, 0, &info);
            const float ms = rc ? 3e38f : (float)info.gpu_ms;
            if (times_ms)
                times_ms[sh * BATCH_SCHEDULES + sc] = ms;
            if (rc == -2) {  // a barrier gave up: stop tuning
                cudaFree(backup);
                return -1;
            }
            if (ms < best_ms) {
                best_ms = ms;
                best = sh * BATCH_SCHEDULES + sc;
            }
        }
    cudaMemcpyAsync(b->mem, backup, sizeof(float) * total, cudaMemcpyDeviceToDevice, b->stream);
    const bool ok = cuda_ok(cudaStreamSynchronize(b->stream), "autotune restore");
    cudaFree(backup);
    b->final_buf = fb;
    if (!ok || best < 0)
        return -1;
    b->shape = best / BATCH_SCHEDULES;
    b->schedule = best % BATCH_SCHEDULES;
    return best;
}

int hydro_batch_problem_info(hydro_batch* b, int p, int* halted_kind, int* halted_step, double* tau)
{
    if (p < 0 || p >= b->nprob) {
        set_error("batch: no such problem");
        return -1;
    }
    *halted_kind = b->halted_kind.empty() ? 0 : b->halted_kind[p];
    *halted_step = b->halted_step.empty() ? 0 : b->halted_step[p];
    *tau = b->tau.empty() ? 0.0 : b->tau[p];
    return 0;
}

int hydro_gb300_batch_run(hydro_problem* probs, int nprob, int steps, hydro_batch_opts* o)
{
    if (!probs || nprob < 1 || !o || !o->cfg) {
        set_error("batch: problems and options are required");
        return -1;
    }
    std::vector<int> m(nprob), n(nprob);
    for (int p = 0; p < nprob; ++p) {
        m[p] = probs[p].m;
        n[p] = probs[p].n;
    }
    hydro_batch* b = nullptr;
    if (hydro_batch_create(&b, nprob, m.data(), n.data()))
        return -1;
    const double gamma = o->ncfg > 6 ? o->cfg[6] : 1.4;
    int rc = 0;
    for (int p = 0; p < nprob && !rc; ++p)
        rc = hydro_batch_upload(b, p, probs[p].rho, probs[p].u, probs[p].v, probs[p].p, probs[p].E, gamma);
    if (!rc && o->autotune_steps > 0)
        rc = hydro_batch_autotune(b, o->cfg, o->ncfg, o->autotune_steps, nullptr) < 0 ? -1 : 0;
    else if (!rc)
        rc = hydro_batch_set_schedule(b, o->shape, o->schedule);
    if (!rc)
        rc = hydro_batch_run(b, o->cfg, o->ncfg, steps, o->stats, &o->info);
    for (int p = 0; p < nprob && !rc; ++p) {
        hydro_problem& q = probs[p];
        rc = hydro_batch_download(b, p, q.rho, q.u, q.v, q.p, q.E);
        if (!rc)
            rc = hydro_batch_problem_info(b, p, &q.halted, &q.halted_step, &q.tau);
    }
    hydro_batch_destroy(b);
    return rc;
}

}  // extern "C"
