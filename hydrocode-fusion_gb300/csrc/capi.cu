// capi.cu -- the C ABI of libhydro_gb300.so: the reference's 2D scheme entry
// points (same signatures and side effects), the native solver API, time-loop
// planning and error reporting.  Host code only; the kernels live in the
// per-precision translation units.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "solver2d.h"

// Weak fallback for the caller-defined configuration array: a driver that
// defines `double config[N_CONF]` (as the reference's drivers do) overrides it.
extern "C" {
__attribute__((weak)) double config[N_CONF];
}

namespace hydro {

static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};

void set_error(const std::string& msg) { g_err = msg; }
void count_launch(unsigned long long k) { g_launches += k; }
bool cuda_ok(cudaError_t e, const char* what)
{
    if (e == cudaSuccess)
        return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

int host_rows_mode()
{
    // measured on GB300 + Grace, 4096^2, 20 steps, the second call on the same
    // host arrays: 24.9-25.1 ms staged both ways, 22.8 ms with the upload
    // direct, 21.9 ms direct both ways; but a direct download into rows the
    // host never touched takes their page faults on the GPU (0.19 s for such
    // a first call, against 27-44 ms with the download staged).  So by
    // default the GPU reads the caller's rows (already written by the caller)
    // and the download stays staged.
    const char* e = getenv("HYDRO_DIRECT_HOST_ROWS");
    const int want = !e ? 1 : strcmp(e, "in") == 0 ? 1 : atoi(e) != 0 ? 3 : 0;
    if (!want)
        return 0;
    int dev = 0, v = 0, ats = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    // the default only where the GPU walks the host's own page tables
    // (address translation services); on request wherever access is coherent
    return v == 1 && (e || ats == 1) ? want : 0;
}

RunConfig run_config_from(const double* cfg, int ncfg)
{
    auto at = [&](int k) { return k < ncfg ? cfg[k] : INFINITY; };
    RunConfig r;
    r.t_all = at(1);
    r.eps = at(4);
    r.N = (int)at(5);
    r.gamma = at(6);
    r.cfl = at(7);
    r.hx = at(10);
    r.hy = at(11);
    r.cfg16 = at(16);
    r.bx = (int)at(17);
    r.by = (int)at(18);
    r.alpha = at(41);
    return r;
}

// Mirrors the control flow of the reference's time loops
// (grp_solver_2D_EUL_source.c:146-286, grp_solver_2D_split_EUL_source.c:148-337):
// plot snapshots, the CFL step from the initial data, clipping of the last
// step to t_all, the tau < eps stop, the non-finite-tau abort and the
// alternating x-half / y / x-half sweeps of the split scheme.
RunPlan plan_run(const RunConfig& rc, double hs, int split, const double* time_plot, int N_plot, int N_T)
{
    RunPlan P;
    P.hs_max = hs;
    int nt = 0, nt_plot = 0, DS = 1, k = 1;
    double time_c = 0.0, tau = rc.cfg16;
    double half_tau = 0.0, half_nu = 0.0, nu = 0.0, mu = 0.0;
    bool stop_after = false;
    int find_x = 0, find_y = 0;
    while (k <= rc.N) {
        int seq_next = (int)P.sweeps.size() + 1;
        if (time_c >= time_plot[nt_plot] && nt_plot < (N_plot - 1)) {
            nt_plot++;
            if (nt < (N_T - 1)) {
                P.snaps.push_back({seq_next, nt});
                nt++;
            }
        }
        if (!split || DS) {
            if (isfinite(rc.t_all) || !isfinite(rc.cfg16) || rc.cfg16 <= 0.0) {
                tau = rc.cfl * hs;
                if (tau < rc.eps)
                    stop_after = true;
                else if ((time_c + tau) > (rc.t_all - rc.eps))
                    tau = rc.t_all - time_c;
                else if (!isfinite(tau))
                    break;  // abort before the step
            }
            if (split) {
                half_tau = tau * 0.5;
                half_nu = half_tau / rc.hx;
                mu = tau / rc.hy;
            } else {
                nu = tau / rc.hx;
                mu = tau / rc.hy;
            }
        }
        if (!split) {
            SweepRec r{k, 0, tau, nu, mu, find_x, find_y, nt, time_c, 0.0};
            find_x = find_y = 1;
            time_c += tau;
            r.time_after = time_c;
            P.sweeps.push_back(r);
            if (stop_after || time_c > (rc.t_all - rc.eps) || !isfinite(time_c))
                break;
            ++k;
        } else {
            SweepRec rx{k, 1, half_tau, half_nu, 0.0, find_x, find_y, nt, time_c, time_c};
            find_x = 1;
            P.sweeps.push_back(rx);
            if (stop_after)
                break;
            if (DS) {
                SweepRec ry{k, 2, tau, 0.0, mu, find_x, find_y, nt, time_c, time_c + tau};
                find_y = 1;
                time_c += tau;
                ry.time_after = time_c;
                P.sweeps.push_back(ry);
            }
            if (stop_after || time_c > (rc.t_all - rc.eps) || !isfinite(time_c))
                break;
            DS = DS ? 0 : 1;
            if (!DS)
                ++k;
        }
    }
    P.end_k = k;
    P.end_time = time_c;
    P.end_tau = tau;
    P.end_nt = nt;
    return P;
}

static int form_from_config(const double* cfg)
{
    double f = cfg[300];
    if (!isfinite(f))
        return HYDRO_FORM_FP64;
    return (int)f;
}

// config[301]: the interface GRP solver (HYDRO_SOLVER_*), the quasi-1D one
// when absent, as in the reference's GRP_2D_flux (flux_solver.c:191).
static int solver_from_config(const double* cfg)
{
    double f = cfg[301];
    if (!isfinite(f))
        return HYDRO_SOLVER_Q1D;
    return (int)f;
}

// The trained network shipped with the library: $HYDRO_MLP_WEIGHTS, else
// weights/riemann_guess_6_64_64_1.f32 next to the library's build folder.
static bool default_mlp(std::vector<float>& w, std::string& path)
{
    if (const char* e = getenv("HYDRO_MLP_WEIGHTS")) {
        path = e;
    } else {
        Dl_info di;
        if (!dladdr((void*)&default_mlp, &di) || !di.dli_fname)
            return false;
        std::string so = di.dli_fname;
        size_t cut = so.rfind('/');
        std::string dir = cut == std::string::npos ? std::string(".") : so.substr(0, cut);
        path = dir + "/../weights/riemann_guess_6_64_64_1.f32";
    }
    FILE* f = fopen(path.c_str(), "rb");
    if (!f)
        return false;
    w.assign(HYDRO_MLP_NPARAM, 0.f);
    size_t got = fread(w.data(), sizeof(float), w.size() + 1, f);
    fclose(f);
    return got == w.size();
}

static Solver2DBase* make_solver(int m, int n, int form, int rs)
{
    switch (form) {
    case HYDRO_FORM_FP64:
        return make_solver2d_f64(m, n, rs);
    case HYDRO_FORM_FP32:
        return make_solver2d_f32(m, n, 0, rs);
    case HYDRO_FORM_FP32_LEARNED: {
        Solver2DBase* s = make_solver2d_f32(m, n, 1, rs);
        if (!s)
            return nullptr;
        // install the shipped network when it is there (hydro2d_set_mlp replaces it)
        std::vector<float> w;
        std::string path;
        if (default_mlp(w, path))
            s->set_mlp(w.data());
        return s;
    }
    default:
        set_error("unknown form");
        return nullptr;
    }
}

// Worker threads of parallel_range, started on first use and kept for the
// life of the process (the staged copies call it once per 64 MB block, and
// starting fifteen threads per call showed up in their times).  One job at a
// time: callers are serialised, and a job ends when every worker has seen it.
namespace {
struct RangePool {
    std::mutex call;  // one job at a time
    std::mutex m;
    std::condition_variable go, done;
    const std::function<void(int, int)>* fn = nullptr;
    int rows = 0, T = 0, pending = 0;
    unsigned gen = 0;
    int nworkers = 0;

    explicit RangePool(int n) : nworkers(n)
    {
        for (int t = 1; t <= n; ++t)
            std::thread([this, t] { work(t); }).detach();
    }
    void work(int t)
    {
        unsigned seen = 0;
        for (;;) {
            const std::function<void(int, int)>* f;
            int r, TT;
            {
                std::unique_lock<std::mutex> lk(m);
                go.wait(lk, [&] { return gen != seen; });
                seen = gen;
                f = fn;
                r = rows;
                TT = T;
            }
            if (t < TT)
                (*f)((int)((long long)r * t / TT), (int)((long long)r * (t + 1) / TT));
            std::lock_guard<std::mutex> lk(m);
            if (--pending == 0)
                done.notify_one();
        }
    }
    void run(int r, int TT, const std::function<void(int, int)>& f)
    {
        std::lock_guard<std::mutex> one(call);
        {
            std::lock_guard<std::mutex> lk(m);
            fn = &f;
            rows = r;
            T = TT;
            pending = nworkers;
            ++gen;
        }
        go.notify_all();
        f(0, (int)((long long)r / TT));
        std::unique_lock<std::mutex> lk(m);
        done.wait(lk, [&] { return pending == 0; });
    }
};
}  // namespace

void parallel_range(int rows, size_t bytes, const std::function<void(int, int)>& fn)
{
    unsigned hw = std::thread::hardware_concurrency();
    const int TMAX = (int)(hw ? (hw < 16 ? hw : 16) : 4);
    int T = bytes < (size_t)(8u << 20) ? 1 : TMAX;
    if (T > rows)
        T = rows;
    if (T <= 1) {
        fn(0, rows);
        return;
    }
    // never destroyed: its workers wait for jobs until the process ends
    static RangePool* pool = new RangePool(TMAX - 1);
    pool->run(rows, T, fn);
}

// Runs fn(j0, j1) over row blocks of an m x n host copy of the 5 state planes
// (the caller's rows are separate allocations, so the packing into and out of
// one buffer is plain memory traffic).
template <typename F>
static void parallel_rows(int m, int n, F fn)
{
    parallel_range(m, (size_t)m * n * 40, fn);
}

HostPair* host_pair()
{
    static HostPair* pp = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        HostPair* h = new HostPair();
        h->bytes = (size_t)64 << 20;
        for (int b = 0; b < 2; ++b) {
            if (cudaHostAlloc(&h->buf[b], h->bytes, cudaHostAllocDefault) != cudaSuccess) {
                cudaGetLastError();  // not pinned: the copies still work, staged by the driver
                h->buf[b] = malloc(h->bytes);
            }
            if (cudaEventCreateWithFlags(&h->ev[b], cudaEventDisableTiming) != cudaSuccess || !h->buf[b]) {
                set_error("host staging buffers");
                return;
            }
        }
        pp = h;
    });
    return pp;
}

// The 2D entry points keep the last call's solver (its device buffers, kernel
// set-up and network) for the next call with the same grid, form and interface
// solver, as a memory pool keeps its blocks: a caller that runs the scheme
// repeatedly pays the solver's set-up once.  HYDRO_SOLVER_CACHE=0 turns it off
// (each call creates and frees its own); hydro_gb300_release_cache() frees the
// kept solver.  The cache object is never destroyed: a solver still held at
// exit goes with the process's CUDA context.
struct SolverCache {
    std::mutex mu;
    Solver2DBase* s = nullptr;
    int m = 0, n = 0, form = -1, rs = -1;
};
static SolverCache& solver_cache()
{
    static SolverCache* c = new SolverCache();
    return *c;
}
static bool solver_cache_on()
{
    const char* e = getenv("HYDRO_SOLVER_CACHE");
    return !(e && atoi(e) == 0);
}
static Solver2DBase* acquire_solver(int m, int n, int form, int rs)
{
    if (solver_cache_on()) {
        SolverCache& c = solver_cache();
        std::lock_guard<std::mutex> guard(c.mu);
        if (c.s && c.m == m && c.n == n && c.form == form && c.rs == rs) {
            Solver2DBase* s = c.s;
            c.s = nullptr;  // one caller at a time uses it
            return s;
        }
    }
    return make_solver(m, n, form, rs);
}
static void release_solver(Solver2DBase* s, int m, int n, int form, int rs)
{
    Solver2DBase* old = s;
    if (solver_cache_on()) {
        SolverCache& c = solver_cache();
        std::lock_guard<std::mutex> guard(c.mu);
        old = c.s;
        c.s = s;
        c.m = m;
        c.n = n;
        c.form = form;
        c.rs = rs;
    }
    delete old;
}

// Shared body of the two 2D scheme entry points.
static void run_2d_entry(const int m, const int n, struct cell_var_stru* CV, double* cpu_time, int N_T, int* N_plot,
                         double time_plot[], int split)
{
    const double t_all = config[1];
    const int form = form_from_config(config), rs = solver_from_config(config);
    Solver2DBase* s = acquire_solver(m, n, form, rs);
    if (!s) {
        fprintf(stderr, "hydro_gb300: cannot create the 2D solver: %s\n", hydro_gb300_last_error());
        exit(5);
    }
    size_t mn = (size_t)m * n;
    // The caller's state is a set of separately allocated rows.  Where the GPU
    // reads pageable host memory coherently (Grace-Blackwell), the kernels
    // gather and scatter those rows themselves; elsewhere the rows are packed
    // into one host buffer and copied.
    const int direct = host_rows_mode();
    const double* const* in_rows[5] = {CV[0].RHO, CV[0].U, CV[0].V, CV[0].P, CV[0].E};
    if ((direct & 1) ? s->upload_rows(in_rows) : s->upload_rows_staged(in_rows)) {
        fprintf(stderr, "hydro_gb300: upload failed: %s\n", hydro_gb300_last_error());
        exit(5);
    }
    std::vector<std::vector<double>> snaps(N_T);
    std::vector<double*> snap_ptr(N_T, nullptr);
    for (int k = 1; k < N_T - 1; ++k) {  // CV[0] keeps the initial data, no copy needed
        snaps[k].resize(5 * mn);
        snap_ptr[k] = snaps[k].data();
    }
    RunConfig rc = run_config_from(config, N_CONF);
    hydro_run_info info;
    int nt = 0;
    if (s->run(rc, split, 0, time_plot, *N_plot, N_T, snap_ptr.data(), &info, &nt)) {
        fprintf(stderr, "hydro_gb300: time loop failed: %s\n", hydro_gb300_last_error());
        exit(5);
    }
    double* const* out_rows[5] = {CV[nt].RHO, CV[nt].U, CV[nt].V, CV[nt].P, CV[nt].E};
    if ((direct & 2) ? s->download_rows(out_rows) : s->download_rows_staged(out_rows)) {
        fprintf(stderr, "hydro_gb300: download failed: %s\n", hydro_gb300_last_error());
        exit(5);
    }
    release_solver(s, m, n, form, rs);
    auto scatter = [&](int k, const double* src) {
        parallel_rows(m, n, [&](int j0, int j1) {
            for (int j = j0; j < j1; ++j) {
                memcpy(CV[k].RHO[j], src + (size_t)j * n, n * sizeof(double));
                memcpy(CV[k].U[j], src + mn + (size_t)j * n, n * sizeof(double));
                memcpy(CV[k].V[j], src + 2 * mn + (size_t)j * n, n * sizeof(double));
                memcpy(CV[k].P[j], src + 3 * mn + (size_t)j * n, n * sizeof(double));
                memcpy(CV[k].E[j], src + 4 * mn + (size_t)j * n, n * sizeof(double));
            }
        });
    };
    for (int k = 1; k < nt; ++k)  // CV[0] already holds the initial data
        scatter(k, snaps[k].data());

    if (info.halted == 1)
        printf("Error on the time step %d (x-face code %d, y-face code %d); the step was discarded.\n", info.k_out,
               info.error_code_x, info.error_code_y);
    else if (info.halted == 2)
        printf("Error on the time step %d (x-face code %d, y-face code %d, or a non-positive update); stopped after the step.\n",
               info.k_out, info.error_code_x, info.error_code_y);
    printf("\nTime is up at time step %d.\n", info.k_out);
    printf("The cost of GPU time for the %s 2D-GRP Eulerian scheme for this problem is %g seconds.\n",
           split ? "dimension-split" : "unsplit", info.gpu_ms * 1e-3);
    config[5] = (double)info.k_out;
    *N_plot = nt + 1;
    if (isfinite(info.time))
        time_plot[nt] = info.time;
    else if (isfinite(t_all))
        time_plot[nt] = t_all;
    else if (isfinite(info.tau))
        time_plot[nt] = info.k_out * info.tau;
    for (int k = 0; k <= nt; ++k)
        cpu_time[k] = info.gpu_ms * 1e-3;
}

}  // namespace hydro

using namespace hydro;

struct hydro2d {
    Solver2DBase* s;
};

extern "C" {

const char* hydro_gb300_last_error(void) { return g_err.c_str(); }
unsigned long long hydro_gb300_kernel_launches(void) { return g_launches.load(); }

void hydro_gb300_release_cache(void)
{
    SolverCache& c = solver_cache();
    Solver2DBase* old = nullptr;
    {
        std::lock_guard<std::mutex> guard(c.mu);
        old = c.s;
        c.s = nullptr;
    }
    delete old;
}

int hydro2d_create_ex(hydro2d_t** out, int m, int n, int form, int solver)
{
    *out = nullptr;
    if (m < 2 || n < 2) {
        set_error("grid must be at least 2 x 2");
        return -1;
    }
    Solver2DBase* s = make_solver(m, n, form, solver);
    if (!s)
        return -1;
    *out = new hydro2d{s};
    return 0;
}

int hydro2d_create(hydro2d_t** out, int m, int n, int form)
{
    return hydro2d_create_ex(out, m, n, form, HYDRO_SOLVER_Q1D);
}

void hydro2d_destroy(hydro2d_t* h)
{
    if (!h)
        return;
    delete h->s;
    delete h;
}

int hydro2d_upload(hydro2d_t* h, const double* rho, const double* u, const double* v, const double* p, const double* E,
                   double gamma)
{
    return h->s->upload(rho, u, v, p, E, gamma);
}

int hydro2d_download(hydro2d_t* h, double* rho, double* u, double* v, double* p, double* E)
{
    return h->s->download(rho, u, v, p, E);
}

int hydro2d_run(hydro2d_t* h, const double* cfg, int ncfg, int split, int stats, hydro_run_info* info)
{
    RunConfig rc = run_config_from(cfg, ncfg);
    double tp[2] = {0.0, rc.t_all};
    int nt = 0;
    return h->s->run(rc, split, stats, tp, 2, 2, nullptr, info, &nt);
}

int hydro2d_num_variants(hydro2d_t* h) { return h->s->num_variants(); }
int hydro2d_set_variant(hydro2d_t* h, int v) { return h->s->set_variant(v); }
int hydro2d_get_variant(hydro2d_t* h, int* shape)
{
    int v = h->s->get_variant();
    if (shape)
        h->s->variant_shape(v, shape);
    return v;
}
int hydro2d_set_mlp(hydro2d_t* h, const float* params) { return h->s->set_mlp(params); }
int hydro2d_conservation(hydro2d_t* h, double hx, double hy, double* sums)
{
    return h->s->conservation(hx, hy, sums);
}

int hydro2d_autotune(hydro2d_t* h, const double* cfg, int ncfg, int steps, float* times_ms)
{
    return h->s->autotune(run_config_from(cfg, ncfg), steps, times_ms);
}

void GRP_solver_2D_EUL_source(const int m, const int n, struct cell_var_stru* CV, double** X, double** Y,
                              double* cpu_time, const char* problem, int N_T, int* N_plot, double time_plot[])
{
    (void)X;
    (void)Y;
    (void)problem;
    run_2d_entry(m, n, CV, cpu_time, N_T, N_plot, time_plot, 0);
}

void GRP_solver_2D_split_EUL_source(const int m, const int n, struct cell_var_stru* CV, double** X, double** Y,
                                    double* cpu_time, const char* problem, int N_T, int* N_plot, double time_plot[])
{
    (void)X;
    (void)Y;
    (void)problem;
    run_2d_entry(m, n, CV, cpu_time, N_T, N_plot, time_plot, 1);
}

}  // extern "C"
