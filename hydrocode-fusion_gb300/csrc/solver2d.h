// solver2d.h -- host-side interface shared by the 2D solver translation units.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hydro_gb300.h"

namespace hydro {

// Run configuration taken from config[] (indices of the reference's doc/config.csv).
struct RunConfig {
    double t_all, eps, gamma, cfl, hx, hy, cfg16, alpha;
    int N, bx, by;
};
RunConfig run_config_from(const double* cfg, int ncfg);

// A plot snapshot request: before which launch the current state is recorded.
struct SnapshotPlan {
    int seq;  // record the state just before launch `seq` (1-based)
    int nt;   // snapshot index it becomes (CV[nt])
};

// The host-side plan of a time loop: one record per kernel launch, computed
// with the same double arithmetic as the reference's loop.
struct SweepRec {
    int k;             // reference step counter during this launch
    int dir;           // 0 unsplit step, 1 x-sweep, 2 y-sweep
    double tau_face;   // time step passed to the GRP flux
    double fac_x, fac_y;  // nu (tau/h_x, or half_tau/h_x) and mu
    int find_x, find_y;
    int nt;            // snapshot index the state lives in during this launch
    double time_before, time_after;
};

struct RunPlan {
    std::vector<SweepRec> sweeps;
    std::vector<SnapshotPlan> snaps;
    int end_k;           // config[5] if nothing halts on the device
    double end_time;     // time_c at the end of the plan
    double end_tau;
    int end_nt;
    double hs_max;       // CFL h/S_max from the initial data
};

// Builds the plan. time_plot: plot times (time_plot[0] = 0, last = t_all), N_T
// stored snapshots at most.
RunPlan plan_run(const RunConfig& rc, double h_S_max, int split, const double* time_plot, int N_plot, int N_T);

// Type-erased solver (FP64 and FP32 instantiations live in separate TUs).
class Solver2DBase {
public:
    virtual ~Solver2DBase() {}
    virtual int upload(const double* rho, const double* u, const double* v, const double* p, const double* E,
                       double gamma) = 0;
    virtual int download(double* rho, double* u, double* v, double* p, double* E) = 0;
    // The same from/to the caller's row arrays (rows[k][j] = row j of field k:
    // rho, u, v, p, E), read and written by the GPU itself; only where the
    // device accesses pageable host memory coherently (host_rows_mode()).
    virtual int upload_rows(const double* const* const rows[5]) = 0;
    virtual int download_rows(double* const* const rows[5]) = 0;
    // The same through the host staging pair (host_pair()): host threads pack
    // a block of rows, converted to the state's precision, into one buffer
    // while the previous block is copied from the other into the pitched
    // state planes (and the reverse on the way out).
    virtual int upload_rows_staged(const double* const* const rows[5]) = 0;
    virtual int download_rows_staged(double* const* const rows[5]) = 0;
    // Runs the plan; snapshots (if any) are written as 5 x-major planes
    // (rho,u,v,p,E) each into snap_out[nt] (host memory, may be null).
    virtual int run(const RunConfig& rc, int split, int stats, const double* time_plot, int N_plot, int N_T,
                    double** snap_out, hydro_run_info* info, int* final_nt) = 0;
    virtual int num_variants() const = 0;
    virtual int set_variant(int v) = 0;
    virtual int get_variant() const = 0;
    virtual void variant_shape(int v, int* shape) const = 0;
    virtual int autotune(const RunConfig& rc, int steps, float* times_ms) = 0;
    virtual int set_mlp(const float* params) = 0;
    virtual int conservation(double hx, double hy, double* out4) = 0;
    int m = 0, n = 0, form = 0;
    int rs = 0;  // interface solver (HYDRO_SOLVER_*)
};

Solver2DBase* make_solver2d_f64(int m, int n, int rs);
Solver2DBase* make_solver2d_f32(int m, int n, int learned, int rs);

// Which of the scheme entry points' row copies the GPU makes itself, reading
// or writing the caller's malloc'd rows (Grace-Blackwell address translation):
// bit 0 the upload, bit 1 the download; 0 where the current device does not
// access pageable host memory coherently.  HYDRO_DIRECT_HOST_ROWS picks it:
// 0 none, 1 both, "in" the upload only; unset, the upload only where the
// GPU walks the host's page tables (address translation services), else none.
int host_rows_mode();

// Two host buffers for the scheme entry points' row copies, pinned where the
// driver grants it (else ordinary memory), kept for the life of the process;
// the lock serialises their users.
struct HostPair {
    void* buf[2];
    size_t bytes;
    cudaEvent_t ev[2];
    std::mutex lock;
};
HostPair* host_pair();
// Runs fn(r0, r1) over [0, rows) on several host threads when the block is
// large (bytes of host memory it touches).
void parallel_range(int rows, size_t bytes, const std::function<void(int, int)>& fn);

// error reporting + launch counting shared by all TUs
void set_error(const std::string& msg);
void count_launch(unsigned long long k = 1);
bool cuda_ok(cudaError_t e, const char* what);

}  // namespace hydro
