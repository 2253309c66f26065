// mf2d.cu -- the two-component GRP interface flux for a batch of faces.
//
// GRP_2D_flux of the reference's MULTIFLUID_BASICS build
// (src/flux_calc/flux_solver.c:158-237) for independent faces: one thread per
// face, the interface solver of mf.cuh.  The batch is laid out field by field
// (struct-of-arrays: in[k * nface + f], out[k * nface + f]) so that every load
// and store of a warp is one coalesced transaction; the field order follows the
// reference's struct i_f_var members (src/include/var_struc.h:116-142).
//
// Compiled with --fmad=false: the FP64 arithmetic rounds as the reference's C
// code does (pow is the C library's method of libm_pow.cuh).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "mf.cuh"
#include "solver2d.h"

namespace hydro {

struct MfParams {
    double tau, eps, gamma_a, gamma_b;
    int store_gamma;
};

// Input field indices (per face): normal, then per side gamma, the 12
// gas-dynamic values and slopes, and the 6 scalar values and slopes.
enum : int {
    MF_NX = 0, MF_NY = 1, MF_L = 2, MF_R = 21, MF_SIDE = 19, MF_NIN = 40, MF_NOUT = 18
};

__device__ __forceinline__ void mf_load_side(const double* __restrict__ in, size_t nf, size_t f, int base,
                                             Gas<double>& G, Side<double>& S, MfScal& X, double eps)
{
    auto ld = [&](int k) { return __ldg(in + (size_t)(base + k) * nf + f); };
    gas_fill(G, ld(0), eps);
    S.rho = ld(1); S.u = ld(2); S.v = ld(3); S.p = ld(4);
    S.drho = ld(5); S.du = ld(6); S.dv = ld(7); S.dp = ld(8);
    S.trho = ld(9); S.tu = ld(10); S.tv = ld(11); S.tp = ld(12);
    X.z = ld(13); X.dz = ld(14); X.tz = ld(15);
    X.phi = ld(16); X.dphi = ld(17); X.tphi = ld(18);
}

// Faces whose exact solve is still iterating at a pass's cap, with their
// Newton state, for the next pass.  nreg regions of `stride` entries each (the
// first pass sorts the faces into one region per wave pattern), count[r] the
// entries of region r.
struct MfQueue {
    int* face;
    double* p;
    int* it;  // iterations done | wave pattern << 16
    int* count;
    int nreg;
    size_t stride;
};

// Iteration caps of the passes.  The first pass (cap 0) completes the uniform
// pairs and sorts every other face by its wave pattern (1-wave rarefaction or
// shock, 3-wave rarefaction or shock), so that the next pass runs warps of
// faces that take the same branches: a warp pays each FP64 instruction in full
// whatever the number of its lanes on that path.  Most faces then converge in
// under ten Newton iterations, but about one in a hundred random faces never
// reaches the absolute tolerance and runs the reference's full 500: in one
// pass a warp would wait for its slowest face, so each pass stops at its cap
// and queues the unfinished faces, which the next pass resumes side by side.
constexpr int MF_NPASS = 5;
constexpr int MF_CAPS[MF_NPASS] = {0, 6, 16, 64, 500};
constexpr int MF_NREG = 4;  // wave patterns
constexpr int MF_NCOUNT = MF_NREG + (MF_NPASS - 2);  // queue counts of all passes but the last

// One face: load, rotate into the face frame (:172-189; the scalars are not
// rotated), solve, assemble.  Returns true when the solve was stopped at cap
// (NW holds its progress; nothing is written).  status[f]: star_dire_check's
// code (1 non-positive, 2 non-finite t-axis value, 3 non-finite derivative, 0
// fine); the outputs are assembled either way.  bad[0] counts the faces with a
// non-zero code, bad[1] is the smallest such index.
__device__ __forceinline__ bool mf_face(const double* __restrict__ in, size_t nf, size_t f, const MfParams& P,
                                        double* __restrict__ out, int* __restrict__ status, int* __restrict__ bad,
                                        int cap, bool resume, MfNewton& NW)
{
    const double n_x = __ldg(in + MF_NX * nf + f), n_y = __ldg(in + MF_NY * nf + f);
    Gas<double> GL, GR;
    Side<double> L, Rr;
    MfScal XL, XR;
    mf_load_side(in, nf, f, MF_L, GL, L, XL, P.eps);
    mf_load_side(in, nf, f, MF_R, GR, Rr, XR, P.eps);
    {
        const double u = L.u * n_x + L.v * n_y, u_R = Rr.u * n_x + Rr.v * n_y;
        const double d_u = L.du * n_x + L.dv * n_y, d_u_R = Rr.du * n_x + Rr.dv * n_y;
        const double t_u = L.tu * n_x + L.tv * n_y, t_u_R = Rr.tu * n_x + Rr.tv * n_y;
        L.v = -L.u * n_y + L.v * n_x;
        Rr.v = -Rr.u * n_y + Rr.v * n_x;
        L.dv = -L.du * n_y + L.dv * n_x;
        Rr.dv = -Rr.du * n_y + Rr.dv * n_x;
        L.tv = -L.tu * n_y + L.tv * n_x;
        Rr.tv = -Rr.tu * n_y + Rr.tv * n_x;
        L.u = u; Rr.u = u_R;
        L.du = d_u; Rr.du = d_u_R;
        L.tu = t_u; Rr.tu = t_u_R;
    }
    double D[4], U[4], DX[2], UX[2];
    if (mf_q1d(L, Rr, XL, XR, GL, GR, P.eps, D, U, DX, UX, cap, resume, NW))
        return true;
    const int rv = star_dire_check2<double>(U, D, P.eps);

    const double tau = P.tau;
    const double rho_mid = U[0] + 0.5 * tau * D[0];
    const double u_mid = (U[1] + 0.5 * tau * D[1]) * n_x - (U[2] + 0.5 * tau * D[2]) * n_y;
    const double v_mid = (U[1] + 0.5 * tau * D[1]) * n_y + (U[2] + 0.5 * tau * D[2]) * n_x;
    const double p_mid = U[3] + 0.5 * tau * D[3];
    const double phi_mid = UX[1] + 0.5 * tau * DX[1];
    const double z_a_mid = UX[0] + 0.5 * tau * DX[0];
    const double gamma_mid = 1.0 / (z_a_mid / (P.gamma_a - 1.0) + (1.0 - z_a_mid) / (P.gamma_b - 1.0)) + 1.0;

    const double F_rho = rho_mid * (u_mid * n_x + v_mid * n_y);
    const double F_e = (gamma_mid / (gamma_mid - 1.0)) * p_mid / rho_mid + 0.5 * (u_mid * u_mid + v_mid * v_mid);
    const double F_e_a = z_a_mid / (P.gamma_a - 1.0) * p_mid / rho_mid + 0.5 * phi_mid * (u_mid * u_mid + v_mid * v_mid);
    double o[MF_NOUT];
    o[0] = F_rho;
    o[1] = F_rho * u_mid + p_mid * n_x;
    o[2] = F_rho * v_mid + p_mid * n_y;
    o[3] = F_rho * F_e;
    o[4] = U[0] + tau * D[0];
    o[5] = (U[1] + tau * D[1]) * n_x - (U[2] + tau * D[2]) * n_y;
    o[6] = (U[1] + tau * D[1]) * n_y + (U[2] + tau * D[2]) * n_x;
    o[7] = U[3] + tau * D[3];
    o[8] = F_rho * phi_mid;
    o[9] = P.store_gamma ? F_rho * gamma_mid : 0.0;
    o[10] = F_rho * F_e_a;
    o[11] = UX[1] + tau * DX[1];
    o[12] = UX[0] + tau * DX[0];
    o[13] = F_rho * u_mid * phi_mid;
    o[14] = F_rho * v_mid * phi_mid;
    o[15] = p_mid * n_x;
    o[16] = p_mid * n_y;
    o[17] = p_mid / rho_mid * F_rho;
#pragma unroll
    for (int k = 0; k < MF_NOUT; ++k)
        __stcs(out + (size_t)k * nf + f, o[k]);
    status[f] = rv;
    if (rv) {
        atomicAdd(&bad[0], 1);
        atomicMin(&bad[1], (int)f);
    }
    return false;
}

// One pass (grid-stride).  qin.face == nullptr: every face from the start;
// else the faces of qin (its count read on the device), resumed.  Faces
// stopped at cap go to qout (unused when cap reaches the reference's limit).
__global__ void __launch_bounds__(128) k_grp2d_flux_mf(int nface, const double* __restrict__ in,
                                                       double* __restrict__ out, int* __restrict__ status,
                                                       MfParams P, int* __restrict__ bad, MfQueue qin, MfQueue qout,
                                                       int cap)
{
    const size_t nf = (size_t)nface;
    const bool resume = qin.face != nullptr;
    // the input regions, concatenated: entry q of the pass is entry q - start[r] of region r
    size_t start[MF_NREG + 1];
    start[0] = 0;
    for (int r = 0; r < MF_NREG; ++r)
        start[r + 1] = start[r] + ((resume && r < qin.nreg) ? (size_t)qin.count[r] : 0);
    const size_t n = resume ? start[MF_NREG] : nf;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        MfNewton NW = {0.0, 0, 0};
        size_t f = q;
        if (resume) {
            int r = 0;
            while (q >= start[r + 1])
                ++r;
            const size_t e = (size_t)r * qin.stride + (q - start[r]);
            f = (size_t)qin.face[e];
            NW.p = qin.p[e];
            NW.it = qin.it[e] & 0xffff;
            NW.crw = qin.it[e] >> 16;
        }
        // (no face stops in the last pass: its cap is the reference's limit)
        if (mf_face(in, nf, f, P, out, status, bad, cap, resume, NW) && qout.face) {
            const int r = qout.nreg > 1 ? (NW.crw & 3) : 0;
            const size_t e = (size_t)r * qout.stride + (size_t)atomicAdd(qout.count + r, 1);
            qout.face[e] = (int)f;
            qout.p[e] = NW.p;
            qout.it[e] = NW.it | NW.crw << 16;
        }
    }
}

// Device buffers of the host entry point, kept between calls (grow only).
struct MfBuffers {
    std::mutex lock;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    double* in = nullptr;
    double* out = nullptr;
    int* status = nullptr;
    int* bad = nullptr;     // failing-face count, first index, faces left by each pass
    MfQueue q[2] = {};      // alternating queues of unfinished faces (face, p, it arrays only)
    size_t cap = 0;  // faces

    bool ensure(size_t n)
    {
        if (!stream) {
            if (!cuda_ok(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream")) return false;
            if (!cuda_ok(cudaEventCreate(&ev[0]), "event") || !cuda_ok(cudaEventCreate(&ev[1]), "event")) return false;
            if (!cuda_ok(cudaMalloc(&bad, (2 + MF_NCOUNT) * sizeof(int)), "alloc")) return false;
        }
        if (n <= cap)
            return true;
        cudaFree(in);
        cudaFree(out);
        cudaFree(status);
        in = out = nullptr;
        status = nullptr;
        for (auto& Q : q) {
            cudaFree(Q.face);
            cudaFree(Q.p);
            cudaFree(Q.it);
            Q.face = Q.it = nullptr;
            Q.p = nullptr;
        }
        cap = 0;
        if (!cuda_ok(cudaMalloc(&in, sizeof(double) * MF_NIN * n), "alloc faces") ||
            !cuda_ok(cudaMalloc(&out, sizeof(double) * MF_NOUT * n), "alloc fluxes") ||
            !cuda_ok(cudaMalloc(&status, sizeof(int) * n), "alloc status"))
            return false;
        // q[0] receives the first pass's faces in one region per wave pattern
        for (int k = 0; k < 2; ++k) {
            const size_t entries = (k == 0 ? MF_NREG : 1) * n;
            if (!cuda_ok(cudaMalloc(&q[k].face, sizeof(int) * entries), "alloc queue") ||
                !cuda_ok(cudaMalloc(&q[k].p, sizeof(double) * entries), "alloc queue") ||
                !cuda_ok(cudaMalloc(&q[k].it, sizeof(int) * entries), "alloc queue"))
                return false;
        }
        cap = n;
        return true;
    }
};

static MfBuffers& mf_buffers()
{
    static MfBuffers b;
    return b;
}

// The passes of one batch on stream s; bad[0 .. 1 + MF_NCOUNT] must hold
// {0, INT_MAX, 0, ...}: failing faces, first failing index, then the number of
// faces the first pass queues per wave pattern and each later pass but the
// last leaves to the next.
static int launch_grp2d_flux_mf(int nface, const double* d_in, double* d_out, int* d_status, const MfParams& P,
                                int* d_bad, MfQueue q[2], cudaStream_t s)
{
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks_needed = ((long long)nface + 127) / 128;
    const long long gcap = (long long)sms * 16;
    const int grid = (int)(blocks_needed < gcap ? blocks_needed : gcap);
    const MfQueue none = {nullptr, nullptr, nullptr, nullptr, 0, 0};
    // the queue arrays alternate; each pass's output counts have their own
    // slots after d_bad[0..1] (MF_NREG for the first pass, one for each later
    // one), so nothing needs resetting between passes
    auto queue_of = [&](int pass) {
        MfQueue r = q[pass & 1];
        r.nreg = pass == 0 ? MF_NREG : 1;
        r.stride = (size_t)nface;
        r.count = d_bad + 2 + (pass == 0 ? 0 : MF_NREG + pass - 1);
        return r;
    };
    for (int pass = 0; pass < MF_NPASS; ++pass) {
        const MfQueue qin = pass == 0 ? none : queue_of(pass - 1);
        const MfQueue qout = pass == MF_NPASS - 1 ? none : queue_of(pass);
        k_grp2d_flux_mf<<<grid, 128, 0, s>>>(nface, d_in, d_out, d_status, P, d_bad, qin, qout, MF_CAPS[pass]);
        count_launch();
        if (!cuda_ok(cudaGetLastError(), "k_grp2d_flux_mf"))
            return -1;
    }
    return 0;
}

// Device to host copy of `bytes` into the caller's (pageable) memory through
// the pinned staging pair: each 64 MB block lands in a pinned buffer while host
// threads move the previous block into place (a pageable copy goes through the
// driver's own staging at a fraction of the link's speed).
static int download_staged(void* dst, const void* src, size_t bytes, cudaStream_t s)
{
    HostPair* hp = host_pair();
    if (!hp)
        return -1;
    std::lock_guard<std::mutex> guard(hp->lock);
    const size_t CH = hp->bytes;
    const size_t nchunk = (bytes + CH - 1) / CH;
    auto issue = [&](size_t c) -> bool {
        const size_t off = c * CH, len = bytes - off < CH ? bytes - off : CH;
        return cuda_ok(cudaMemcpyAsync(hp->buf[c & 1], static_cast<const char*>(src) + off, len,
                                       cudaMemcpyDeviceToHost, s),
                       "download") &&
               cuda_ok(cudaEventRecord(hp->ev[c & 1], s), "staging event");
    };
    if (nchunk == 0)
        return 0;
    if (!issue(0))
        return -1;
    for (size_t c = 0; c < nchunk; ++c) {
        if (c + 1 < nchunk && !issue(c + 1))
            return -1;
        if (!cuda_ok(cudaEventSynchronize(hp->ev[c & 1]), "download wait"))
            return -1;
        const size_t off = c * CH, len = bytes - off < CH ? bytes - off : CH;
        const char* from = static_cast<const char*>(hp->buf[c & 1]);
        char* to = static_cast<char*>(dst) + off;
        const int parts = 64;
        parallel_range(parts, len, [&](int r0, int r1) {
            const size_t a = len * (size_t)r0 / parts, b = len * (size_t)r1 / parts;
            memcpy(to + a, from + a, b - a);
        });
    }
    return 0;
}

// Host to device copy of `bytes` from the caller's (pageable) memory through
// the pinned staging pair: host threads fill one pinned buffer while the other
// is on its way to the device.  A buffer is refilled only after its previous
// copy has completed (its event).
static int upload_staged(void* dst, const void* src, size_t bytes, cudaStream_t s)
{
    HostPair* hp = host_pair();
    if (!hp)
        return -1;
    std::lock_guard<std::mutex> guard(hp->lock);
    const size_t CH = hp->bytes;
    const size_t nchunk = (bytes + CH - 1) / CH;
    for (size_t c = 0; c < nchunk; ++c) {
        const size_t off = c * CH, len = bytes - off < CH ? bytes - off : CH;
        if (c >= 2 && !cuda_ok(cudaEventSynchronize(hp->ev[c & 1]), "upload wait"))
            return -1;
        char* to = static_cast<char*>(hp->buf[c & 1]);
        const char* from = static_cast<const char*>(src) + off;
        const int parts = 64;
        parallel_range(parts, len, [&](int r0, int r1) {
            const size_t a = len * (size_t)r0 / parts, b = len * (size_t)r1 / parts;
            memcpy(to + a, from + a, b - a);
        });
        if (!cuda_ok(cudaMemcpyAsync(static_cast<char*>(dst) + off, to, len, cudaMemcpyHostToDevice, s), "upload") ||
            !cuda_ok(cudaEventRecord(hp->ev[c & 1], s), "staging event"))
            return -1;
    }
    // the buffers are free again once the last copies are done
    return cuda_ok(cudaStreamSynchronize(s), "upload sync") ? 0 : -1;
}

}  // namespace hydro

using namespace hydro;

extern "C" int hydro_grp2d_flux_mf(int nface, const double* in, double* out, int* status, const double* cfg,
                                   int ncfg, double tau, hydro_face_info* info)
{
    if (info)
        memset(info, 0, sizeof(*info));
    if (nface < 0 || (nface > 0 && (!in || !out || !status))) {
        set_error("hydro_grp2d_flux_mf: bad arguments");
        return -2;
    }
    if (info)
        info->first_bad = -1;
    if (nface == 0)
        return 0;
    // config[] entries the flux reads; an entry beyond ncfg is the reference's
    // default (INFINITY, src/file_io/config_handle.c)
    auto conf = [&](int k) { return (cfg && k < ncfg) ? cfg[k] : INFINITY; };
    MfParams P;
    P.tau = tau;
    P.eps = conf(4);
    P.gamma_a = conf(6);
    P.gamma_b = conf(106);
    P.store_gamma = conf(60) != 0.0;  // (_Bool)config[60]: NaN and INFINITY count as set

    MfBuffers& B = mf_buffers();
    std::lock_guard<std::mutex> guard(B.lock);
    if (!B.ensure((size_t)nface))
        return -1;
    const size_t nf = (size_t)nface;
    int init_bad[2 + MF_NCOUNT] = {0, 0x7fffffff};
    if (!cuda_ok(cudaMemcpyAsync(B.bad, init_bad, sizeof(init_bad), cudaMemcpyHostToDevice, B.stream), "upload") ||
        upload_staged(B.in, in, sizeof(double) * MF_NIN * nf, B.stream))
        return -1;
    cudaEventRecord(B.ev[0], B.stream);
    if (launch_grp2d_flux_mf(nface, B.in, B.out, B.status, P, B.bad, B.q, B.stream))
        return -1;
    cudaEventRecord(B.ev[1], B.stream);
    int bad[2 + MF_NCOUNT] = {0};
    if (download_staged(out, B.out, sizeof(double) * MF_NOUT * nf, B.stream) ||
        download_staged(status, B.status, sizeof(int) * nf, B.stream) ||
        !cuda_ok(cudaMemcpyAsync(bad, B.bad, sizeof(bad), cudaMemcpyDeviceToHost, B.stream), "download") ||
        !cuda_ok(cudaStreamSynchronize(B.stream), "flux sync"))
        return -1;
    if (info) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, B.ev[0], B.ev[1]);
        info->kernel_ms = ms;
        info->n_bad = bad[0];
        info->first_bad = bad[0] ? bad[1] : -1;
        info->first_code = bad[0] ? status[bad[1]] : 0;
        info->resumed[0] = 0;
        for (int r = 0; r < MF_NREG; ++r)
            info->resumed[0] += bad[2 + r];
        for (int k = 1; k < MF_NPASS - 1; ++k)
            info->resumed[k] = bad[2 + MF_NREG + k - 1];
    }
    return 0;
}
