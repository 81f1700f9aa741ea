// Batched ensembles: many independent eulerpsi or qg instances with their own
// grid sizes and masks advance together, one launch per kernel for all
// members.
//
// * Cells of all members are cut into 32x32 tiles (32 x 8 threads, four rows
//   each) listed in one tile table; each block of a batched kernel looks up
//   its (member, tile) and runs the same tile code as the single-model
//   kernels (stage_dev.cuh).
// * The Poisson/Helmholtz solves of all members run in one batched solver
//   (solver.cu): each member has its own multigrid hierarchy and CG state.
// * max|U| is reduced per member (per-tile maxima, combined in a fixed order
//   by one block per member); each member has its own CFL time step and
//   Kahan time.
// * Fields of all members live in one arena per field; member b starts at
//   element offset off_b (a multiple of 32 elements) with its own pitch.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fluids2d_gb300.h"
#include "mesh_host.h"
#include "solver.cuh"
#include "stage.cuh"
#include "stage_dev.cuh"

int f2d_internal_fail(int code, const char* msg);

namespace f2d {

struct Member {
    CUtensorMap tq[2];  // TMA maps of the two prognostic buffers (aligned as CUtensorMap)
    Geom g;
    long long off;      // element offset of the member in every arena
    double rdx2, rdy2;  // 1/dx**2, 1/dy**2
    float frdx2, frdy2;  // the same in FP32
    int t0, nt;         // range in the cell-tile table
    int n0, nn;         // range in the level-0 node-tile table
    int nl, ltail, ksweeps;
    int pad;
    long long poff;     // offset of the member's packed (NY, NX) array in the
                        // all-members host layout of f2d_ensemble_fields_*
};

struct EnsGlobals {
    int status;  // TMA time-outs of the stage kernels
    int pad;
};

// 1/dx**2, 1/dy**2 of a member in precision T (no conversion in the kernel)
template <typename T> struct Rd;
template <> struct Rd<double> {
    static __device__ __forceinline__ double x(const Member& m) { return m.rdx2; }
    static __device__ __forceinline__ double y(const Member& m) { return m.rdy2; }
};
template <> struct Rd<float> {
    static __device__ __forceinline__ float x(const Member& m) { return m.frdx2; }
    static __device__ __forceinline__ float y(const Member& m) { return m.frdy2; }
};

template <typename T>
__device__ __forceinline__ T* at(void* base, long long off)
{
    return (T*)base + off;
}

// ---- stage and diagnostics --------------------------------------------------
struct EnsArenas {
    void *q[2], *ds1, *ds2, *Ux, *Uy, *rhs, *psi, *fv;
    // the warm start of the stage solves (WarmArrays, stage.cuh): psi at the
    // step start and of stage 1, the previous step's stage increments
    double *psi_s0, *psi_p1, *psi_d1, *psi_d2;
    const uint32_t* code;
};

template <typename T, int M>
__global__ void __launch_bounds__(TX * TY, sizeof(T) == 4 ? 5 : 3)
k_ens_fluxform_stage(const int4* __restrict__ tiles, const Member* __restrict__ mem,
                     EnsArenas a, int par, int stage, DevScalars* scs, EnsGlobals* eg)
{
    __shared__ FluxformSmem<T, M> sm;
    const int4 tl = tiles[blockIdx.x];
    const Member& mb = mem[tl.x];
    const long long o = mb.off;
    const int k = stage & 15;  // stage = k | integrator << 4
    const DevScalars& sc = scs[tl.x];
    // LFRA: one stage; the filtered previous state alternates between the
    // tendency arenas with the parity (in: ds1 at parity 0, out: the other)
    const bool lf = ((stage >> 4) & 15) == 3;
    if (lf && sc.ite == 0) stage |= 256;
    void* pin = lf && par ? a.ds2 : a.ds1;
    void* pout = lf ? (par ? a.ds1 : a.ds2) : k < 3 ? (k == 1 ? a.ds1 : a.ds2) : nullptr;
    fluxform_tile<T, M>(sm, &mb.tq[par], at<T>(a.q[par], o), at<T>(a.q[1 - par], o),
                        at<T>(a.Ux, o), at<T>(a.Uy, o), a.code + o,
                        pout ? at<T>(pout, o) : nullptr, at<T>(pin, o), at<T>(a.ds2, o),
                        (const T*)nullptr, stage, mb.g, sc.dt, sc.ragamma, &eg->status,
                        tl.y, tl.z);
}

// Warm start of the solve of RK3 stage mode+1 (psi_warm_point, stage.cuh) on
// every member's array (all P x NY elements: the pads are 0 and stay 0),
// with the member's own step-size ratio: blockIdx.y is the member, the
// blocks of a member stride over its elements in 16-byte pairs, two pairs
// per thread and pass (the member arrays start 32-element aligned, P is
// even). Mode 2 also records the
// member's dt_warm (block 0 of the member; mode 2 reads no dt_warm).
__global__ void __launch_bounds__(256) k_ens_psi_warm(const Member* __restrict__ mem,
                                                       EnsArenas a, int mode, DevScalars* scs)
{
    const Member& mb = mem[blockIdx.y];
    const Geom g = mb.g;
    DevScalars& sc = scs[blockIdx.y];
    const bool hist = sc.dt_warm > 0.0;
    const double rho = hist ? sc.dt / sc.dt_warm : 0.0;
    WarmArrays w;
    w.psi = at<double>(a.psi, mb.off);
    w.s0 = a.psi_s0 + mb.off;
    w.p1 = a.psi_p1 + mb.off;
    w.d1 = a.psi_d1 + mb.off;
    w.d2 = a.psi_d2 + mb.off;
    const long long n = g.P * (long long)g.NY;
    // pairs of elements, two pairs per thread and pass (see psi_warm_pairs)
    constexpr int U = 2;
    const long long step = 2ll * gridDim.x * blockDim.x;
    for (long long k0 = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x); k0 < n;
         k0 += U * step) {
        long long k[U];
        bool ok[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            k[u] = k0 + u * step;
            ok[u] = k[u] < n;
        }
        psi_warm_pairs<U>(mode, w, k, ok, hist, rho);
    }
    if (mode == 2 && blockIdx.x == 0 && threadIdx.x == 0) sc.dt_warm = sc.dt;
}

// centerstovertices (+ beta-plane term) into the FP64 right-hand side
template <typename Tin>
__global__ void k_ens_c2v(const int4* __restrict__ tiles, const Member* __restrict__ mem,
                          EnsArenas a, int par, int use_fv)
{
    const int4 tl = tiles[blockIdx.x];
    const Member& mb = mem[tl.x];
    const Geom g = mb.g;
    const int i = tl.y + threadIdx.x;
    if (i >= g.NX) return;
    const Tin* q = at<Tin>(a.q[par], mb.off);
    const uint32_t* code = a.code + mb.off;
    const double* fv = use_fv ? at<double>(a.fv, mb.off) : nullptr;
    double* rhs = at<double>(a.rhs, mb.off);
    // every load of the thread's rows is issued before any is used (clamped
    // indices, the mask applied after): one memory round trip, not one per
    // row and condition
    uint32_t cd[FRT];
    Tin a0[FRT], a1[FRT], a2[FRT], a3[FRT];
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int j = min(tl.z + threadIdx.y + 8 * r, g.NY - 1);
        const int jm = max(j - 1, 0), im = max(i - 1, 0);
        const long long o = (long long)j * g.P + i, om = (long long)jm * g.P;
        cd[r] = code[o];
        a0[r] = q[om + im];                  // (j-1, i-1)
        a1[r] = q[(long long)j * g.P + im];  // (j, i-1)
        a2[r] = q[om + i];                   // (j-1, i)
        a3[r] = q[o];                        // (j, i)
    }
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int j = tl.z + threadIdx.y + 8 * r;
        if (j >= g.NY) break;
        const long long o = (long long)j * g.P + i;
        Tin s = Tin(0);  // the average in the precision of the state
        if (j >= 1 && i >= 1 && (cd[r] & B_MSKV))
            s = Tin(0.25) * (((a0[r] + a1[r]) + a2[r]) + a3[r]);
        double v = conv<double>(s);
        if (fv) v -= fv[o];
        rhs[o] = v;
    }
}

// perpgrad (contravariant) from FP64 psi, optional halo fill, per-member max|U|
template <typename T>
__global__ void k_ens_perpgrad(const int4* __restrict__ tiles, const Member* __restrict__ mem,
                               EnsArenas a, int fillU, DevScalars* scs, double* partials)
{
    const int4 tl = tiles[blockIdx.x];
    const Member& mb = mem[tl.x];
    const Geom g = mb.g;
    T m[2] = {T(0), T(0)};
    // the member's constants and pointers in registers (stores through Ux, Uy
    // could alias the member table, which would reload them after each)
    const long long moff = mb.off;
    const T rx = Rd<T>::x(mb), ry = Rd<T>::y(mb);
    T* Ux = at<T>(a.Ux, moff);
    T* Uy = at<T>(a.Uy, moff);
    const uint32_t* code = a.code + moff;
    // the loads of all the thread's rows first (clamped indices), then the
    // masked differences: one memory round trip
    const double* psi = at<double>(a.psi, moff);
    const int ic = min(tl.y + threadIdx.x, g.NX - 1);
    uint32_t cdv[FRT];
    double p0[FRT], pn[FRT], pe[FRT];
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int jc = min(tl.z + threadIdx.y + 8 * r, g.NY - 1);
        const long long o = (long long)jc * g.P + ic;
        cdv[r] = code[o];
        p0[r] = psi[o];
        pn[r] = psi[(long long)min(jc + 1, g.NY - 1) * g.P + ic];
        pe[r] = psi[(long long)jc * g.P + min(ic + 1, g.NX - 1)];
    }
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int i = tl.y + threadIdx.x, j = tl.z + threadIdx.y + 8 * r;
        if (j >= g.NY || i >= g.NX) continue;
        const long long o = (long long)j * g.P + i;
        const bool own = !fillU || periodic_owner(g, i);
        if (own) {
            // FP64 difference, scaling in the precision of U
            const uint32_t cd = cdv[r];
            T ux = T(0), uy = T(0);
            if (j <= g.NY - 2 && (cd & B_MSKX)) ux = -conv<T>(pn[r] - p0[r]) * ry;
            if (i <= g.NX - 2 && (cd & B_MSKY)) uy = conv<T>(pe[r] - p0[r]) * rx;
            if (fillU) {
                store_filled(Ux, g, j, i, ux);
                store_filled(Uy, g, j, i, uy);
            } else {
                Ux[o] = ux;
                Uy[o] = uy;
            }
            m[0] = nanmax(m[0], fabs(ux));
            m[1] = nanmax(m[1], fabs(uy));
        }
    }
    // the tile's maxima only (no fence or ticket: k_ens_umax combines a
    // member's tiles)
    (void)scs;
    double w[2];
    if constexpr (std::is_same<T, float>::value) {
        block_total_f<2, true>(m, w);
    } else {
        __shared__ double sh[64];
        w[0] = m[0];
        w[1] = m[1];
        block_reduce<2, true>(w, sh);
    }
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        partials[2 * (size_t)blockIdx.x] = w[0];
        partials[2 * (size_t)blockIdx.x + 1] = w[1];
    }
}

// every member's max|U.x|, max|U.y| from k_ens_perpgrad's tile maxima (the
// member's tiles t0 .. t0+nt), one block per member; NaN propagates
__global__ void __launch_bounds__(256) k_ens_umax(const Member* __restrict__ mem,
                                                   DevScalars* scs,
                                                   const double* __restrict__ partials)
{
    const Member& mb = mem[blockIdx.x];
    double acc[2];
    final_sum<2, true>(acc, partials, mb.t0, mb.nt, threadIdx.x, blockDim.x);
    __shared__ double sh[64];
    block_reduce<2, true>(acc, sh);
    if (threadIdx.x == 0) {
        scs[blockIdx.x].maxUx = acc[0];
        scs[blockIdx.x].maxUy = acc[1];
    }
}

__global__ void k_ens_fill_psi(const Member* __restrict__ mem, EnsArenas a, int nmem)
{
    const int b = blockIdx.x;
    const Member& mb = mem[b];
    const Geom g = mb.g;
    if (!g.xper) return;
    double* x = at<double>(a.psi, mb.off);
    for (int t = threadIdx.x; t < g.NY * 6; t += blockDim.x) {
        const int j = t / 6, k = t % 6;
        const long long r = (long long)j * g.P;
        if (k < 3) x[r + k] = x[r + g.NX - 6 + k];
        else x[r + g.NX - 6 + k] = x[r + k];
    }
}

__global__ void k_ens_set_dt(DevScalars* scs, int n, EnsGlobals* eg)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    DevScalars& s = scs[b];
    const double dt = pymin(s.cfl / (s.maxUx + s.maxUy + 1e-99), s.dtmax);
    s.dt = dt;
    if (!(dt == dt)) atomicOr(&eg->status, ST_NONFINITE);  // a NaN velocity
}

__global__ void k_ens_pushforward(DevScalars* scs, int n)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    DevScalars& s = scs[b];
    const double y = s.dt - s.c;
    const double t = s.t + y;
    s.c = (t - s.t) - y;
    s.t = t;
    s.ite += 1;
}

// ---- host side ----------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 ens_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)ptr;
    }
    return fn;
}

}  // namespace f2d

using namespace f2d;

struct f2d_ensemble_s {
    f2d_params p;
    int n = 0, prec = 0;
    size_t es = 8;
    cudaStream_t stream = nullptr, s2 = nullptr;
    bool own_stream = false;
    std::vector<Member> hmem;
    std::vector<void*> allocs;
    Member* dmem = nullptr;
    DevScalars* scs = nullptr;
    EnsGlobals* eg = nullptr;
    double* partials = nullptr;
    int4* cell_tiles = nullptr;
    int ncell = 0;
    size_t total = 0;  // elements per arena
    size_t packed = 0;  // elements of all members' packed (NY, NX) arrays
    double* io64 = nullptr;  // device copy of the packed layout (lazy)
    EnsArenas ar;
    BatchSolver bs;
    void* code = nullptr;
    void* gmask = nullptr;
    void* stage64 = nullptr;
    int cur = 0;
    cudaGraphExec_t gx[2][2] = {};  // [diag, run][parity]
    int launches[2] = {0, 0};
    int rec = 0;
};

#define ECK(call)                                                                     \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return f2d_internal_fail((int)e_, (std::string(#call) + ": " +           \
                                               cudaGetErrorString(e_)).c_str());      \
    } while (0)

static void* ens_alloc(f2d_ensemble_s* e, size_t bytes)
{
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    e->allocs.push_back(p);
    return p;
}

static bool ens_eager()
{
    static int v = -1;
    if (v < 0) {
        const char* x = getenv("F2D_EAGER");
        v = (x && *x && *x != '0') ? 1 : 0;
    }
    return v == 1;
}

static int ens_record_solve(f2d_ensemble_s* e, cudaStream_t s)
{
    e->bs.v.x64 = e->ar.psi;
    e->bs.v.b64 = e->ar.rhs;
    int fixed = 0;
    int r = bs_record(e->bs, s, e->s2, &fixed);
    if (r) return f2d_internal_fail(r, "ensemble Poisson solve recording failed");
    k_ens_fill_psi<<<e->n, 256, 0, s>>>(e->dmem, e->ar, e->n);
    e->rec += fixed + 1;
    return 0;
}

// warm: the warm start of the solve of RK3 stage warm+1 (launch_psi_warm,
// all members at once: they step in lockstep, so member 0's step count is
// everyone's); warm < 0: the previous solution as it is
static int ens_record_diag(f2d_ensemble_s* e, int par, cudaStream_t s, int warm = -1)
{
    const dim3 blk(32, 8);
    const int use_fv = e->p.model == F2D_MODEL_QG && e->p.beta != 0;
    if (e->prec == 0)
        k_ens_c2v<double><<<e->ncell, blk, 0, s>>>(e->cell_tiles, e->dmem, e->ar, par, use_fv);
    else
        k_ens_c2v<float><<<e->ncell, blk, 0, s>>>(e->cell_tiles, e->dmem, e->ar, par, use_fv);
    e->rec += 1;
    if (warm >= 0) {
        k_ens_psi_warm<<<dim3(48, e->n), 256, 0, s>>>(e->dmem, e->ar, warm, e->scs);
        e->rec += 1;
    }
    int r = ens_record_solve(e, s);
    if (r) return r;
    const int fillU = e->p.model == F2D_MODEL_EULERPSI;
    if (e->prec == 0)
        k_ens_perpgrad<double><<<e->ncell, blk, 0, s>>>(e->cell_tiles, e->dmem, e->ar, fillU,
                                                        e->scs, e->partials);
    else
        k_ens_perpgrad<float><<<e->ncell, blk, 0, s>>>(e->cell_tiles, e->dmem, e->ar, fillU,
                                                       e->scs, e->partials);
    k_ens_umax<<<e->n, 256, 0, s>>>(e->dmem, e->scs, e->partials);
    e->rec += 2;
    ECK(cudaGetLastError());
    return 0;
}

static int ens_record_step(f2d_ensemble_s* e, int par, cudaStream_t s)
{
    const dim3 blk(32, 8);
    k_ens_set_dt<<<(e->n + 127) / 128, 128, 0, s>>>(e->scs, e->n, e->eg);
    e->rec += 1;
    const int nst = e->p.integrator == F2D_INTEG_EF || e->p.integrator == F2D_INTEG_LFRA
                        ? 1 : 3;  // odd: flips the parity
    for (int k = 1; k <= nst; ++k) {
        const int sk = k | (e->p.integrator << 4);
#define ENS_FF(T, M)                                                                       \
    k_ens_fluxform_stage<T, M><<<e->ncell, blk, 0, s>>>(e->cell_tiles, e->dmem, e->ar, par, \
                                                        sk, e->scs, e->eg)
        const int M = e->p.compflux;
        if (e->prec == 0) {
            if (M == METHOD_WENO) ENS_FF(double, METHOD_WENO);
            else if (M == METHOD_UPWIND) ENS_FF(double, METHOD_UPWIND);
            else if (M == METHOD_CENTERED) ENS_FF(double, METHOD_CENTERED);
            else ENS_FF(double, METHOD_CWENO);
        } else {
            if (M == METHOD_WENO) ENS_FF(float, METHOD_WENO);
            else if (M == METHOD_UPWIND) ENS_FF(float, METHOD_UPWIND);
            else if (M == METHOD_CENTERED) ENS_FF(float, METHOD_CENTERED);
            else ENS_FF(float, METHOD_CWENO);
        }
#undef ENS_FF
        e->rec += 1;
        par = 1 - par;
        int r = ens_record_diag(e, par, s, e->p.integrator == F2D_INTEG_RK3 ? k - 1 : -1);
        if (r) return r;
    }
    k_ens_pushforward<<<(e->n + 127) / 128, 128, 0, s>>>(e->scs, e->n);
    e->rec += 1;
    ECK(cudaGetLastError());
    return 0;
}

static int ens_run_graph(f2d_ensemble_s* e, int kind)
{
    const int par = e->cur;
    if (ens_eager()) {
        e->rec = 0;
        int r = kind == 0 ? ens_record_diag(e, par, e->stream) : ens_record_step(e, par, e->stream);
        if (r) return r;
        e->launches[kind] = e->rec;
        if (kind == 1) e->cur = 1 - par;
        return 0;
    }
    if (!e->gx[kind][par]) {
        e->rec = 0;
        ECK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed));
        int r = kind == 0 ? ens_record_diag(e, par, e->stream) : ens_record_step(e, par, e->stream);
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
        if (r) {
            if (graph) cudaGraphDestroy(graph);
            return r;
        }
        ECK(ce);
        cudaGraphExec_t ex;
        ce = cudaGraphInstantiate(&ex, graph, 0);
        cudaGraphDestroy(graph);
        ECK(ce);
        e->gx[kind][par] = ex;
        e->launches[kind] = e->rec;
    }
    ECK(cudaGraphLaunch(e->gx[kind][par], e->stream));
    if (kind == 1) e->cur = 1 - par;
    return 0;
}

static void* ens_field(f2d_ensemble_s* e, const char* name, int* es)
{
    const bool pv = e->p.model == F2D_MODEL_QG;
    *es = (int)e->es;
    if (!strcmp(name, pv ? "pv" : "omega")) return e->ar.q[e->cur];
    if (!strcmp(name, "U.x")) return e->ar.Ux;
    if (!strcmp(name, "U.y")) return e->ar.Uy;
    *es = 8;
    if (!strcmp(name, "psi")) return e->ar.psi;
    if (!strcmp(name, pv ? "work" : "vomega")) return e->ar.rhs;
    return nullptr;
}

namespace f2d {
int tma_wait_test_set_ensemble(int enabled, unsigned long long limit_ns)
{
    TmaWaitTest v;
    v.enabled = enabled ? 1u : 0u;
    v.pad = 0;
    v.limit_ns = limit_ns;
    return (int)cudaMemcpyToSymbol(g_tma_wait_test, &v, sizeof(v));
}
}  // namespace f2d

extern "C" {

int f2d_ensemble_create(const f2d_params* p, int count, const int* nxs, const int* nys,
                        const int8_t* const* msks, f2d_ensemble* out)
{
    if (!p || !nxs || !nys || !out || count < 1)
        return f2d_internal_fail(1, "bad ensemble arguments");
    if (p->model != F2D_MODEL_EULERPSI && p->model != F2D_MODEL_QG)
        return f2d_internal_fail(1, "ensembles run the eulerpsi and qg models");
    if (p->tracer) return f2d_internal_fail(1, "ensembles carry no tracer equation");
    if (p->integrator < F2D_INTEG_RK3 || p->integrator > F2D_INTEG_LFRA)
        return f2d_internal_fail(1, "unknown integrator (rk3, ef, enrk3, LFRA)");
    if (p->dt > 0)
        return f2d_internal_fail(1, "ensembles use the per-member CFL time step (dt = 0)");
    auto* e = new f2d_ensemble_s();
    e->p = *p;
    e->n = count;
    e->prec = p->precision == F2D_PREC_FP64 ? 0 : 1;
    e->es = e->prec == 0 ? 8 : 4;
    auto bail = [&](int code) {
        f2d_ensemble_destroy(e);
        return code;
    };
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e->s2, cudaStreamNonBlocking) != cudaSuccess)
        return bail(f2d_internal_fail(2, "stream creation failed"));
    e->own_stream = true;
    // member geometry and arena offsets
    std::vector<MeshHost> meshes(count);
    e->hmem.resize(count);
    size_t off = 0, poff = 0;
    for (int b = 0; b < count; ++b) {
        f2d_params q = *p;
        q.nx = nxs[b];
        q.ny = nys[b];
        std::string err;
        if (mesh_build_host(q, msks ? msks[b] : nullptr, meshes[b], err))
            return bail(f2d_internal_fail(7, ("member " + std::to_string(b) + ": " + err).c_str()));
        Member& mb = e->hmem[b];
        memset(&mb, 0, sizeof(mb));
        Geom& g = mb.g;
        g.ny = q.ny;
        g.nx = q.nx;
        g.NY = q.ny + 6;
        g.NX = q.nx + 6;
        g.P = (g.NX + 15) / 16 * 16;
        g.xper = q.xperiodic ? 1 : 0;
        mb.off = (long long)off;
        mb.poff = (long long)poff;
        poff += (size_t)g.NX * g.NY;
        const double dx = q.Lx / q.nx, dy = q.Ly / q.ny;
        mb.rdx2 = 1 / pow(dx, 2.0);
        mb.rdy2 = 1 / pow(dy, 2.0);
        mb.frdx2 = (float)mb.rdx2;
        mb.frdy2 = (float)mb.rdy2;
        off += ((size_t)g.P * g.NY + 31) / 32 * 32;
    }
    e->total = off;
    e->packed = poff;
    const size_t es = e->es;
    auto A = [&](size_t bytes_per) { return ens_alloc(e, e->total * bytes_per); };
    e->ar.q[0] = A(es);
    e->ar.q[1] = A(es);
    e->ar.ds1 = A(es);
    e->ar.ds2 = A(es);
    e->ar.Ux = A(es);
    e->ar.Uy = A(es);
    e->ar.rhs = A(8);
    e->ar.psi = A(8);
    e->ar.psi_s0 = (double*)A(8);
    e->ar.psi_p1 = (double*)A(8);
    e->ar.psi_d1 = (double*)A(8);
    e->ar.psi_d2 = (double*)A(8);
    e->ar.fv = A(8);
    e->code = A(4);
    e->gmask = A(1);
    BSVecs v;
    memset(&v, 0, sizeof(v));
    v.x64 = e->ar.psi;
    v.b64 = e->ar.rhs;
    v.nelem = (long long)e->total;
    v.r64 = A(8);
    v.p = A(8);
    v.p2 = A(8);
    v.q = A(8);
    v.z = A(es);
    v.za = A(es);
    v.rin = e->prec == 0 ? v.r64 : A(4);
    e->stage64 = A(8);
    e->scs = (DevScalars*)ens_alloc(e, sizeof(DevScalars) * count);
    e->eg = (EnsGlobals*)ens_alloc(e, sizeof(EnsGlobals));
    for (void* q : {e->ar.q[0], e->ar.q[1], e->ar.ds1, e->ar.ds2, e->ar.Ux, e->ar.Uy,
                    e->ar.rhs, e->ar.psi, (void*)e->ar.psi_s0, (void*)e->ar.psi_p1,
                    (void*)e->ar.psi_d1, (void*)e->ar.psi_d2,
                    e->ar.fv, e->code, e->gmask, v.r64, v.p, v.p2, v.q, v.z, v.za,
                    v.rin, e->stage64, (void*)e->scs, (void*)e->eg})
        if (!q) return bail(f2d_internal_fail(2, "out of device memory for the ensemble"));
    e->ar.code = (const uint32_t*)e->code;
    // codes, masks, TMA maps, solver descriptors per member
    auto enc = ens_encode_fn();
    if (!enc) return bail(f2d_internal_fail(3, "cuTensorMapEncodeTiled unavailable"));
    std::vector<int4> cells;
    std::vector<BSMemberDesc> descs(count);
    std::vector<std::vector<uint8_t>> hmasks(count);
    for (int b = 0; b < count; ++b) {
        Member& mb = e->hmem[b];
        const Geom& g = mb.g;
        const MeshHost& M = meshes[b];
        std::vector<uint32_t> code((size_t)g.P * g.NY, 0);
        std::vector<uint8_t>& gm = hmasks[b];
        gm.assign((size_t)g.P * g.NY, 0);
        for (int j = 0; j < g.NY; ++j)
            for (int i = 0; i < g.NX; ++i) {
                code[(size_t)j * g.P + i] = M.code[(size_t)j * g.NX + i];
                gm[(size_t)j * g.P + i] = M.gv[(size_t)j * g.NX + i] >= 0;
            }
        if (cudaMemcpy((uint32_t*)e->code + mb.off, code.data(), code.size() * 4,
                       cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy((uint8_t*)e->gmask + mb.off, gm.data(), gm.size(),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(f2d_internal_fail(2, "mask upload failed"));
        for (int k = 0; k < 2; ++k) {
            cuuint64_t dims[2] = {(cuuint64_t)g.NX, (cuuint64_t)g.NY};
            cuuint64_t strides[1] = {(cuuint64_t)(g.P * es)};
            cuuint32_t box[2] = {(cuuint32_t)SW, (cuuint32_t)FSH};
            cuuint32_t estr[2] = {1, 1};
            CUresult r = enc(&mb.tq[k],
                             e->prec == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                          : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                             2, (char*)e->ar.q[k] + mb.off * es, dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return bail(f2d_internal_fail(3, "tensor map encode failed"));
        }
        // solver descriptor: node (J,I) of level 0 at arena offset off0 + J*P + I
        const double dx = p->Lx / g.nx, dy = p->Ly / g.ny, area = dx * dy;
        BSMemberDesc& d = descs[b];
        d.nyn = g.ny + 1;
        d.nxn = g.xper ? g.nx : g.nx + 1;
        d.pitch = g.P;
        d.off0 = mb.off + 3 * g.P + 3;
        d.per = g.xper;
        d.hmask = gm.data();
        d.hoff0 = 3 * g.P + 3;
        d.cx = dy / dx;
        d.cy = dx / dy;
        d.maindiag = p->model == F2D_MODEL_QG ? area * pow(p->f0, 2.0) / (p->g * p->H) : 0.0;
        // cell tiles
        mb.t0 = (int)cells.size();
        for (int j0 = 0; j0 < g.NY; j0 += FTY)
            for (int i0 = 0; i0 < g.NX; i0 += TX) cells.push_back(make_int4(b, i0, j0, 0));
        mb.nt = (int)cells.size() - mb.t0;
    }
    {
        int r = bs_build(e->bs, descs, (const uint8_t*)e->gmask, e->prec, v, e->scs);
        if (r) return bail(f2d_internal_fail(r, "ensemble multigrid set-up failed"));
        e->bs.tol = p->poisson_tol;
        e->bs.maxit = p->poisson_maxit;
        // default schedule (the autotuner may change tol_in and nu)
        e->bs.tol_in = 1e-6;
        e->bs.maxouter = std::max(2, p->poisson_maxit / 10);
        e->bs.nu = 2;
    }
    e->ncell = (int)cells.size();
    e->cell_tiles = (int4*)ens_alloc(e, cells.size() * sizeof(int4));
    e->partials = (double*)ens_alloc(e, (cells.size() * 2 + 64) * sizeof(double));
    e->dmem = (Member*)ens_alloc(e, sizeof(Member) * count);
    if (!e->cell_tiles || !e->partials || !e->dmem)
        return bail(f2d_internal_fail(2, "out of device memory"));
    cudaMemcpy(e->cell_tiles, cells.data(), cells.size() * sizeof(int4), cudaMemcpyHostToDevice);
    cudaMemcpy(e->dmem, e->hmem.data(), sizeof(Member) * count, cudaMemcpyHostToDevice);
    // time lines
    std::vector<DevScalars> hs(count);
    for (auto& h : hs) {
        memset(&h, 0, sizeof(h));
        h.dt = 0.01;
        h.cfl = p->cfl;
        h.dtmax = p->dtmax;
        h.ragamma = p->ragamma;
    }
    cudaMemcpy(e->scs, hs.data(), sizeof(DevScalars) * count, cudaMemcpyHostToDevice);
    if (cudaDeviceSynchronize() != cudaSuccess)
        return bail(f2d_internal_fail(2, "ensemble set-up failed"));
    *out = e;
    return 0;
}

int f2d_ensemble_destroy(f2d_ensemble e)
{
    if (!e) return 0;
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto& k : e->gx)
        for (auto& x : k)
            if (x) cudaGraphExecDestroy(x);
    bs_free(e->bs);
    for (void* p : e->allocs) cudaFree(p);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    if (e->s2) cudaStreamDestroy(e->s2);
    delete e;
    return 0;
}

int f2d_ensemble_set_stream(f2d_ensemble e, void* stream)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    ECK(cudaStreamSynchronize(e->stream));
    if (e->own_stream) cudaStreamDestroy(e->stream);
    if (stream) {
        e->stream = (cudaStream_t)stream;
        e->own_stream = false;
    } else {
        ECK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        e->own_stream = true;
    }
    return 0;
}

static int ens_io(f2d_ensemble e, int b, const char* name, double* host, bool set, bool async)
{
    if (!e || !name || !host) return f2d_internal_fail(1, "null argument");
    if (b < 0 || b >= e->n) return f2d_internal_fail(1, "member index out of range");
    int es = 8;
    void* base = ens_field(e, name, &es);
    if (!base && set && !strcmp(name, "f")) {  // vertex Coriolis term of member b
        base = e->ar.fv;
        es = 8;
    }
    if (!base) return f2d_internal_fail(8, (std::string("no ensemble field ") + name).c_str());
    const Member& mb = e->hmem[b];
    const Geom& g = mb.g;
    char* d = (char*)base + mb.off * es;
    char* d64 = es == 8 ? d : (char*)e->stage64;
    if (set) {
        ECK(cudaMemcpy2DAsync(d64, g.P * 8, host, g.NX * 8, g.NX * 8, g.NY,
                              cudaMemcpyHostToDevice, e->stream));
        if (es == 4) {
            int r = launch_convert(0, 1, d64, d, g, e->stream);
            if (r) return f2d_internal_fail(r, "conversion failed");
        }
    } else {
        if (es == 4) {
            int r = launch_convert(1, 0, d, d64, g, e->stream);
            if (r) return f2d_internal_fail(r, "conversion failed");
        }
        ECK(cudaMemcpy2DAsync(host, g.NX * 8, d64, g.P * 8, g.NX * 8, g.NY,
                              cudaMemcpyDeviceToHost, e->stream));
    }
    if (!async) ECK(cudaStreamSynchronize(e->stream));
    return 0;
}

int f2d_ensemble_field_set(f2d_ensemble e, int member, const char* name, const double* host)
{
    return ens_io(e, member, name, (double*)host, true, false);
}
int f2d_ensemble_field_get(f2d_ensemble e, int member, const char* name, double* host)
{
    return ens_io(e, member, name, host, false, false);
}
int f2d_ensemble_field_set_async(f2d_ensemble e, int member, const char* name,
                                 const double* host)
{
    return ens_io(e, member, name, (double*)host, true, true);
}
int f2d_ensemble_field_get_async(f2d_ensemble e, int member, const char* name, double* host)
{
    return ens_io(e, member, name, host, false, true);
}

// All members' field at once: between the arena (pitched, precision T) and
// the packed FP64 layout (member b's (NY, NX) array at poff_b), one cell
// tile (32 columns x FTY rows) per block
extern "C++" {
template <typename T, bool SET>
__global__ void k_ens_pack(const int4* __restrict__ tiles, const Member* __restrict__ mem,
                           T* arena, double* packed)
{
    const int4 tl = tiles[blockIdx.x];
    const Member& mb = mem[tl.x];
    const int i = tl.y + threadIdx.x;
    if (i >= mb.g.NX) return;
#pragma unroll
    for (int q = 0; q < FTY / 8; ++q) {
        const int j = tl.z + threadIdx.y + 8 * q;
        if (j >= mb.g.NY) break;
        const long long a = mb.off + (long long)j * mb.g.P + i;
        const long long k = mb.poff + (long long)j * mb.g.NX + i;
        if (SET) arena[a] = (T)packed[k];
        else packed[k] = (double)arena[a];
    }
}
}  // extern "C++"

static int ens_io_all(f2d_ensemble e, const char* name, double* host, bool set, bool async)
{
    if (!e || !name || !host) return f2d_internal_fail(1, "null argument");
    int es = 8;
    void* base = ens_field(e, name, &es);
    if (!base) return f2d_internal_fail(8, (std::string("no ensemble field ") + name).c_str());
    if (!e->io64) {
        e->io64 = (double*)ens_alloc(e, e->packed * sizeof(double));
        if (!e->io64) return f2d_internal_fail(2, "out of device memory");
    }
    const size_t bytes = e->packed * sizeof(double);
    const dim3 blk(32, 8);
#define ENS_PACK(T, SET)                                                                 \
    k_ens_pack<T, SET><<<e->ncell, blk, 0, e->stream>>>(e->cell_tiles, e->dmem, (T*)base, \
                                                          e->io64)
    if (set) {
        ECK(cudaMemcpyAsync(e->io64, host, bytes, cudaMemcpyHostToDevice, e->stream));
        if (es == 8) ENS_PACK(double, true);
        else ENS_PACK(float, true);
    } else {
        if (es == 8) ENS_PACK(double, false);
        else ENS_PACK(float, false);
        ECK(cudaMemcpyAsync(host, e->io64, bytes, cudaMemcpyDeviceToHost, e->stream));
    }
#undef ENS_PACK
    ECK(cudaGetLastError());
    if (!async) ECK(cudaStreamSynchronize(e->stream));
    return 0;
}

int f2d_ensemble_fields_set(f2d_ensemble e, const char* name, const double* host, int async)
{
    return ens_io_all(e, name, (double*)host, true, async != 0);
}
int f2d_ensemble_fields_get(f2d_ensemble e, const char* name, double* host, int async)
{
    return ens_io_all(e, name, host, false, async != 0);
}
int64_t f2d_ensemble_packed_size(f2d_ensemble e)
{
    return e ? (int64_t)e->packed : -1;
}

int f2d_ensemble_diag(f2d_ensemble e)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    return ens_run_graph(e, 0);
}

int f2d_ensemble_autotune(f2d_ensemble e, int reps, int* th, int* nu, double* tol_in,
                          double* ms)
{
    if (!e || reps < 1) return f2d_internal_fail(1, "bad autotune arguments");
    // the right-hand side and solution of the current state
    int r = ens_run_graph(e, 0);
    if (r) return r;
    ECK(cudaStreamSynchronize(e->stream));
    BSTune t;
    memset(&t, 0, sizeof(t));
    const int err = bs_autotune(e->bs, e->stream, e->s2, e->ar.psi, e->ar.rhs,
                                e->total * sizeof(double), reps, &t);
    // the step and diagnostic graphs captured the previous schedule
    for (auto& k : e->gx)
        for (auto& g : k)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    if (err) return f2d_internal_fail(err, "multigrid autotune failed");
    if (th) *th = t.th;
    if (nu) *nu = t.nu;
    if (tol_in) *tol_in = t.tol_in;
    if (ms) *ms = t.ms;
    return 0;
}

int f2d_ensemble_run(f2d_ensemble e, int nsteps)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    for (int k = 0; k < nsteps; ++k) {
        int r = ens_run_graph(e, 1);
        if (r) return r;
    }
    return 0;
}

int f2d_ensemble_time_get(f2d_ensemble e, int member, double* t, double* dt, int64_t* ite)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    if (member < 0 || member >= e->n) return f2d_internal_fail(1, "member out of range");
    DevScalars h;
    ECK(cudaMemcpyAsync(&h, e->scs + member, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    if (t) *t = h.t;
    if (dt) *dt = h.dt;
    if (ite) *ite = h.ite;
    return 0;
}

int f2d_ensemble_sync(f2d_ensemble e)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    ECK(cudaStreamSynchronize(e->stream));
    EnsGlobals h;
    ECK(cudaMemcpy(&h, e->eg, sizeof(h), cudaMemcpyDeviceToHost));
    BSGlobals bg;
    ECK(cudaMemcpy(&bg, e->bs.eg, sizeof(bg), cudaMemcpyDeviceToHost));
    h.status |= bg.status;
    if (h.status) {
        int zero = 0;
        ECK(cudaMemcpy(&e->eg->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
        ECK(cudaMemcpy(&e->bs.eg->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
        std::string msg = "ensemble device status:";
        if (h.status & ST_TMA_TIMEOUT) msg += " TMA tile load timed out;";
        if (h.status & ST_STAGE_ALIGN) msg += " TMA staging buffer misaligned;";
        if (h.status & ST_PCG_MAXIT) msg += " a Poisson solve reached max iterations;";
        if (h.status & ST_NONFINITE) msg += " non-finite value (residual or time step);";
        return f2d_internal_fail(100 + h.status, msg.c_str());
    }
    return 0;
}

int f2d_ensemble_stats(f2d_ensemble e, int64_t* cells, int64_t* poisson_iters_sum,
                       int64_t* loop_iters, int64_t* launches_per_step,
                       int64_t* launches_per_iter)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    std::vector<DevScalars> h(e->n);
    ECK(cudaMemcpyAsync(h.data(), e->scs, sizeof(DevScalars) * e->n, cudaMemcpyDeviceToHost,
                        e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    int64_t c = 0, it = 0;
    for (int b = 0; b < e->n; ++b) {
        c += (int64_t)e->hmem[b].g.nx * e->hmem[b].g.ny;
        it += h[b].total_iters;
    }
    if (cells) *cells = c;
    if (poisson_iters_sum) *poisson_iters_sum = it;
    if (loop_iters) {
        BSGlobals g;
        ECK(cudaMemcpy(&g, e->bs.eg, sizeof(g), cudaMemcpyDeviceToHost));
        *loop_iters = g.loops_in;
    }
    if (launches_per_step) *launches_per_step = e->launches[1];
    if (launches_per_iter) *launches_per_iter = e->bs.body_launches;
    return 0;
}

int f2d_ensemble_set_schedule(f2d_ensemble e, int tile_rows, int sweeps, double tol_in)
{
    if (!e) return f2d_internal_fail(1, "null ensemble");
    ECK(cudaStreamSynchronize(e->stream));
    const int r = bs_set_schedule(e->bs, tile_rows, sweeps, tol_in);
    // the step and diagnostic graphs captured the previous schedule
    for (auto& k : e->gx)
        for (auto& g : k)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    if (r == 1)
        return f2d_internal_fail(1, "schedule: tile_rows 32 or 64, sweeps 1 or 2, 0 < tol_in < 1");
    if (r) return f2d_internal_fail(r, "ensemble multigrid rebuild failed");
    return 0;
}

int f2d_ensemble_refine_rounds(f2d_ensemble e, int64_t* rounds)
{
    if (!e || !rounds) return f2d_internal_fail(1, "null argument");
    std::vector<DevScalars> h(e->n);
    ECK(cudaMemcpyAsync(h.data(), e->scs, sizeof(DevScalars) * e->n, cudaMemcpyDeviceToHost,
                        e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    int64_t r = 0;
    for (int b = 0; b < e->n; ++b) r += h[b].total_outer;
    *rounds = r;
    return 0;
}

int f2d_ensemble_time_solver(f2d_ensemble e, int reps, int flush_l2, double* avg_ms,
                             int64_t* nodes, int* elem_bytes)
{
    if (!e || !avg_ms) return f2d_internal_fail(1, "null argument");
    ECK(cudaStreamSynchronize(e->stream));
    long long n = 0;
    int es = 0;
    int r = bs_time_down(e->bs, e->stream, reps, flush_l2, avg_ms, &n, &es);
    if (r) return f2d_internal_fail(r, "solver kernel timing failed (no grid level?)");
    if (nodes) *nodes = n;
    if (elem_bytes) *elem_bytes = es;
    return 0;
}

int f2d_ensemble_solver_pipelined(f2d_ensemble e, int* pipelined)
{
    if (!e || !pipelined) return f2d_internal_fail(1, "null argument");
    *pipelined = e->bs.pipe ? 1 : 0;
    return 0;
}

int f2d_ensemble_time_stage(f2d_ensemble e, int stage, int reps, int flush_l2,
                            double* avg_ms)
{
    if (!e || !avg_ms || reps < 1 || stage < 1 || stage > 3)
        return f2d_internal_fail(1, "bad arguments");
    const size_t flush_bytes = 256ull << 20;
    void* fl = nullptr;
    if (flush_l2) ECK(cudaMalloc(&fl, flush_bytes));
    cudaEvent_t a, b;
    ECK(cudaEventCreate(&a));
    ECK(cudaEventCreate(&b));
    double total = 0.0;
    const dim3 blk(32, 8);
    const int par = e->cur;
    for (int r = 0; r < reps; ++r) {
        if (fl) cudaMemsetAsync(fl, r & 0xff, flush_bytes, e->stream);
        cudaEventRecord(a, e->stream);
#define ENS_FF(T, M)                                                                       \
    k_ens_fluxform_stage<T, M><<<e->ncell, blk, 0, e->stream>>>(e->cell_tiles, e->dmem,   \
                                                                e->ar, par,               \
                                                                stage | (e->p.integrator << 4), \
                                                                e->scs,                   \
                                                                e->eg)
        const int M = e->p.compflux;
        if (e->prec == 0) {
            if (M == METHOD_WENO) ENS_FF(double, METHOD_WENO);
            else if (M == METHOD_UPWIND) ENS_FF(double, METHOD_UPWIND);
            else if (M == METHOD_CENTERED) ENS_FF(double, METHOD_CENTERED);
            else ENS_FF(double, METHOD_CWENO);
        } else {
            if (M == METHOD_WENO) ENS_FF(float, METHOD_WENO);
            else if (M == METHOD_UPWIND) ENS_FF(float, METHOD_UPWIND);
            else if (M == METHOD_CENTERED) ENS_FF(float, METHOD_CENTERED);
            else ENS_FF(float, METHOD_CWENO);
        }
#undef ENS_FF
        cudaEventRecord(b, e->stream);
        if (cudaEventSynchronize(b) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        total += ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (fl) cudaFree(fl);
    ECK(cudaGetLastError());
    *avg_ms = total / reps;
    return 0;
}

}  // extern "C"
