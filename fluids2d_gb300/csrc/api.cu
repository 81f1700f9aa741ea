// C ABI of the library (include/fluids2d_gb300.h): models (eulerpsi, rsw,
// qg, euler, boussinesq, qgrsw, with an optional tracer), fields, time
// stepping recorded once per parity into CUDA graphs (step, run, diagnostics,
// qg_projection, the adjoint's snapshot and adjoint steps), the Poisson and
// Neumann solves, the multigrid autotuner, Bulk diagnostics and float32
// snapshots.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/fluids2d_gb300.h"
#include "adjoint.cuh"
#include "mesh_host.h"
#include "nsolver.cuh"
#include "stage_dev.cuh"
#include "solver.cuh"
#include "stage.cuh"

namespace f2d {
int launch_compflux(int, double*, const double*, const double*, const int8_t*, long long,
                    long long, long long, cudaStream_t);
int launch_vortexforce(int, double*, const double*, const double*, const int8_t*,
                       long long, long long, int, long long, long long, cudaStream_t);
int launch_innerproduct(int, double*, const double*, const double*, const int8_t*,
                        long long, long long, long long, cudaStream_t);
}  // namespace f2d

using namespace f2d;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code ? code : 1;
}

// error reporting for the other translation units of the library
int f2d_internal_fail(int code, const char* msg) { return fail(code, msg); }

#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return fail((int)e_, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CKI(call)                                                  \
    do {                                                           \
        int e_ = (call);                                           \
        if (e_)                                                    \
            return fail(e_, std::string(#call) + ": " +            \
                                cudaGetErrorString((cudaError_t)e_)); \
    } while (0)

// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
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

struct Field {
    void* buf[2] = {nullptr, nullptr};
    bool pingpong = false;
    int es = 8;  // element size: 8 (FP64) or 4 (FP32)
};

// Workspace of the discrete adjoint (eulerpsi): checkpoints of the
// vorticity, the snapshot arena of one recomputed segment (3 stage states
// per step, each with its face velocities) and the FP64 adjoint fields.
struct AdjState {
    int nsteps = 0, every = 0, nckpt = 0, cap_every = 0;
    double dt = 0, dt_graph = 0;
    bool ready = false;
    std::vector<void*> ckpt;
    void* arena = nullptr;
    int* slot = nullptr;
    double *yb = nullptr, *d1 = nullptr, *d2 = nullptr, *d3 = nullptr;
    double *gx = nullptr, *gy = nullptr, *ubx = nullptr, *uby = nullptr;
    // psib: the adjoint Poisson right-hand side; rbs[k]: the adjoint solve's
    // solution for RK3 stage k+1, kept per stage so that each adjoint solve
    // starts from the same stage's solution of the step after it
    double *psib = nullptr, *rbs[3] = {nullptr, nullptr, nullptr};
    // the forward's streamfunction after every stage (slot 3n + k after
    // stage k of step n, slot 0 after the initial diagnostics), so that the
    // recompute of a segment needs no Poisson solve; used when it fits
    double* psic = nullptr;
    long long psic_slots = 0;
    int* pslot = nullptr;
    bool use_psic = false;
};

struct f2d_model_s {
    f2d_params p;
    Geom g;
    MeshHost mesh;
    int prec = 0;
    size_t es = 8;
    cudaStream_t stream = nullptr, s2 = nullptr;
    bool own_stream = false;
    uint32_t* d_code = nullptr;
    uint8_t* d_gmask = nullptr;
    void* d_fv = nullptr;  // mesh.f (qg beta-plane)
    DevScalars* sc = nullptr;
    double* partials = nullptr;
    // Bulk diagnostics ring (records of 5 doubles) and FP32 snapshot staging
    double* bulk_ring = nullptr;
    int* bulk_count = nullptr;
    double bulk_summsk = -1.0;  // domsum(msk), cached per mask
    float* f32_stage = nullptr;
    std::map<std::string, Field> fields;
    std::vector<void*> allocs;
    double dx, dy, area, rdx2, rdy2, goa, fc, maindiag, cx, cy, dt_const;
    bool cfl_dt = true;
    bool dt_applied = false;  // the constant dt of set_dt is in sc->dt
    // multigrid: [0] vertex Poisson, [1] Helmholtz
    BatchSolver bs[2];  // [0] vertex Poisson, [1] qg Helmholtz
    bool bs_ready[2] = {false, false};
    void *pr = nullptr, *pz = nullptr, *pp = nullptr, *pq = nullptr;
    void *pp2 = nullptr, *pza = nullptr;
    void* prmg = nullptr;  // V-cycle right-hand side (== pr in FP64)
    void* stage64 = nullptr;  // FP64 staging for field I/O of FP32 fields
    void *sb = nullptr, *sx = nullptr;  // scratch for f2d_poisson_solve
    std::map<void*, CUtensorMap> tmaps;
    int cur = 0;
    // graphs: [kind][parity]; kinds: 0 diag, 1 step, 2 run, 3 solve0, 4 solve1,
    // 5 step with adjoint snapshots, 6 adjoint step, 7 right-hand side alone,
    // 8-10 integrator stage 1-3 (with its diagnostics; the last stage of a
    // step also advances the time line), 11 step that caches the
    // streamfunction of every stage, 12 snapshot step that takes it from the
    // cache instead of solving
    cudaGraphExec_t gx[13][2] = {};
    int launches[13][2] = {};
    // prognostic variables (states.py:22-34 order) and whether the forcing
    // fields "frc.<var>" exist
    std::vector<std::string> prog;
    bool has_frc = false;
    AdjState adj;
    // euler: the Neumann cell-centred pressure solve and its right-hand side
    NSolver ns;
    bool ns_ready = false;
    double* nrhs = nullptr;
    int body_launches = 0;
    int rec_launches = 0;
};

static void* dalloc(f2d_model_s* m, size_t bytes)
{
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    m->allocs.push_back(p);
    return p;
}

// the models stepped in momentum-pressure form with the Neumann pressure
// projection (euler, boussinesq: equations.py:9-44)
static bool projected(int model)
{
    return model == F2D_MODEL_EULER || model == F2D_MODEL_BOUSSINESQ;
}

static size_t field_bytes(const f2d_model_s* m, size_t es)
{
    return (size_t)m->g.P * m->g.NY * es;
}

static int add_field(f2d_model_s* m, const char* name, bool pp, int es)
{
    Field f;
    f.pingpong = pp;
    f.es = es;
    for (int k = 0; k < (pp ? 2 : 1); ++k) {
        f.buf[k] = dalloc(m, field_bytes(m, es));
        if (!f.buf[k]) return fail(2, std::string("out of device memory for ") + name);
    }
    m->fields[name] = f;
    return 0;
}

static void* fb(f2d_model_s* m, const char* name, int parity = -1)
{
    auto it = m->fields.find(name);
    if (it == m->fields.end()) return nullptr;
    const Field& f = it->second;
    if (!f.pingpong) return f.buf[0];
    return f.buf[parity < 0 ? m->cur : parity];
}

static int field_es(f2d_model_s* m, const char* name)
{
    auto it = m->fields.find(name);
    return it == m->fields.end() ? 0 : it->second.es;
}

// TMA tile map of a stencil-state buffer (element size of the state)
static int make_tmap(f2d_model_s* m, void* buf, bool flux_tile = false)
{
    if (m->tmaps.count(buf)) return 0;
    auto fn = encode_fn();
    if (!fn) return fail(3, "cuTensorMapEncodeTiled is not available from the driver");
    CUtensorMap map;
    cuuint64_t dims[2] = {(cuuint64_t)m->g.NX, (cuuint64_t)m->g.NY};
    cuuint64_t strides[1] = {(cuuint64_t)(m->g.P * m->es)};
    // tile + halo: SW x FSH for the flux-form stage (and the tracer of any
    // model), SW x SH for the momentum kernel of rsw, euler and boussinesq
    cuuint32_t box[2] = {(cuuint32_t)SW,
                         (cuuint32_t)(!flux_tile && (m->p.model == F2D_MODEL_RSW ||
                                                     m->p.model == F2D_MODEL_QGRSW ||
                                                     projected(m->p.model))
                                          ? SH
                                          : FSH)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(&map, m->prec == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                       : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                    2, buf, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(3, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    m->tmaps[buf] = map;
    return 0;
}

static const CUtensorMap* tmap(f2d_model_s* m, void* buf) { return &m->tmaps[buf]; }

// ---------------------------------------------------------------------------
// Recording of diag / stage / step on a stream (eager or under capture).
// ---------------------------------------------------------------------------
static int ensure_mg(f2d_model_s* m, int which)
{
    if (m->bs_ready[which]) return 0;
    const Geom& g = m->g;
    std::vector<uint8_t> hm((size_t)g.P * g.NY, 0);
    for (int j = 0; j < g.NY; ++j)
        for (int i = 0; i < g.NX; ++i)
            hm[(size_t)j * g.P + i] = m->mesh.gv[(size_t)j * g.NX + i] >= 0 ? 1 : 0;
    // fluid vertices must lie in the node box (3+J, 3+I) of level 0
    const int nyn = g.ny + 1, nxn = g.xper ? g.nx : g.nx + 1;
    for (int j = 0; j < g.NY; ++j)
        for (int i = 0; i < g.NX; ++i)
            if (hm[(size_t)j * g.P + i] &&
                (j < 3 || j >= 3 + nyn || i < 3 || i >= 3 + nxn))
                return fail(4, "fluid vertex outside the interior (mask halo must be 0)");
    BSMemberDesc d;
    d.nyn = nyn;
    d.nxn = nxn;
    d.pitch = g.P;
    d.off0 = 3 * g.P + 3;
    d.per = g.xper;
    d.hmask = hm.data();
    d.hoff0 = 3 * g.P + 3;
    d.cx = m->cx;
    d.cy = m->cy;
    d.maindiag = which == 0 ? 0.0 : m->maindiag;
    BSVecs v;
    memset(&v, 0, sizeof(v));
    v.r64 = m->pr;
    v.p = m->pp;
    v.p2 = m->pp2;
    v.q = m->pq;
    v.z = m->pz;
    v.za = m->pza;
    v.rin = m->prmg;
    v.nelem = (long long)g.P * g.NY;
    BatchSolver& bs = m->bs[which];
    int e = bs_build(bs, {d}, m->d_gmask, m->prec, v, m->sc);
    if (e) return fail(e, "multigrid setup failed");
    bs.tol = m->p.poisson_tol;
    bs.maxit = m->p.poisson_maxit;
    // default schedule (the autotuner may change tol_in and nu)
    bs.tol_in = 1e-6;
    bs.maxit_in = 30;
    bs.maxouter = std::max(2, m->p.poisson_maxit / 10);
    bs.nu = 2;
    m->bs_ready[which] = true;
    return 0;
}

// the Neumann cell-centred solver of the euler model (Poisson2D(mesh, "c"),
// elliptic.py:71-87): fluid cells of vertex_msk(mesh, "c"), i.e. msk with the
// periodic halo columns removed, inside the interior box (3+J, 3+I)
static int ensure_ns(f2d_model_s* m)
{
    if (m->ns_ready) return 0;
    const Geom& g = m->g;
    std::vector<uint8_t> hm((size_t)g.P * g.NY, 0);
    for (int j = 3; j < 3 + g.ny; ++j)
        for (int i = 3; i < 3 + g.nx; ++i)
            hm[(size_t)j * g.P + i] = m->mesh.msk[(size_t)j * g.NX + i] ? 1 : 0;
    int e = ns_build(m->ns, g.ny, g.nx, g.P, 3 * (long long)g.P + 3, g.xper, hm.data(),
                     (double*)fb(m, "p"), m->nrhs, m->cx, m->cy, m->prec);
    if (e == 6) return fail(4, "the euler model needs at least one fluid cell");
    if (e) return fail(e, "Neumann multigrid setup failed");
    m->ns.tol = m->p.poisson_tol;
    m->ns.maxit = m->p.poisson_maxit;
    m->ns_ready = true;
    return 0;
}

static bool eager_mode();

static int rec_solve(f2d_model_s* m, int which, const void* b, void* x, cudaStream_t s)
{
    int e = ensure_mg(m, which);
    if (e) return e;
    BatchSolver& bs = m->bs[which];
    bs.v.x64 = x;
    bs.v.b64 = (void*)b;
    int fixed = 0;
    CKI(bs_record(bs, s, m->s2, &fixed));
    m->rec_launches += fixed;
    m->body_launches = bs.body_launches;
    if (m->g.xper) {
        CKI(launch_fill_periodic(0, x, m->g, s));  // psi is FP64
        m->rec_launches += 1;
    }
    return 0;
}

// the warm start of the solve of RK3 stage warm+1 (warm < 0: the previous
// solution as it is)
static int rec_warm(f2d_model_s* m, int warm, cudaStream_t s)
{
    if (warm < 0) return 0;
    WarmArrays w;
    w.psi = (double*)fb(m, "psi");
    w.s0 = (double*)fb(m, "psi.s0");
    w.p1 = (double*)fb(m, "psi.p1");
    w.d1 = (double*)fb(m, "psi.d1");
    w.d2 = (double*)fb(m, "psi.d2");
    CKI(launch_psi_warm(warm, w, (long long)m->g.P * m->g.NY, m->sc, s));
    m->rec_launches += 1;
    return 0;
}

static int rec_diag(f2d_model_s* m, int par, cudaStream_t s, int warm = -1)
{
    const Geom& g = m->g;
    switch (m->p.model) {
    case F2D_MODEL_EULERPSI: {
        CKI(launch_c2v(m->prec, 0, fb(m, "omega", par), fb(m, "vomega"), m->d_code, nullptr, g,
                       s));
        m->rec_launches += 1;
        int e = rec_warm(m, warm, s);
        if (e) return e;
        e = rec_solve(m, 0, fb(m, "vomega"), fb(m, "psi"), s);
        if (e) return e;
        CKI(launch_perpgrad(0, m->prec, fb(m, "psi"), fb(m, "U.x"), fb(m, "U.y"), m->d_code,
                            m->rdy2, m->rdx2, 1, g, m->sc, m->partials, s));
        m->rec_launches += 2;  // perpgrad + k_umax_finish
        return 0;
    }
    case F2D_MODEL_QG: {
        const void* fv = m->p.beta != 0 ? m->d_fv : nullptr;
        CKI(launch_c2v(m->prec, 0, fb(m, "pv", par), fb(m, "work"), m->d_code, fv, g, s));
        m->rec_launches += 1;
        int e = rec_warm(m, warm, s);
        if (e) return e;
        e = rec_solve(m, 1, fb(m, "work"), fb(m, "psi"), s);
        if (e) return e;
        CKI(launch_perpgrad(0, m->prec, fb(m, "psi"), fb(m, "U.x"), fb(m, "U.y"), m->d_code,
                            m->rdy2, m->rdx2, 0, g, m->sc, m->partials, s));
        m->rec_launches += 2;  // perpgrad + k_umax_finish
        return 0;
    }
    case F2D_MODEL_EULER:
    case F2D_MODEL_BOUSSINESQ: {
        // pressure_projection (operators.py:114-119), then sharp, vorticity,
        // kinetic energy (equations.py:17-22; the boussinesq diag, 37-43, is
        // the same: its fill(s.u) names no mesh and fills nothing)
        CKI(launch_euler_div(m->prec, fb(m, "u.x", par), fb(m, "u.y", par), fb(m, "div"),
                             m->nrhs, m->d_code, m->rdx2, m->rdy2, m->area, g, s));
        int e = ensure_ns(m);
        if (e) return e;
        int fixed = 0;
        CKI(ns_record(m->ns, s, m->s2, eager_mode(), &fixed));
        if (g.xper) CKI(launch_fill_periodic(0, fb(m, "p"), g, s));
        CKI(launch_euler_project(m->prec, fb(m, "u.x", par), fb(m, "u.y", par),
                                 (const double*)fb(m, "p"), m->d_code, g, s));
        m->rec_launches += 3 + fixed + (g.xper ? 1 : 0);
        RswDiag a;
        memset(&a, 0, sizeof(a));
        a.ux = fb(m, "u.x", par);
        a.uy = fb(m, "u.y", par);
        a.Ux = fb(m, "U.x");
        a.Uy = fb(m, "U.y");
        a.omega = fb(m, "omega");
        a.ke = fb(m, "ke");
        a.rdx2 = m->rdx2;
        a.rdy2 = m->rdy2;
        a.euler = 1;
        CKI(make_tmap(m, (void*)a.ux));
        CKI(make_tmap(m, (void*)a.uy));
        CKI(launch_rsw_diag(m->p.innerproduct, m->prec, tmap(m, (void*)a.ux),
                            tmap(m, (void*)a.uy), a, m->d_code, g, m->sc, s));
        // max|U.x|, max|U.y| for set_dt (model.py:83-85)
        CKI(launch_maxabs2(m->prec, a.Ux, a.Uy, g, m->sc, m->partials, s));
        m->rec_launches += 2;
        return 0;
    }
    case F2D_MODEL_QGRSW: {
        // sharp, vorticity and its fill (equations.py:127-133)
        RswDiag a;
        memset(&a, 0, sizeof(a));
        a.ux = fb(m, "u.x", par);
        a.uy = fb(m, "u.y", par);
        a.Ux = fb(m, "U.x");
        a.Uy = fb(m, "U.y");
        a.omega = fb(m, "omega");
        a.rdx2 = m->rdx2;
        a.rdy2 = m->rdy2;
        a.euler = 1;
        a.noke = 1;
        CKI(make_tmap(m, (void*)a.ux));
        CKI(make_tmap(m, (void*)a.uy));
        CKI(launch_rsw_diag(m->p.innerproduct, m->prec, tmap(m, (void*)a.ux),
                            tmap(m, (void*)a.uy), a, m->d_code, g, m->sc, s));
        // max|U.x|, max|U.y| for set_dt (model.py:83-85)
        CKI(launch_maxabs2(m->prec, a.Ux, a.Uy, g, m->sc, m->partials, s));
        m->rec_launches += 2;
        return 0;
    }
    case F2D_MODEL_RSW: {
        RswDiag a;
        memset(&a, 0, sizeof(a));
        a.ux = fb(m, "u.x", par);
        a.uy = fb(m, "u.y", par);
        a.h = fb(m, "h", par);
        a.Ux = fb(m, "U.x");
        a.Uy = fb(m, "U.y");
        a.omega = fb(m, "omega");
        a.ke = fb(m, "ke");
        a.p = fb(m, "p");
        a.rdx2 = m->rdx2;
        a.rdy2 = m->rdy2;
        a.goa = m->goa;
        CKI(make_tmap(m, (void*)a.ux));
        CKI(make_tmap(m, (void*)a.uy));
        CKI(launch_rsw_diag(m->p.innerproduct, m->prec, tmap(m, (void*)a.ux),
                            tmap(m, (void*)a.uy), a, m->d_code, g, m->sc, s));
        m->rec_launches += 1;
        return 0;
    }
    }
    return fail(5, "unknown model");
}

static int rec_qgrsw_stage(f2d_model_s* m, int k, int par, cudaStream_t s, bool tend);

// the forcing field of prognostic variable f (null without forcing)
static void* frc(f2d_model_s* m, const char* f)
{
    return m->has_frc ? fb(m, (std::string("frc.") + f).c_str()) : nullptr;
}

// the fused right-hand-side + RK3-update kernel of stage k, parity par -> 1-par;
// tend: the right-hand side alone (the reference's rhs(s, ds), with any
// forcing term) into the fields "rhs.<var>", the state untouched
static int launch_stage_kernel(f2d_model_s* m, int k, int par, cudaStream_t s,
                               bool tend = false)
{
    const Geom& g = m->g;
    const int out = 1 - par;
    const bool lf = m->p.integrator == F2D_INTEG_LFRA && !tend;
    const int sk = tend ? (1 | (INTEG_TENDENCY << 4)) : (k | (m->p.integrator << 4));
    auto ds = [&](const char* f, int kk) -> void* {
        return fb(m, (std::string("ds") + std::to_string(kk) + "." + f).c_str());
    };
    auto rhs = [&](const char* f) -> void* {
        return fb(m, (std::string("rhs.") + f).c_str());
    };
    if (m->p.model == F2D_MODEL_QGRSW) {
        // tendency, projection and update (counts its own launches)
        int e = rec_qgrsw_stage(m, k, par, s, tend);
        if (e) return e;
    } else if (m->p.model == F2D_MODEL_RSW || projected(m->p.model)) {
        // rsw; euler = the same momentum kernel without the mass equation,
        // Coriolis and pressure (equations.py:11-15); boussinesq = euler +
        // buoyancy + the flux divergence of b in the place of h (29-35)
        const bool eu = m->p.model == F2D_MODEL_EULER;
        const bool bq = m->p.model == F2D_MODEL_BOUSSINESQ;
        const char* hn = bq ? "b" : "h";
        RswIn a;
        memset(&a, 0, sizeof(a));
        a.euler = eu ? 1 : bq ? 2 : 0;
        a.bdy = 0.5 * m->dy;
        a.ux = fb(m, "u.x", par);
        a.uy = fb(m, "u.y", par);
        a.h = eu ? nullptr : fb(m, hn, par);
        a.uxo = fb(m, "u.x", out);
        a.uyo = fb(m, "u.y", out);
        a.ho = eu ? nullptr : fb(m, hn, out);
        a.Ux = fb(m, "U.x");
        a.Uy = fb(m, "U.y");
        a.ke = fb(m, "ke");
        a.p = fb(m, "p");
        // LFRA: the filtered previous state alternates between the two
        // tendency buffers with the parity (in: 1 + par, out: 2 - par)
        const int kin = lf ? 1 + par : 1, kout = lf ? 2 - par : k;
        if (tend) {
            a.dux = rhs("u.x");
            a.duy = rhs("u.y");
            a.dh = eu ? nullptr : rhs(hn);
        } else if (kout < 3) {
            a.dux = ds("u.x", kout);
            a.duy = ds("u.y", kout);
            a.dh = eu ? nullptr : ds(hn, kout);
        }
        a.fx = frc(m, "u.x");
        a.fy = frc(m, "u.y");
        a.fh = eu ? nullptr : frc(m, hn);
        a.dux1 = ds("u.x", kin);
        a.duy1 = ds("u.y", kin);
        a.dh1 = eu ? nullptr : ds(hn, kin);
        a.dux2 = ds("u.x", 2);
        a.duy2 = ds("u.y", 2);
        a.dh2 = eu ? nullptr : ds(hn, 2);
        a.fc = m->fc;
        void* om = fb(m, "omega");
        void* hm = eu ? om : (void*)a.h;  // euler stages no thickness tile
        CKI(make_tmap(m, hm));
        CKI(make_tmap(m, om));
        CKI(launch_rsw_stage(m->p.vortexforce, m->prec, tmap(m, hm), tmap(m, om), a,
                             m->d_code, sk, g, m->sc, s));
        m->rec_launches += 1;
    } else {
        const char* q = m->p.model == F2D_MODEL_EULERPSI ? "omega" : "pv";
        void* qin = fb(m, q, par);
        CKI(make_tmap(m, qin));
        CKI(launch_fluxform_stage(m->p.compflux, m->prec, tmap(m, qin), qin, fb(m, q, out),
                                  fb(m, "U.x"), fb(m, "U.y"), m->d_code,
                                  tend ? rhs(q) : lf ? ds(q, 2 - par) : k < 3 ? ds(q, k) : nullptr,
                                  ds(q, lf ? 1 + par : 1), ds(q, 2), frc(m, q), sk, g,
                                  m->sc, s));
        m->rec_launches += 1;
    }
    if (m->p.tracer) {
        // the passive tracer equation appended to the model's right-hand side
        // (addtracerequation, equations.py:217-226): divflux of the tracer
        // with the stage input's U, same integrator coefficients
        void* qin = fb(m, "tracer", par);
        CKI(make_tmap(m, qin, true));
        CKI(launch_fluxform_stage(m->p.compflux, m->prec, tmap(m, qin), qin,
                                  fb(m, "tracer", out), fb(m, "U.x"), fb(m, "U.y"), m->d_code,
                                  tend ? rhs("tracer")
                                       : lf ? ds("tracer", 2 - par)
                                            : k < 3 ? ds("tracer", k) : nullptr,
                                  ds("tracer", lf ? 1 + par : 1), ds("tracer", 2),
                                  frc(m, "tracer"), sk, g, m->sc, s));
        m->rec_launches += 1;
    }
    return 0;
}

// qgrsw stage (equations.py:106-125): the raw RSW tendency (vortex force,
// Coriolis, mass flux; momentum kernel in tendency mode), the vertex PV of it
// (vorticity + stretching), the Helmholtz solve, then the projected tendency
// (perpgrad, thickness) and the integrator update in one pass. The raw
// tendency lives in ds3, the projected one of stage k < 3 in ds<k> (LFRA:
// the filtered previous state alternates between ds1 and ds2 with the
// parity).
// the raw qgrsw tendency of stage k from parity par into ds3 (read by the
// projection pass while it writes the projected tendency of stage k < 3 into
// ds<k>): the momentum kernel in tendency mode
static int launch_qgrsw_tendency(f2d_model_s* m, int k, int par, cudaStream_t s)
{
    const int kt = 3;
    const int sk = k | (m->p.integrator << 4);
    auto ds = [&](const char* f, int kk) -> void* {
        return fb(m, (std::string("ds") + std::to_string(kk) + "." + f).c_str());
    };
    RswIn a;
    memset(&a, 0, sizeof(a));
    a.euler = 3;
    a.ux = fb(m, "u.x", par);
    a.uy = fb(m, "u.y", par);
    a.h = fb(m, "h", par);
    a.Ux = fb(m, "U.x");
    a.Uy = fb(m, "U.y");
    a.dux = ds("u.x", kt);
    a.duy = ds("u.y", kt);
    a.dh = ds("h", kt);
    a.fc = m->fc;
    void* om = fb(m, "omega");
    a.w = om;
    CKI(make_tmap(m, (void*)a.h));
    CKI(make_tmap(m, om));
    CKI(launch_rsw_stage(m->p.vortexforce, m->prec, tmap(m, (void*)a.h), tmap(m, om), a,
                         m->d_code, sk, m->g, m->sc, s));
    m->rec_launches += 1;
    return 0;
}

static int rec_qgrsw_stage(f2d_model_s* m, int k, int par, cudaStream_t s, bool tend)
{
    const Geom& g = m->g;
    const int out = 1 - par;
    const bool lf = m->p.integrator == F2D_INTEG_LFRA && !tend;
    const int kt = 3;
    const int sk = k | (m->p.integrator << 4);
    auto ds = [&](const char* f, int kk) -> void* {
        return fb(m, (std::string("ds") + std::to_string(kk) + "." + f).c_str());
    };
    int e0 = launch_qgrsw_tendency(m, k, par, s);
    if (e0) return e0;
    RswIn a;
    memset(&a, 0, sizeof(a));
    a.euler = 3;
    a.ux = fb(m, "u.x", par);
    a.uy = fb(m, "u.y", par);
    a.h = fb(m, "h", par);
    a.Ux = fb(m, "U.x");
    a.Uy = fb(m, "U.y");
    a.dux = ds("u.x", kt);
    a.duy = ds("u.y", kt);
    a.dh = ds("h", kt);
    // add_stretching's -f0/H (operators.py:199)
    const double cs = -m->p.f0 / m->p.H;
    CKI(launch_qgrsw_pv(m->prec, a.dux, a.duy, a.dh, (double*)fb(m, "pv"), m->d_code, cs, 0.0,
                        g, s));
    m->rec_launches += 1;
    int e = rec_solve(m, 1, fb(m, "pv"), fb(m, "psi"), s);
    if (e) return e;
    QgProj q;
    memset(&q, 0, sizeof(q));
    q.ux = a.ux;
    q.uy = a.uy;
    q.h = a.h;
    q.uxo = fb(m, "u.x", out);
    q.uyo = fb(m, "u.y", out);
    q.ho = fb(m, "h", out);
    q.cx = a.dux;
    q.cy = a.duy;
    q.ch = a.dh;
    if (tend) {
        q.sx = fb(m, "rhs.u.x");
        q.sy = fb(m, "rhs.u.y");
        q.sh = fb(m, "rhs.h");
    } else if (!lf && k < 3) {
        q.sx = ds("u.x", k);
        q.sy = ds("u.y", k);
        q.sh = ds("h", k);
    }
    q.fx = frc(m, "u.x");
    q.fy = frc(m, "u.y");
    q.fh = frc(m, "h");
    const int k1 = lf ? 1 + par : 1;
    q.d1x = ds("u.x", k1);
    q.d1y = ds("u.y", k1);
    q.d1h = ds("h", k1);
    q.d2x = ds("u.x", 2);
    q.d2y = ds("u.y", 2);
    q.d2h = ds("h", 2);
    if (lf) {
        q.px = ds("u.x", 2 - par);
        q.py = ds("u.y", 2 - par);
        q.ph = ds("h", 2 - par);
    }
    // thickness_from_psi's f0 * area / g (operators.py:208)
    q.c2 = m->p.f0 * m->area / m->p.g;
    q.mode = tend ? 2 : 0;
    q.store = !lf && k < 3 && !tend;
    CKI(launch_qgrsw_update(m->prec, q, (const double*)fb(m, "psi"), m->d_code, sk, g, m->sc,
                            s));
    m->rec_launches += 1;
    return 0;
}

// qg_projection (operators.py:176-183, anomaly=False) of the state at
// parity par in place: PV of (u, h - h0), Helmholtz solve into psi, then
// u = perpgrad(psi), h = verticestocenters(psi f0 area / g) + h0, times msk
static int rec_qg_projection(f2d_model_s* m, int par, cudaStream_t s)
{
    const Geom& g = m->g;
    const double h0 = m->p.H * m->area;  // H * area - hb, hb = 0 (meshes.py:47)
    void* ux = fb(m, "u.x", par);
    void* uy = fb(m, "u.y", par);
    void* h = fb(m, "h", par);
    CKI(launch_qgrsw_pv(m->prec, ux, uy, h, (double*)fb(m, "pv"), m->d_code,
                        -m->p.f0 / m->p.H, h0, g, s));
    m->rec_launches += 1;
    int e = rec_solve(m, 1, fb(m, "pv"), fb(m, "psi"), s);
    if (e) return e;
    QgProj q;
    memset(&q, 0, sizeof(q));
    q.cx = ux;
    q.cy = uy;
    q.ch = h;
    q.c2 = m->p.f0 * m->area / m->p.g;
    q.h0 = h0;
    q.mode = 1;
    CKI(launch_qgrsw_update(m->prec, q, (const double*)fb(m, "psi"), m->d_code, 1, g, m->sc,
                            s));
    m->rec_launches += 1;
    return 0;
}

// one RK3 stage from parity `par` to 1-par, then the diagnostics (the
// SSP-RK3 stages of eulerpsi and qg with the extrapolated warm start)
static int rec_stage(f2d_model_s* m, int k, int par, cudaStream_t s)
{
    int e = launch_stage_kernel(m, k, par, s);
    if (e) return e;
    const bool warm = m->p.integrator == F2D_INTEG_RK3 &&
                      (m->p.model == F2D_MODEL_EULERPSI || m->p.model == F2D_MODEL_QG);
    return rec_diag(m, 1 - par, s, warm ? k - 1 : -1);
}

static int nstages(const f2d_model_s* m)
{
    return m->p.integrator == F2D_INTEG_EF || m->p.integrator == F2D_INTEG_LFRA ? 1 : 3;
}

static int rec_step(f2d_model_s* m, int par, bool with_dt, cudaStream_t s)
{
    if (with_dt && m->cfl_dt) {
        CKI(launch_set_dt(m->sc, s));
        m->rec_launches += 1;
    }
    // SSP-RK3 / enrk3: 3 stages, ef and LFRA: 1 (an odd count: a step flips
    // the parity)
    const int nst = nstages(m);
    for (int k = 1; k <= nst; ++k) {
        int e = rec_stage(m, k, par, s);
        if (e) return e;
        par = 1 - par;
    }
    CKI(launch_pushforward(m->sc, s));
    m->rec_launches += 1;
    return 0;
}

// one step that first snapshots every stage state (w, U.x, U.y) into the
// adjoint arena (slot counter on the device, advanced per stage)
static int rec_step_snap(f2d_model_s* m, int par, cudaStream_t s)
{
    AdjState& a = m->adj;
    const long long fsz = (long long)m->g.P * m->g.NY;
    for (int k = 1; k <= 3; ++k) {
        CKI(launch_adj_snap(m->prec, fb(m, "omega", par), fb(m, "U.x"), fb(m, "U.y"), a.arena,
                            fsz, a.slot, s));
        CKI(launch_adj_slot(a.slot, 1, s));
        m->rec_launches += 2;
        int e = rec_stage(m, k, par, s);
        if (e) return e;
        par = 1 - par;
    }
    CKI(launch_pushforward(m->sc, s));
    m->rec_launches += 1;
    return 0;
}

// the eulerpsi diagnostics of a recomputed stage from the forward's cached
// streamfunction (slot *pslot, then advanced): perpgrad of it, no solve
static int rec_diag_cached(f2d_model_s* m, cudaStream_t s)
{
    AdjState& a = m->adj;
    const long long fsz = (long long)m->g.P * m->g.NY;
    CKI(launch_adj_psi((double*)fb(m, "psi"), a.psic, fsz, a.pslot, 0, s));
    CKI(launch_adj_slot(a.pslot, 1, s));
    CKI(launch_perpgrad(0, m->prec, fb(m, "psi"), fb(m, "U.x"), fb(m, "U.y"), m->d_code,
                        m->rdy2, m->rdx2, 1, m->g, m->sc, m->partials, s));
    m->rec_launches += 4;
    return 0;
}

// the forward's streamfunction into cache slot *pslot, then advanced
static int rec_psi_store(f2d_model_s* m, cudaStream_t s)
{
    AdjState& a = m->adj;
    const long long fsz = (long long)m->g.P * m->g.NY;
    CKI(launch_adj_psi((double*)fb(m, "psi"), a.psic, fsz, a.pslot, 1, s));
    CKI(launch_adj_slot(a.pslot, 1, s));
    m->rec_launches += 2;
    return 0;
}

// one forward step (fixed dt) that caches the streamfunction of every stage
static int rec_step_store(f2d_model_s* m, int par, cudaStream_t s)
{
    for (int k = 1; k <= 3; ++k) {
        int e = rec_stage(m, k, par, s);
        if (e) return e;
        if ((e = rec_psi_store(m, s))) return e;
        par = 1 - par;
    }
    CKI(launch_pushforward(m->sc, s));
    m->rec_launches += 1;
    return 0;
}

// the snapshot step of the recompute with the cached streamfunctions
static int rec_step_snap_cached(f2d_model_s* m, int par, cudaStream_t s)
{
    AdjState& a = m->adj;
    const long long fsz = (long long)m->g.P * m->g.NY;
    for (int k = 1; k <= 3; ++k) {
        CKI(launch_adj_snap(m->prec, fb(m, "omega", par), fb(m, "U.x"), fb(m, "U.y"), a.arena,
                            fsz, a.slot, s));
        CKI(launch_adj_slot(a.slot, 1, s));
        m->rec_launches += 2;
        int e = launch_stage_kernel(m, k, par, s);
        if (e) return e;
        if ((e = rec_diag_cached(m, s))) return e;
        par = 1 - par;
    }
    CKI(launch_pushforward(m->sc, s));
    m->rec_launches += 1;
    return 0;
}

// yb += D'(w)^T db for the stage state of snapshot slot (*slot + soff)
static int rec_adj_vjp(f2d_model_s* m, int soff, const double* db, cudaStream_t s)
{
    AdjState& a = m->adj;
    const Geom& g = m->g;
    const long long fsz = (long long)g.P * g.NY;
    CKI(launch_adj_vjp_pre(m->p.compflux, m->prec, g, m->d_code, a.arena, fsz, a.slot, soff, db,
                           a.gx, a.gy, a.ubx, a.uby, m->rdx2, m->rdy2, a.psib, s));
    m->rec_launches += 2;
    int e = rec_solve(m, 0, a.psib, a.rbs[soff], s);
    if (e) return e;
    CKI(launch_adj_vjp_post(g, m->d_code, a.gx, a.gy, fsz, a.rbs[soff], a.yb, s));
    m->rec_launches += 1;
    return 0;
}

// one adjoint RK3 step (integrators.py:92-107 reversed, fixed dt): the
// stages' snapshots are slots (*slot - 3) .. (*slot - 1)
static int rec_adj_step(f2d_model_s* m, cudaStream_t s)
{
    AdjState& a = m->adj;
    const Geom& g = m->g;
    const double dt = a.dt;
    CKI(launch_adj_slot(a.slot, -3, s));
    CKI(launch_adj_comb(g, a.yb, a.d1, a.d2, a.d3, 0, -dt / 12, -dt / 12, 2 * dt / 3, s));
    m->rec_launches += 2;
    int e = rec_adj_vjp(m, 2, a.d3, s);
    if (e) return e;
    CKI(launch_adj_comb(g, a.yb, a.d1, a.d2, a.d3, 1, -3 * dt / 4, dt / 4, 0, s));
    m->rec_launches += 1;
    e = rec_adj_vjp(m, 1, a.d2, s);
    if (e) return e;
    CKI(launch_adj_comb(g, a.yb, a.d1, a.d2, a.d3, 2, dt, 0, 0, s));
    m->rec_launches += 1;
    return rec_adj_vjp(m, 0, a.d1, s);
}

// F2D_EAGER=1 runs every recorded sequence directly on the stream (the
// Poisson loop then synchronises once per iteration): a profiling aid, since
// kernel profilers do not list kernels inside conditional graph nodes.
static bool eager_mode()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("F2D_EAGER");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

// integrator stage k alone (its right-hand side and update, then the
// diagnostics); the last stage of the step also advances the time line
static int rec_one_stage(f2d_model_s* m, int k, int par, cudaStream_t s)
{
    int e = rec_stage(m, k, par, s);
    if (e) return e;
    if (k == nstages(m)) {
        CKI(launch_pushforward(m->sc, s));
        m->rec_launches += 1;
    }
    return 0;
}

static int record_kind(f2d_model_s* m, int kind, int par, cudaStream_t s)
{
    switch (kind) {
    case 0: return rec_diag(m, par, s);
    case 1: return rec_step(m, par, false, s);
    case 2: return rec_step(m, par, true, s);
    case 3: return rec_qg_projection(m, par, s);
    case 5: return rec_step_snap(m, par, s);
    case 6: return rec_adj_step(m, s);
    case 7: return launch_stage_kernel(m, 1, par, s, true);
    case 11: return rec_step_store(m, par, s);
    case 12: return rec_step_snap_cached(m, par, s);
    case 8:
    case 9:
    case 10: return rec_one_stage(m, kind - 7, par, s);
    }
    return fail(1, "unknown graph kind");
}

static bool flips(int kind)
{
    return kind == 1 || kind == 2 || kind == 5 || (kind >= 8 && kind <= 10) || kind == 11 ||
           kind == 12;
}

// capture kind (0 diag, 1 step, 2 run, 3 qg projection of the state,
// 5 snapshot step, 6 adjoint step) for
// the current parity, then launch
static int run_graph(f2d_model_s* m, int kind)
{
    const int par = m->cur;
    if (eager_mode()) {
        if (m->p.model == F2D_MODEL_EULERPSI || m->p.model == F2D_MODEL_QG ||
            m->p.model == F2D_MODEL_QGRSW) {
            int e0 = ensure_mg(m, m->p.model == F2D_MODEL_EULERPSI ? 0 : 1);
            if (e0) return e0;
        } else if (projected(m->p.model)) {
            int e0 = ensure_ns(m);
            if (e0) return e0;
        }
        m->rec_launches = 0;
        int e = record_kind(m, kind, par, m->stream);
        if (e) return e;
        m->launches[kind][par] = m->rec_launches;
        if (flips(kind)) m->cur = 1 - par;
        return 0;
    }
    if (!m->gx[kind][par]) {
        // multigrid set-up allocates, so it happens before the capture
        if (m->p.model == F2D_MODEL_EULERPSI || m->p.model == F2D_MODEL_QG ||
            m->p.model == F2D_MODEL_QGRSW) {
            int e0 = ensure_mg(m, m->p.model == F2D_MODEL_EULERPSI ? 0 : 1);
            if (e0) return e0;
        } else if (projected(m->p.model)) {
            int e0 = ensure_ns(m);
            if (e0) return e0;
        }
        m->rec_launches = 0;
        CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeRelaxed));
        int e = record_kind(m, kind, par, m->stream);
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
        if (e) {
            if (graph) cudaGraphDestroy(graph);
            return e;
        }
        if (ce != cudaSuccess) return fail((int)ce, std::string("capture: ") + cudaGetErrorString(ce));
        cudaGraphExec_t ex;
        ce = cudaGraphInstantiate(&ex, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess)
            return fail((int)ce, std::string("graph instantiate: ") + cudaGetErrorString(ce));
        m->gx[kind][par] = ex;
        m->launches[kind][par] = m->rec_launches;
    }
    CK(cudaGraphLaunch(m->gx[kind][par], m->stream));
    if (flips(kind)) m->cur = 1 - par;  // three stages flip the parity
    return 0;
}

static void drop_graphs(f2d_model_s* m)
{
    for (auto& k : m->gx)
        for (auto& e : k)
            if (e) {
                cudaGraphExecDestroy(e);
                e = nullptr;
            }
}

static int setup_mesh(f2d_model_s* m, const int8_t* msk)
{
    std::string err;
    if (mesh_build_host(m->p, msk, m->mesh, err)) return fail(7, err);
    m->bulk_summsk = -1.0;
    const Geom& g = m->g;
    std::vector<uint32_t> code((size_t)g.P * g.NY, 0);
    std::vector<uint8_t> gm((size_t)g.P * g.NY, 0);
    for (int j = 0; j < g.NY; ++j)
        for (int i = 0; i < g.NX; ++i) {
            code[(size_t)j * g.P + i] = m->mesh.code[(size_t)j * g.NX + i];
            gm[(size_t)j * g.P + i] = m->mesh.gv[(size_t)j * g.NX + i] >= 0;
        }
    CK(cudaMemcpy(m->d_code, code.data(), code.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->d_gmask, gm.data(), gm.size(), cudaMemcpyHostToDevice));
    for (int w = 0; w < 2; ++w) {
        bs_free(m->bs[w]);
        m->bs_ready[w] = false;
    }
    ns_free(m->ns);
    m->ns_ready = false;
    drop_graphs(m);
    return 0;
}

// ---------------------------------------------------------------------------
extern "C" {

int f2d_abi_version(void) { return F2D_ABI_VERSION; }
const char* f2d_last_error(void) { return g_err.c_str(); }

int f2d_params_default(f2d_params* p)
{
    if (!p) return fail(1, "null params");
    memset(p, 0, sizeof(*p));
    p->model = F2D_MODEL_EULERPSI;
    p->nx = 40;
    p->ny = 40;
    p->halowidth = 3;
    p->Lx = 1.0;
    p->Ly = 1.0;
    p->f0 = 10.0;
    p->beta = 0.0;
    p->g = 1.0;
    p->H = 1.0;
    p->cfl = 0.9;
    p->dtmax = 9e99;
    p->dt = 0.0;
    p->compflux = p->vortexforce = p->innerproduct = F2D_METHOD_WENO;
    p->maxorder = 6;
    p->noslip = F2D_SLIP_FREE;
    p->precision = F2D_PREC_FP64;
    p->poisson_tol = 1e-12;
    p->poisson_maxit = 200;
    p->integrator = F2D_INTEG_RK3;
    p->ragamma = 0.1;
    return 0;
}

int f2d_set_order(const int8_t* msk, int64_t n, int64_t shift, int maxorder, int8_t* order)
{
    if (!msk || !order || n < 0) return fail(1, "bad arguments");
    set_order_host(msk, n, shift, maxorder, order);
    return 0;
}

int f2d_mesh_build(const f2d_params* p, const int8_t* msk, int8_t* mskx, int8_t* msky,
                   int8_t* mskv, double* slipcoef, int8_t* orders, int32_t* gv)
{
    if (!p) return fail(1, "null params");
    MeshHost M;
    std::string err;
    if (mesh_build_host(*p, msk, M, err)) return fail(7, err);
    const size_t N = (size_t)M.NY * M.NX;
    if (mskx) memcpy(mskx, M.mskx.data(), N);
    if (msky) memcpy(msky, M.msky.data(), N);
    if (mskv) memcpy(mskv, M.mskv.data(), N);
    if (slipcoef) memcpy(slipcoef, M.slip.data(), N * 8);
    if (orders)
        for (int k = 0; k < 6; ++k) memcpy(orders + k * N, M.ord[k].data(), N);
    if (gv) memcpy(gv, M.gv.data(), N * 4);
    return 0;
}

int f2d_compflux(int method, double* flx, const double* U, const double* q, const int8_t* o,
                 int64_t s, int64_t i0, int64_t i1, void* stream)
{
    CKI(launch_compflux(method, flx, U, q, o, s, i0, i1, (cudaStream_t)stream));
    return 0;
}

int f2d_vortexforce(int method, double* du, const double* V, const double* q,
                    const int8_t* o, int64_t s, int64_t s2, int sign, int64_t i0, int64_t i1,
                    void* stream)
{
    CKI(launch_vortexforce(method, du, V, q, o, s, s2, sign, i0, i1, (cudaStream_t)stream));
    return 0;
}

int f2d_innerproduct(int method, double* ke, const double* U, const double* q,
                     const int8_t* o, int64_t s, int64_t i0, int64_t i1, void* stream)
{
    CKI(launch_innerproduct(method, ke, U, q, o, s, i0, i1, (cudaStream_t)stream));
    return 0;
}

int f2d_model_create(const f2d_params* p, const int8_t* msk, f2d_model* out)
{
    if (!p || !out) return fail(1, "null argument");
    if (p->precision != F2D_PREC_FP64 && p->precision != F2D_PREC_FP32)
        return fail(1, "unknown precision");
    if (p->model < 0 || p->model > 5) return fail(1, "unknown model");

    if (p->integrator < F2D_INTEG_RK3 || p->integrator > F2D_INTEG_LFRA)
        return fail(1, "unknown integrator (rk3, ef, enrk3, LFRA)");
    if (p->xperiodic && p->nx < 6) return fail(1, "x-periodic needs nx >= 6");
    if (p->compflux < F2D_METHOD_WENO || p->compflux > F2D_METHOD_CWENO ||
        p->vortexforce < F2D_METHOD_WENO || p->vortexforce > F2D_METHOD_CWENO)
        return fail(1, "unknown flux method (weno, upwind, centered, cweno)");
    if (p->innerproduct < F2D_METHOD_WENO || p->innerproduct > F2D_METHOD_CLASSIC)
        return fail(1, "unknown innerproduct method (weno, upwind, centered, cweno, "
                       "classic)");
    if ((p->model == F2D_MODEL_RSW || p->model == F2D_MODEL_BOUSSINESQ ||
         p->model == F2D_MODEL_QGRSW) &&
        p->vortexforce != p->compflux)
        return fail(1, "the fused rsw/boussinesq stage uses one flux method for "
                       "vortexforce and compflux; they must be equal");
    auto* m = new f2d_model_s();
    m->p = *p;
    m->prec = p->precision == F2D_PREC_FP64 ? 0 : 1;
    m->es = m->prec == 0 ? 8 : 4;
    Geom& g = m->g;
    g.ny = p->ny;
    g.nx = p->nx;
    g.NY = p->ny + 6;
    g.NX = p->nx + 6;
    g.P = (g.NX + 15) / 16 * 16;
    g.xper = p->xperiodic ? 1 : 0;
    // mesh constants, evaluated like the reference's Python expressions
    m->dx = p->Lx / p->nx;
    m->dy = p->Ly / p->ny;
    m->area = m->dx * m->dy;
    m->rdx2 = 1 / pow(m->dx, 2.0);
    m->rdy2 = 1 / pow(m->dy, 2.0);
    m->goa = p->g / m->area;
    m->fc = p->f0 * m->area * 0.25;
    m->maindiag = m->area * pow(p->f0, 2.0) / (p->g * p->H);
    m->cx = m->dy / m->dx;  // dx2 of get_Laplacian_sparse (E-W)
    m->cy = m->dx / m->dy;  // dy2 (N-S)
    int e = 0;
    auto bail = [&](int code) {
        f2d_model_destroy(m);
        return code;
    };
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&m->s2, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(2, "stream creation failed"));
    m->own_stream = true;
    m->d_code = (uint32_t*)dalloc(m, (size_t)g.P * g.NY * 4);
    m->d_gmask = (uint8_t*)dalloc(m, (size_t)g.P * g.NY);
    m->sc = (DevScalars*)dalloc(m, sizeof(DevScalars));
    const size_t nb = pt_grid_blocks(g) + 64;
    m->partials = (double*)dalloc(m, nb * 4 * sizeof(double));
    if (!m->d_code || !m->d_gmask || !m->sc || !m->partials)
        return bail(fail(2, "out of device memory"));
    // fields of the state (states.py:7-17) and of the RK3 scratch
    std::vector<std::pair<const char*, bool>> fl;
    std::vector<const char*> prog;
    if (p->model == F2D_MODEL_EULERPSI) {
        fl = {{"omega", true}, {"U.x", false}, {"U.y", false}, {"psi", false},
              {"vomega", false}, {"flx.x", false}, {"flx.y", false}};
        prog = {"omega"};
    } else if (p->model == F2D_MODEL_EULER) {
        fl = {{"u.x", true}, {"u.y", true}, {"U.x", false}, {"U.y", false},
              {"omega", false}, {"ke", false}, {"p", false}, {"div", false},
              {"flx.x", false}, {"flx.y", false}};
        prog = {"u.x", "u.y"};
    } else if (p->model == F2D_MODEL_BOUSSINESQ) {
        fl = {{"b", true}, {"u.x", true}, {"u.y", true}, {"U.x", false}, {"U.y", false},
              {"omega", false}, {"ke", false}, {"p", false}, {"div", false},
              {"flx.x", false}, {"flx.y", false}};
        prog = {"b", "u.x", "u.y"};
    } else if (p->model == F2D_MODEL_QGRSW) {
        fl = {{"u.x", true}, {"u.y", true}, {"h", true}, {"U.x", false}, {"U.y", false},
              {"omega", false}, {"ke", false}, {"p", false}, {"flx.x", false},
              {"flx.y", false}, {"pv", false}, {"psi", false}};
        prog = {"u.x", "u.y", "h"};
    } else if (p->model == F2D_MODEL_RSW) {
        fl = {{"u.x", true}, {"u.y", true}, {"h", true}, {"U.x", false}, {"U.y", false},
              {"omega", false}, {"ke", false}, {"p", false}, {"flx.x", false},
              {"flx.y", false}, {"pv", false}};
        prog = {"u.x", "u.y", "h"};
    } else {
        fl = {{"pv", true}, {"U.x", false}, {"U.y", false}, {"h", false}, {"flx.x", false},
              {"flx.y", false}, {"work", false}, {"psi", false}};
        prog = {"pv"};
    }
    if (p->tracer) {
        // states.py:31-34: the tracer is the last prognostic variable
        fl.push_back({"tracer", true});
        prog.push_back("tracer");
    }
    // the Poisson solution and right-hand side are FP64 in both forms; the
    // stencil state has the model's precision
    auto is64 = [&](const char* n) {
        // the pressure of the Neumann projection is the FP64 solve's unknown
        return !strcmp(n, "psi") || !strcmp(n, "vomega") || !strcmp(n, "work") ||
               (p->model == F2D_MODEL_QGRSW && !strcmp(n, "pv")) ||
               (projected(p->model) && !strcmp(n, "p"));
    };
    for (auto& f : fl)
        if ((e = add_field(m, f.first, f.second, is64(f.first) ? 8 : (int)m->es)))
            return bail(e);
    // the streamfunctions of this step's start and first stage and the
    // previous step's stage increments (the warm start of the stage solves,
    // rec_warm)
    if (p->model == F2D_MODEL_EULERPSI || p->model == F2D_MODEL_QG)
        for (const char* f : {"psi.s0", "psi.p1", "psi.d1", "psi.d2"})
            if ((e = add_field(m, f, false, 8))) return bail(e);
    // qgrsw keeps the third stage's (or LFRA's) tendency too: it is
    // projected between the tendency kernel and the update
    for (const char* f : prog) m->prog.push_back(f);
    const int nds = p->model == F2D_MODEL_QGRSW ? 3 : 2;
    for (int k = 1; k <= nds; ++k)
        for (const char* f : prog)
            if ((e = add_field(m, (std::string("ds") + std::to_string(k) + "." + f).c_str(),
                               false, (int)m->es)))
                return bail(e);
    if (projected(p->model)) {
        m->nrhs = (double*)dalloc(m, field_bytes(m, 8));
        if (!m->nrhs) return bail(fail(2, "out of device memory"));
    } else if (p->model != F2D_MODEL_RSW) {
        m->pr = dalloc(m, field_bytes(m, 8));
        m->pp = dalloc(m, field_bytes(m, 8));
        m->pq = dalloc(m, field_bytes(m, 8));
        m->pz = dalloc(m, field_bytes(m, m->es));
        m->pp2 = dalloc(m, field_bytes(m, 8));
        m->pza = dalloc(m, field_bytes(m, m->es));
        m->prmg = m->prec == 0 ? m->pr : dalloc(m, field_bytes(m, 4));
        m->d_fv = dalloc(m, field_bytes(m, 8));
        if (!m->pr || !m->pz || !m->pp || !m->pq || !m->d_fv || !m->prmg ||
            !m->pp2 || !m->pza)
            return bail(fail(2, "out of device memory"));
    }
    if (m->prec != 0) {
        m->stage64 = dalloc(m, field_bytes(m, 8));
        if (!m->stage64) return bail(fail(2, "out of device memory"));
    }
    if ((e = setup_mesh(m, msk))) return bail(e);
    // time line (timeline.py:4-12) and set_dt constants (model.py:71-87)
    DevScalars h;
    memset(&h, 0, sizeof(h));
    h.dt = p->dt > 0 ? p->dt : 0.01;
    h.cfl = p->cfl;
    h.dtmax = p->dtmax;
    h.ragamma = p->ragamma;
    m->cfl_dt = !(p->dt > 0) && p->model != F2D_MODEL_RSW;
    if (p->dt > 0) m->dt_const = p->dt;
    else if (p->model == F2D_MODEL_RSW) {
        const double c = pow(p->g * p->H, 0.5);
        const double maxU = c / m->dx + c / m->dy;
        m->dt_const = fmin(p->cfl / maxU, p->dtmax);
    }
    if (cudaMemcpy(m->sc, &h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(2, "scalar upload failed"));
    *out = m;
    return 0;
}

int f2d_model_destroy(f2d_model m)
{
    if (!m) return 0;
    if (m->stream) cudaStreamSynchronize(m->stream);
    drop_graphs(m);
    for (int w = 0; w < 2; ++w) bs_free(m->bs[w]);
    ns_free(m->ns);
    if (m->adj.psic) cudaFree(m->adj.psic);
    for (void* p : m->allocs) cudaFree(p);
    if (m->own_stream && m->stream) cudaStreamDestroy(m->stream);
    if (m->s2) cudaStreamDestroy(m->s2);
    delete m;
    return 0;
}

int f2d_model_set_mask(f2d_model m, const int8_t* msk)
{
    if (!m || !msk) return fail(1, "null argument");
    CK(cudaStreamSynchronize(m->stream));
    return setup_mesh(m, msk);
}

int f2d_model_set_stream(f2d_model m, void* stream)
{
    if (!m) return fail(1, "null model");
    CK(cudaStreamSynchronize(m->stream));
    if (m->own_stream) cudaStreamDestroy(m->stream);
    if (stream) {
        m->stream = (cudaStream_t)stream;
        m->own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
        m->own_stream = true;
    }
    return 0;
}

static int field_io(f2d_model m, const char* name, double* host, bool set, bool async)
{
    if (!m || !name || !host) return fail(1, "null argument");
    void* d = fb(m, name);
    if (!d) return fail(8, std::string("no field named ") + name);
    const Geom& g = m->g;
    const int es = field_es(m, name);
    // FP32 fields go through the FP64 staging array and a conversion kernel
    void* d64 = es == 8 ? d : m->stage64;
    if (set) {
        CK(cudaMemcpy2DAsync(d64, g.P * 8, host, g.NX * 8, g.NX * 8, g.NY,
                             cudaMemcpyHostToDevice, m->stream));
        if (es == 4) CKI(launch_convert(0, 1, d64, d, g, m->stream));
    } else {
        if (es == 4) CKI(launch_convert(1, 0, d, d64, g, m->stream));
        CK(cudaMemcpy2DAsync(host, g.NX * 8, d64, g.P * 8, g.NX * 8, g.NY,
                             cudaMemcpyDeviceToHost, m->stream));
    }
    if (set && (!strcmp(name, "U.x") || !strcmp(name, "U.y")))
        CKI(launch_maxabs2(m->prec, fb(m, "U.x"), fb(m, "U.y"), g, m->sc, m->partials,
                           m->stream));
    if (!async) CK(cudaStreamSynchronize(m->stream));
    return 0;
}

int f2d_field_set(f2d_model m, const char* name, const double* host)
{
    return field_io(m, name, (double*)host, true, false);
}
static const int BULK_CAP = 1000;  // Bulk.ndiags (diagnostics.py:21)

int f2d_bulk_record(f2d_model m)
{
    if (!m) return fail(1, "null model");
    if (!fb(m, "ke") || !fb(m, "omega"))
        return fail(1, "Bulk needs the ke and omega fields (rsw, euler, boussinesq, qgrsw)");
    if (!m->bulk_ring) {
        m->bulk_ring = (double*)dalloc(m, sizeof(double) * 5 * BULK_CAP);
        m->bulk_count = (int*)dalloc(m, sizeof(int));
        if (!m->bulk_ring || !m->bulk_count) return fail(2, "out of device memory");
    }
    // domsum(msk) over the whole array (diagnostics.py:15), once per mask
    if (m->bulk_summsk < 0) {
        double sm = 0.0;
        for (int8_t v : m->mesh.msk) sm += v;
        m->bulk_summsk = sm;
    }
    const double summsk = m->bulk_summsk;
    if (summsk <= 0) return fail(1, "the mask has no wet cell");
    BulkArgs a;
    a.ke = fb(m, "ke");
    a.omega = fb(m, "omega");
    a.Ux = fb(m, "U.x");
    a.Uy = fb(m, "U.y");
    a.ring = m->bulk_ring;
    a.count = m->bulk_count;
    a.cap = BULK_CAP;
    a.summsk = summsk;
    a.area = m->area;
    a.dx = m->dx;
    a.dy = m->dy;
    CKI(launch_bulk(m->prec, a, m->g, m->sc, m->partials, m->stream));
    return 0;
}

int f2d_bulk_read(f2d_model m, double* host, int capacity, int* nrec)
{
    if (!m || !nrec) return fail(1, "null argument");
    *nrec = 0;
    if (!m->bulk_ring) return 0;
    int n = 0;
    CK(cudaMemcpyAsync(&n, m->bulk_count, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (n > capacity) return fail(1, "host buffer too small for the Bulk records");
    if (n > 0) {
        CK(cudaMemcpyAsync(host, m->bulk_ring, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost,
                           m->stream));
        CK(cudaMemsetAsync(m->bulk_count, 0, sizeof(int), m->stream));
        CK(cudaStreamSynchronize(m->stream));
    }
    *nrec = n;
    return 0;
}

int f2d_field_get_f32(f2d_model m, const char* name, float* host)
{
    if (!m || !name || !host) return fail(1, "null argument");
    void* d = fb(m, name);
    if (!d) return fail(8, std::string("no field named ") + name);
    if (!m->f32_stage) {
        m->f32_stage = (float*)dalloc(m, sizeof(float) * (size_t)m->g.NY * m->g.NX);
        if (!m->f32_stage) return fail(2, "out of device memory");
    }
    CKI(launch_to_f32(field_es(m, name) == 8 ? 0 : 1, d, m->f32_stage, m->g, m->stream));
    CK(cudaMemcpyAsync(host, m->f32_stage, sizeof(float) * (size_t)m->g.NY * m->g.NX,
                       cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return 0;
}

int f2d_field_get(f2d_model m, const char* name, double* host)
{
    return field_io(m, name, host, false, false);
}
int f2d_field_set_async(f2d_model m, const char* name, const double* host)
{
    return field_io(m, name, (double*)host, true, true);
}
int f2d_field_get_async(f2d_model m, const char* name, double* host)
{
    return field_io(m, name, host, false, true);
}

int f2d_field_device(f2d_model m, const char* name, void** ptr, int64_t* pitch, int* es)
{
    if (!m || !name) return fail(1, "null argument");
    void* d = fb(m, name);
    if (!d) return fail(8, std::string("no field named ") + name);
    if (ptr) *ptr = d;
    if (pitch) *pitch = m->g.P;
    if (es) *es = field_es(m, name);
    return 0;
}

int f2d_field_names(f2d_model m, char* buf, size_t len)
{
    if (!m || !buf || !len) return fail(1, "null argument");
    std::string s;
    for (auto& kv : m->fields) {
        // the state's fields (not the integrator's scratch, the warm-start
        // history, the rhs and forcing fields)
        const std::string& n = kv.first;
        if (n.rfind("ds", 0) == 0 || n.rfind("psi.", 0) == 0 || n.rfind("rhs.", 0) == 0 ||
            n.rfind("frc.", 0) == 0)
            continue;
        if (!s.empty()) s += ",";
        s += kv.first;
    }
    if (s.size() + 1 > len) return fail(1, "buffer too small");
    memcpy(buf, s.c_str(), s.size() + 1);
    return 0;
}

int f2d_set_coriolis(f2d_model m, const double* f)
{
    if (!m || !f) return fail(1, "null argument");
    if (!m->d_fv) return fail(8, "model has no vertex Coriolis field");
    const Geom& g = m->g;
    CK(cudaMemcpy2DAsync(m->d_fv, g.P * 8, f, g.NX * 8, g.NX * 8, g.NY,
                         cudaMemcpyHostToDevice, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return 0;
}

int f2d_diag(f2d_model m)
{
    if (!m) return fail(1, "null model");
    return run_graph(m, 0);
}

int f2d_qg_projection(f2d_model m)
{
    if (!m) return fail(1, "null model");
    if (m->p.model != F2D_MODEL_QGRSW) return fail(1, "qg_projection acts on a qgrsw model");
    return run_graph(m, 3);
}

int f2d_step(f2d_model m, int n)
{
    if (!m) return fail(1, "null model");
    for (int k = 0; k < n; ++k) {
        int e = run_graph(m, 1);
        if (e) return e;
    }
    return 0;
}

int f2d_rhs(f2d_model m)
{
    if (!m) return fail(1, "null model");
    // the tendency fields exist before any capture (allocation)
    for (const auto& f : m->prog) {
        const std::string n = "rhs." + f;
        if (!fb(m, n.c_str())) {
            int e = add_field(m, n.c_str(), false, (int)m->es);
            if (e) return e;
        }
    }
    return run_graph(m, 7);
}

int f2d_stage(f2d_model m, int k)
{
    if (!m) return fail(1, "null model");
    if (k < 1 || k > nstages(m))
        return fail(1, "stage " + std::to_string(k) + " out of range: the integrator has " +
                           std::to_string(nstages(m)) + " stage(s)");
    return run_graph(m, 7 + k);
}

int f2d_forcing_set(f2d_model m, const char* name, const double* host)
{
    if (!m || !name || !host) return fail(1, "null argument");
    bool known = false;
    for (const auto& f : m->prog) known = known || f == name;
    if (!known)
        return fail(8, std::string("no prognostic variable named ") + name +
                           " for a forcing term");
    if (!m->has_frc) {
        // all forcing fields at once (zero), then every recorded graph is
        // dropped: the stage kernels are recorded with the forcing pointers
        for (const auto& f : m->prog) {
            int e = add_field(m, ("frc." + f).c_str(), false, (int)m->es);
            if (e) return e;
        }
        m->has_frc = true;
        drop_graphs(m);
    }
    return field_io(m, ("frc." + std::string(name)).c_str(), (double*)host, true, false);
}

int f2d_forcing_clear(f2d_model m)
{
    if (!m) return fail(1, "null model");
    if (!m->has_frc) return 0;
    for (const auto& f : m->prog)
        CK(cudaMemsetAsync(fb(m, ("frc." + f).c_str()), 0, field_bytes(m, m->es), m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return 0;
}

int f2d_set_dt(f2d_model m)
{
    if (!m) return fail(1, "null model");
    if (m->cfl_dt) {
        CKI(launch_set_dt(m->sc, m->stream));
    } else {
        CK(cudaMemcpyAsync(&m->sc->dt, &m->dt_const, 8, cudaMemcpyHostToDevice, m->stream));
        CK(cudaStreamSynchronize(m->stream));
        m->dt_applied = true;
    }
    return 0;
}

int f2d_run(f2d_model m, int n)
{
    if (!m) return fail(1, "null model");
    if (!m->cfl_dt && !m->dt_applied) {
        int e = f2d_set_dt(m);
        if (e) return e;
    }
    for (int k = 0; k < n; ++k) {
        int e = run_graph(m, 2);
        if (e) return e;
    }
    return 0;
}

int f2d_time_get(f2d_model m, double* t, double* dt, int64_t* ite)
{
    if (!m) return fail(1, "null model");
    DevScalars h;
    CK(cudaMemcpyAsync(&h, m->sc, sizeof(h), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (t) *t = h.t;
    if (dt) *dt = h.dt;
    if (ite) *ite = h.ite;
    return 0;
}

int f2d_time_set(f2d_model m, double t, double dt, int64_t ite)
{
    if (!m) return fail(1, "null model");
    DevScalars h;
    CK(cudaMemcpyAsync(&h, m->sc, sizeof(h), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    h.t = t;
    h.dt = dt;
    h.ite = ite;
    h.c = 0.0;
    m->dt_applied = false;
    CK(cudaMemcpyAsync(m->sc, &h, sizeof(h), cudaMemcpyHostToDevice, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    return 0;
}

int f2d_poisson_solve(f2d_model m, int which, const double* b, double* x, int* iters,
                      double* relres)
{
    if (!m || !b || !x) return fail(1, "null argument");
    if (which != 0 && which != 1) return fail(1, "which must be 0 or 1");
    if (!m->pr) return fail(8, "this model has no Poisson workspace");
    if (which == 1 && m->p.model == F2D_MODEL_EULERPSI)
        return fail(8, "the Helmholtz operator exists for qg/rsw models only");
    const Geom& g = m->g;
    if (!m->sb) {
        m->sb = dalloc(m, field_bytes(m, 8));
        m->sx = dalloc(m, field_bytes(m, 8));
        if (!m->sb || !m->sx) return fail(2, "out of device memory");
    }
    CK(cudaMemcpy2DAsync(m->sb, g.P * 8, b, g.NX * 8, g.NX * 8, g.NY, cudaMemcpyHostToDevice,
                         m->stream));
    CK(cudaMemcpy2DAsync(m->sx, g.P * 8, x, g.NX * 8, g.NX * 8, g.NY, cudaMemcpyHostToDevice,
                         m->stream));
    const int kind = 3 + which;
    DevScalars h0;
    CK(cudaMemcpyAsync(&h0, m->sc, sizeof(h0), cudaMemcpyDeviceToHost, m->stream));
    if (eager_mode()) {
        // the profiling mode: the solve's loops driven from the host
        int e0 = ensure_mg(m, which);
        if (e0) return e0;
        int e = rec_solve(m, which, m->sb, m->sx, m->stream);
        if (e) return e;
    } else if (!m->gx[kind][0]) {
        int e0 = ensure_mg(m, which);
        if (e0) return e0;
        m->rec_launches = 0;
        CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeRelaxed));
        int e = rec_solve(m, which, m->sb, m->sx, m->stream);
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(m->stream, &graph);
        if (e) {
            if (graph) cudaGraphDestroy(graph);
            return e;
        }
        if (ce != cudaSuccess) return fail((int)ce, cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&m->gx[kind][0], graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail((int)ce, cudaGetErrorString(ce));
    }
    if (!eager_mode()) CK(cudaGraphLaunch(m->gx[kind][0], m->stream));
    CK(cudaMemcpy2DAsync(x, g.NX * 8, m->sx, g.P * 8, g.NX * 8, g.NY, cudaMemcpyDeviceToHost,
                         m->stream));
    DevScalars h;
    CK(cudaMemcpyAsync(&h, m->sc, sizeof(h), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    // CG iterations of this solve (the FP32 form: inner iterations summed
    // over its refinement rounds)
    if (iters) *iters = (int)(h.total_iters - h0.total_iters);
    if (relres) *relres = h.bb > 0 ? sqrt(h.rr / h.bb) : 0.0;
    return 0;
}

int f2d_sync(f2d_model m)
{
    if (!m) return fail(1, "null model");
    CK(cudaStreamSynchronize(m->stream));
    int st = 0;
    CK(cudaMemcpy(&st, &m->sc->status, sizeof(int), cudaMemcpyDeviceToHost));
    for (int w = 0; w < 2; ++w)
        if (m->bs_ready[w]) {
            BSGlobals bg;
            CK(cudaMemcpy(&bg, m->bs[w].eg, sizeof(bg), cudaMemcpyDeviceToHost));
            if (bg.status) {
                st |= bg.status;
                int zero = 0;
                CK(cudaMemcpy(&m->bs[w].eg->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
            }
        }
    if (m->ns_ready) {
        NGlobals ng;
        CK(cudaMemcpy(&ng, m->ns.eg, sizeof(ng), cudaMemcpyDeviceToHost));
        if (ng.status) {
            st |= ng.status;
            int zero = 0;
            CK(cudaMemcpy(&m->ns.eg->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
        }
    }
    if (st) {
        int zero = 0;
        CK(cudaMemcpy(&m->sc->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
        std::string msg = "device status:";
        if (st & ST_TMA_TIMEOUT) msg += " TMA tile load timed out;";
        if (st & ST_STAGE_ALIGN) msg += " TMA staging buffer misaligned;";
        if (st & ST_PCG_MAXIT) msg += " Poisson solve reached max iterations;";
        if (st & ST_NONFINITE) msg += " non-finite value (residual or time step);";
        return fail(100 + st, msg);
    }
    return 0;
}

// test hook: the integer-pipe conversions against the hardware ones
__global__ void k_test_conv(const double* __restrict__ x64, long long n64,
                            float* __restrict__ sw32, float* __restrict__ hw32,
                            const float* __restrict__ x32, long long n32,
                            double* __restrict__ sw64, double* __restrict__ hw64)
{
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < n64) {
        sw32[k] = f64_to_f32_rn(x64[k]);
        hw32[k] = __double2float_rn(x64[k]);
    }
    if (k < n32) {
        sw64[k] = f32_to_f64(x32[k]);
        hw64[k] = (double)x32[k];
    }
}

int f2d_test_conversions(const double* x64, int64_t n64, float* sw32, float* hw32,
                         const float* x32, int64_t n32, double* sw64, double* hw64)
{
    if (n64 < 0 || n32 < 0 || (n64 && (!x64 || !sw32 || !hw32)) ||
        (n32 && (!x32 || !sw64 || !hw64)))
        return fail(1, "bad arguments");
    const long long n = std::max<long long>(std::max<long long>(n64, n32), 1);
    void *d64 = nullptr, *d32 = nullptr, *o32 = nullptr, *o64 = nullptr;
    const size_t b64 = sizeof(double) * std::max<long long>(n64, 1);
    const size_t b32 = sizeof(float) * std::max<long long>(n32, 1);
    int err = 0;
    if (cudaMalloc(&d64, b64) != cudaSuccess || cudaMalloc(&d32, b32) != cudaSuccess ||
        cudaMalloc(&o32, 2 * sizeof(float) * std::max<long long>(n64, 1)) != cudaSuccess ||
        cudaMalloc(&o64, 2 * sizeof(double) * std::max<long long>(n32, 1)) != cudaSuccess)
        err = fail(2, "out of device memory");
    if (!err) {
        if (n64) cudaMemcpy(d64, x64, sizeof(double) * n64, cudaMemcpyHostToDevice);
        if (n32) cudaMemcpy(d32, x32, sizeof(float) * n32, cudaMemcpyHostToDevice);
        float* s32 = (float*)o32;
        double* s64 = (double*)o64;
        k_test_conv<<<(unsigned)((n + 255) / 256), 256>>>(
            (const double*)d64, n64, s32, s32 + std::max<long long>(n64, 1), (const float*)d32,
            n32, s64, s64 + std::max<long long>(n32, 1));
        if (cudaDeviceSynchronize() != cudaSuccess) err = fail(3, "conversion test kernel failed");
        if (!err && n64) {
            cudaMemcpy(sw32, s32, sizeof(float) * n64, cudaMemcpyDeviceToHost);
            cudaMemcpy(hw32, s32 + n64, sizeof(float) * n64, cudaMemcpyDeviceToHost);
        }
        if (!err && n32) {
            cudaMemcpy(sw64, s64, sizeof(double) * n32, cudaMemcpyDeviceToHost);
            cudaMemcpy(hw64, s64 + n32, sizeof(double) * n32, cudaMemcpyDeviceToHost);
        }
    }
    for (void* p : {d64, d32, o32, o64})
        if (p) cudaFree(p);
    return err;
}

int f2d_test_tma_wait(int enabled, double limit_ms)
{
    if (enabled && !(limit_ms > 0 && limit_ms <= 1000))
        return fail(1, "f2d_test_tma_wait: limit_ms must be in (0, 1000]");
    const unsigned long long ns =
        enabled ? (unsigned long long)(limit_ms * 1e6) : 0ull;
    CK(cudaDeviceSynchronize());
    int e = tma_wait_test_set_stage(enabled, ns);
    if (!e) e = tma_wait_test_set_ensemble(enabled, ns);
    if (e) return fail(e, std::string("f2d_test_tma_wait: ") +
                              cudaGetErrorString((cudaError_t)e));
    return 0;
}

int f2d_refine_rounds(f2d_model m, int64_t* rounds)
{
    if (!m || !rounds) return fail(1, "null argument");
    DevScalars h;
    CK(cudaMemcpyAsync(&h, m->sc, sizeof(h), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    *rounds = h.total_outer;
    return 0;
}

int f2d_stats(f2d_model m, int64_t* poisson_iters, int64_t* launches_per_step,
              int64_t* launches_per_iter)
{
    if (!m) return fail(1, "null model");
    DevScalars h;
    CK(cudaMemcpyAsync(&h, m->sc, sizeof(h), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    if (poisson_iters) *poisson_iters = h.total_iters;
    if (poisson_iters && m->ns_ready) {
        DevScalars hn;
        CK(cudaMemcpy(&hn, m->ns.sc, sizeof(hn), cudaMemcpyDeviceToHost));
        *poisson_iters = hn.total_iters;
    }
    if (launches_per_step) {
        // kernels outside the Poisson loop bodies of one step; each Poisson
        // iteration adds body_launches more
        int n = m->launches[2][0] ? m->launches[2][0] : m->launches[1][0];
        *launches_per_step = n;
    }
    if (launches_per_iter) *launches_per_iter = m->p.model == F2D_MODEL_RSW ? 0 : m->body_launches;
    return 0;
}

int f2d_time_stage(f2d_model m, int stage, int reps, int flush_l2, double* avg_ms)
{
    if (!m || !avg_ms || reps < 1 || stage < 1 || stage > 3) return fail(1, "bad arguments");
    // the stage kernel reads parity cur and writes the other buffer; repeated
    // launches recompute the same values, so the model state is unchanged
    const size_t flush_bytes = 256ull << 20;  // twice the 126 MB L2
    void* fl = nullptr;
    if (flush_l2) CK(cudaMalloc(&fl, flush_bytes));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    double total = 0.0;
    int e = 0;
    for (int r = 0; r < reps && !e; ++r) {
        if (fl) cudaMemsetAsync(fl, r & 0xff, flush_bytes, m->stream);
        cudaEventRecord(a, m->stream);
        // qgrsw: the tendency kernel (its solve is timed by f2d_time_solver)
        e = m->p.model == F2D_MODEL_QGRSW ? launch_qgrsw_tendency(m, stage, m->cur, m->stream)
                                          : launch_stage_kernel(m, stage, m->cur, m->stream);
        cudaEventRecord(b, m->stream);
        if (cudaEventSynchronize(b) != cudaSuccess) e = fail(2, "event sync failed");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        total += ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (fl) cudaFree(fl);
    if (e) return e;
    *avg_ms = total / reps;
    return 0;
}

int f2d_autotune(f2d_model m, int reps, int* th, int* nu, double* tol_in, double* ms)
{
    if (!m || reps < 1) return fail(1, "bad autotune arguments");
    if (m->p.model == F2D_MODEL_RSW || projected(m->p.model))
        return fail(1, "the autotuner tunes the multigrid of eulerpsi, qg and qgrsw");
    const int which = m->p.model == F2D_MODEL_EULERPSI ? 0 : 1;
    // the right-hand side and solution of the current state's diagnostics
    int e = run_graph(m, 0);
    if (e) return e;
    const void* b = fb(m, which == 0 ? "vomega" : "work");
    if (m->p.model == F2D_MODEL_QGRSW) {
        // the right-hand side of the first stage's projection
        int e0 = ensure_mg(m, 1);
        if (e0) return e0;
        e0 = launch_qgrsw_tendency(m, 1, m->cur, m->stream);
        if (e0) return e0;
        CKI(launch_qgrsw_pv(m->prec, fb(m, "ds3.u.x"), fb(m, "ds3.u.y"), fb(m, "ds3.h"),
                            (double*)fb(m, "pv"), m->d_code, -m->p.f0 / m->p.H, 0.0, m->g,
                            m->stream));
        b = fb(m, "pv");
    }
    CK(cudaStreamSynchronize(m->stream));
    BSTune t;
    memset(&t, 0, sizeof(t));
    const int err = bs_autotune(m->bs[which], m->stream, m->s2, fb(m, "psi"), b,
                                field_bytes(m, 8), reps, &t);
    drop_graphs(m);
    if (err) return fail(err, "multigrid autotune failed");
    m->body_launches = 0;
    if (th) *th = t.th;
    if (nu) *nu = t.nu;
    if (tol_in) *tol_in = t.tol_in;
    if (ms) *ms = t.ms;
    return 0;
}

int f2d_set_schedule(f2d_model m, int tile_rows, int sweeps, double tol_in)
{
    if (!m) return fail(1, "null model");
    if (m->p.model == F2D_MODEL_RSW || projected(m->p.model))
        return fail(1, "the schedule is that of the multigrid of eulerpsi, qg and qgrsw");
    const int which = m->p.model == F2D_MODEL_EULERPSI ? 0 : 1;
    int e = ensure_mg(m, which);
    if (e) return e;
    CK(cudaStreamSynchronize(m->stream));
    e = bs_set_schedule(m->bs[which], tile_rows, sweeps, tol_in);
    drop_graphs(m);
    if (e == 1) return fail(1, "schedule: tile_rows 32 or 64, sweeps 1 or 2, 0 < tol_in < 1");
    if (e) return fail(e, "multigrid rebuild failed");
    m->body_launches = 0;
    return 0;
}

int f2d_time_solver(f2d_model m, int reps, int flush_l2, double* avg_ms, int64_t* nodes,
                    int* elem_bytes)
{
    if (!m || !avg_ms) return fail(1, "null argument");
    if (m->p.model == F2D_MODEL_RSW) return fail(1, "rsw has no Poisson solve");
    if (projected(m->p.model))
        return fail(1, "the Neumann solve of the euler and boussinesq models has no "
                       "timing hook");
    const int which = m->p.model == F2D_MODEL_EULERPSI ? 0 : 1;
    if (!m->bs_ready[which]) return fail(9, "the solver has not run yet");
    CK(cudaStreamSynchronize(m->stream));
    long long n = 0;
    int es = 0;
    int e = bs_time_down(m->bs[which], m->stream, reps, flush_l2, avg_ms, &n, &es);
    if (e) return fail(e, "solver kernel timing failed (no grid level?)");
    if (nodes) *nodes = n;
    if (elem_bytes) *elem_bytes = es;
    return 0;
}

int f2d_solver_pipelined(f2d_model m, int* pipelined)
{
    if (!m || !pipelined) return fail(1, "null argument");
    if (m->p.model == F2D_MODEL_RSW || projected(m->p.model))
        return fail(1, "the model has no vertex Poisson solve");
    const int which = m->p.model == F2D_MODEL_EULERPSI ? 0 : 1;
    if (!m->bs_ready[which]) return fail(9, "the solver has not run yet");
    *pipelined = m->bs[which].pipe ? 1 : 0;
    return 0;
}

// ---- discrete adjoint of the eulerpsi step ------------------------------------
static int adj_check(f2d_model m)
{
    if (!m) return fail(1, "null model");
    if (m->p.model != F2D_MODEL_EULERPSI) return fail(1, "the adjoint covers the eulerpsi model");
    if (m->g.xper) return fail(1, "the adjoint covers closed (non-periodic) domains");
    if (m->p.compflux != F2D_METHOD_WENO && m->p.compflux != F2D_METHOD_UPWIND)
        return fail(1, "the adjoint covers the weno and upwind flux methods");
    if (m->p.integrator != F2D_INTEG_RK3) return fail(1, "the adjoint covers SSP-RK3");
    if (m->p.tracer) return fail(1, "the adjoint covers the eulerpsi model without a tracer");
    return 0;
}

// device FP64 (NY x NX, unpitched) <-> a field of the model (any precision)
static int adj_put(f2d_model_s* m, void* field, const double* src)
{
    const Geom& g = m->g;
    void* d64 = m->es == 8 ? field : m->stage64;
    CK(cudaMemcpy2DAsync(d64, g.P * 8, src, g.NX * 8, g.NX * 8, g.NY, cudaMemcpyDeviceToDevice,
                         m->stream));
    if (m->es == 4) CKI(launch_convert(0, 1, d64, field, g, m->stream));
    return 0;
}

static int adj_take(f2d_model_s* m, const void* field, double* dst)
{
    const Geom& g = m->g;
    const void* d64 = field;
    if (m->es == 4) {
        CKI(launch_convert(1, 0, field, m->stage64, g, m->stream));
        d64 = m->stage64;
    }
    CK(cudaMemcpy2DAsync(dst, g.NX * 8, d64, g.P * 8, g.NX * 8, g.NY, cudaMemcpyDeviceToDevice,
                         m->stream));
    return 0;
}

int f2d_adjoint_forward(f2d_model m, const double* w0, double* wT, int nsteps, double dt,
                        int every)
{
    int e = adj_check(m);
    if (e) return e;
    if (!w0 || !wT || nsteps < 0 || every < 1 || !(dt > 0)) return fail(1, "bad arguments");
    e = ensure_mg(m, 0);
    if (e) return e;
    AdjState& a = m->adj;
    const Geom& g = m->g;
    const size_t fb64 = field_bytes(m, 8), fbs = field_bytes(m, m->es);
    if (!a.yb) {
        double** v[] = {&a.yb, &a.d1, &a.d2, &a.d3, &a.ubx, &a.uby, &a.psib,
                        &a.rbs[0], &a.rbs[1], &a.rbs[2]};
        for (double** p : v)
            if (!(*p = (double*)dalloc(m, fb64))) return fail(2, "out of device memory");
        a.gx = (double*)dalloc(m, 6 * fb64);
        a.gy = (double*)dalloc(m, 6 * fb64);
        a.slot = (int*)dalloc(m, 256);
        if (!a.gx || !a.gy || !a.slot) return fail(2, "out of device memory");
    }
    if (every > a.cap_every) {
        a.arena = dalloc(m, (size_t)every * 9 * fbs);
        if (!a.arena) return fail(2, "out of device memory");
        a.cap_every = every;
        for (int kind : {5, 6})
            for (auto& k : m->gx[kind])
                if (k) {
                    cudaGraphExecDestroy(k);
                    k = nullptr;
                }
    }
    const int nck = nsteps / every + 1;
    while ((int)a.ckpt.size() < nck) {
        void* c = dalloc(m, fbs);
        if (!c) return fail(2, "out of device memory");
        a.ckpt.push_back(c);
    }
    a.nsteps = nsteps;
    a.every = every;
    a.nckpt = nck;
    a.dt = dt;
    if (a.dt_graph != dt)
        for (auto& k : m->gx[6])
            if (k) {
                cudaGraphExecDestroy(k);
                k = nullptr;
            }
    // fixed time step for the stage kernels
    m->dt_const = dt;
    m->cfl_dt = false;
    CK(cudaMemcpyAsync(&m->sc->dt, &m->dt_const, 8, cudaMemcpyHostToDevice, m->stream));
    m->dt_applied = true;
    // the streamfunction cache (3 nsteps + 1 FP64 fields) when it fits in a
    // third of the free device memory
    {
        const long long slots = 3ll * nsteps + 1;
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b));
        if (slots > a.psic_slots && (double)slots * fb64 <= free_b / 3.0) {
            if (a.psic) {
                cudaFree(a.psic);
                a.psic = nullptr;
                a.psic_slots = 0;
            }
            void* p = nullptr;
            if (cudaMalloc(&p, (size_t)slots * fb64) == cudaSuccess) {
                a.psic = (double*)p;
                a.psic_slots = slots;
            }
            for (int kind : {11, 12})
                for (auto& k : m->gx[kind])
                    if (k) {
                        cudaGraphExecDestroy(k);
                        k = nullptr;
                    }
        }
        if (!a.pslot && !(a.pslot = (int*)dalloc(m, 256))) return fail(2, "out of device memory");
        a.use_psic = a.psic && a.psic_slots >= slots;
    }
    if ((e = adj_put(m, fb(m, "omega", m->cur), w0))) return e;
    if ((e = run_graph(m, 0))) return e;
    if (a.use_psic) {
        CK(cudaMemsetAsync(a.pslot, 0, sizeof(int), m->stream));
        if ((e = rec_psi_store(m, m->stream))) return e;
    }
    for (int n = 0; n < nsteps; ++n) {
        if (n % every == 0)
            CK(cudaMemcpyAsync(a.ckpt[n / every], fb(m, "omega", m->cur), fbs,
                               cudaMemcpyDeviceToDevice, m->stream));
        if ((e = run_graph(m, a.use_psic ? 11 : 1))) return e;
    }
    if ((e = adj_take(m, fb(m, "omega", m->cur), wT))) return e;
    (void)g;
    a.ready = true;
    return 0;
}

int f2d_adjoint_backward(f2d_model m, const double* lamT, double* lam0)
{
    int e = adj_check(m);
    if (e) return e;
    AdjState& a = m->adj;
    if (!a.ready) return fail(9, "f2d_adjoint_forward must run first");
    if (!lamT || !lam0) return fail(1, "null argument");
    const Geom& g = m->g;
    const size_t fbs = field_bytes(m, m->es);
    CK(cudaMemcpy2DAsync(a.yb, g.P * 8, lamT, g.NX * 8, g.NX * 8, g.NY,
                         cudaMemcpyDeviceToDevice, m->stream));
    for (double* r : a.rbs) CK(cudaMemsetAsync(r, 0, field_bytes(m, 8), m->stream));
    // the time step of the forward run (the model's dt may have changed)
    m->dt_const = a.dt;
    CK(cudaMemcpyAsync(&m->sc->dt, &m->dt_const, 8, cudaMemcpyHostToDevice, m->stream));
    for (int sgm = a.nckpt - 1; sgm >= 0; --sgm) {
        const int n0 = sgm * a.every;
        const int n = std::min(a.every, a.nsteps - n0);
        if (n <= 0) continue;
        CK(cudaMemcpyAsync(fb(m, "omega", m->cur), a.ckpt[sgm], fbs, cudaMemcpyDeviceToDevice,
                           m->stream));
        if (a.use_psic) {
            // the diagnostics of the checkpoint from the cached streamfunction
            // (slot 3 n0), then the recomputed stages from slots 3 n0 + 1 ..
            const int p0 = 3 * n0;
            CK(cudaMemcpyAsync(a.pslot, &p0, sizeof(int), cudaMemcpyHostToDevice, m->stream));
            if ((e = rec_diag_cached(m, m->stream))) return e;
        } else if ((e = run_graph(m, 0))) {
            return e;
        }
        CK(cudaMemsetAsync(a.slot, 0, sizeof(int), m->stream));
        for (int k = 0; k < n; ++k)
            if ((e = run_graph(m, a.use_psic ? 12 : 5))) return e;
        for (int k = 0; k < n; ++k)
            if ((e = run_graph(m, 6))) return e;
        a.dt_graph = a.dt;
    }
    CK(cudaMemcpy2DAsync(lam0, g.NX * 8, a.yb, g.P * 8, g.NX * 8, g.NY,
                         cudaMemcpyDeviceToDevice, m->stream));
    return 0;
}

}  // extern "C"
