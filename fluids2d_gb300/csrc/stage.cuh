// Launchers of the fused stage and diagnostic kernels (stage.cu).
#pragma once
#include "common.cuh"

namespace f2d {

struct RswIn {
    const void *ux, *uy, *h;        // prognostic, stage input
    const void* w;                  // omega (qgrsw: the wrap of the edge tiles)
    void *uxo, *uyo, *ho;           // prognostic, stage output
    const void *Ux, *Uy, *ke, *p;   // diagnostics of the stage input
    void *dux, *duy, *dh;           // this stage's tendencies (stored if != 0)
    const void *dux1, *duy1, *dh1;  // earlier tendencies
    const void *dux2, *duy2, *dh2;
    const void *fx, *fy, *fh;       // forcing terms added to the tendencies (or null)
    double fc;                      // f0 * area * 0.25 (operators.py:33)
    double bdy;                     // 0.5 * dy (addbuoyancy, operators.py:152-153)
    // 0 rsw; 1 euler (vortex force + grad ke only); 2 boussinesq (euler +
    // buoyancy, with the buoyancy b advected in place of h); 3 qgrsw (the
    // raw tendency of vortex force, Coriolis and mass flux into dux/duy/dh,
    // no update)
    int euler;
};

struct RswDiag {
    const void *ux, *uy, *h;
    void *Ux, *Uy, *omega, *ke, *p;
    double rdx2, rdy2;  // 1/dx**2, 1/dy**2 (operators.py:62-63)
    double goa;         // g/area (operators.py:111)
    int euler;          // euler model: no pressure from h
    int noke;           // qgrsw: no kinetic energy (equations.py:127-133)
};

int launch_fluxform_stage(int method, int prec, const CUtensorMap* tq,
                          const void* qin, void* qout, const void* Ux,
                          const void* Uy, const uint32_t* code, void* ds_out,
                          const void* ds1, const void* ds2, const void* frc, int stage,
                          const Geom& g, DevScalars* sc, cudaStream_t s);
int launch_rsw_stage(int method, int prec, const CUtensorMap* th,
                     const CUtensorMap* tw, const RswIn& a, const uint32_t* code,
                     int stage, const Geom& g, DevScalars* sc, cudaStream_t s);
int launch_rsw_diag(int method, int prec, const CUtensorMap* tux,
                    const CUtensorMap* tuy, const RswDiag& a, const uint32_t* code,
                    const Geom& g, DevScalars* sc, cudaStream_t s);
int launch_c2v(int prec_in, int prec_out, const void* q, void* v, const uint32_t* code,
               const void* fv, const Geom& g, cudaStream_t s);
int launch_perpgrad(int prec_psi, int prec_U, const void* psi, void* Ux, void* Uy,
                    const uint32_t* code, double rdy2, double rdx2, int fillU,
                    const Geom& g, DevScalars* sc, double* partials, cudaStream_t s);
int launch_convert(int prec_in, int prec_out, const void* in, void* out, const Geom& g,
                   cudaStream_t s);
int launch_maxabs2(int prec, const void* Ux, const void* Uy, const Geom& g,
                   DevScalars* sc, double* partials, cudaStream_t s);
int launch_fill_periodic(int prec, void* a, const Geom& g, cudaStream_t s);
int launch_set_dt(DevScalars* sc, cudaStream_t s);
// Warm start of the Poisson solve of SSP-RK3 stage mode+1. The stage states
// are y1 = y0 + dt L1, y2 = y0 + dt/4 (L1 + L2), y3 = y0 + dt/6 (L1 + L2) +
// 2dt/3 L3 (integrators.py:92-107, L_k the tendency at the stage's input),
// and psi solves a linear problem in y, so with S_k = dt A^-1 B(L_k):
// psi1 = psi0 + S1, psi2 = psi0 + (S1 + S2)/4. The guesses extrapolate the
// S_k, not psi: S1 (the tendency at t) ~ the previous step's S2 (taken at
// y1 ~ y(t)); S2 (at y1 ~ t+dt) ~ S1 + the previous step's S2 - S1; S3 (at
// y2 ~ t+dt/2) ~ (S1 + S2)/2. The previous step's increments are kept as
// d1 = 4 psi2 - 3 psi0 - psi1 = S2 and d2 = 4 psi2 - 2 psi0 - 2 psi1 = S2 - S1,
// scaled by dt / dt_warm when the step size changed. On eulerpsi 128^2
// (the oracle's operator) the starting relative residuals of stages 1 and
// 2 fall from 3.8e-4 and 1.9e-4 (linear extrapolation of psi itself) to
// 3.2e-5 and 2.0e-5; stage 3's guess, 2 psi2 - psi0, is the same in both
// (1.3e-5). A guess only moves the solve's starting point.
struct WarmArrays {
    double* psi;  // in: the last solution; out: the guess
    double* s0;   // psi at the step start
    double* p1;   // psi of stage 1
    double* d1;   // the previous step's increments (see above)
    double* d2;
};

// The arrays do not overlap; every load of a point is issued before its
// stores (a store ahead of a load through another pointer would hold the
// load back until the store's address is known not to alias it).
__device__ __forceinline__ void psi_warm_point(int mode, const WarmArrays& w, long long k,
                                               bool hist, double rho)
{
    const double a = w.psi[k];
    if (mode == 0) {  // a = psi0
        const double d1 = hist ? w.d1[k] : 0.0;
        w.s0[k] = a;
        if (hist) w.psi[k] = a + rho * d1;
    } else if (mode == 1) {  // a = psi1
        const double s0 = w.s0[k];
        const double d2 = hist ? w.d2[k] : 0.0;
        w.p1[k] = a;
        double g = s0 + 0.5 * (a - s0);
        if (hist) g += 0.25 * rho * d2;
        w.psi[k] = g;
    } else {  // a = psi2
        const double s0 = w.s0[k], p1 = w.p1[k];
        w.d1[k] = (4.0 * a - 3.0 * s0) - p1;
        w.d2[k] = (4.0 * a - 2.0 * s0) - 2.0 * p1;
        w.psi[k] = 2.0 * a - s0;
    }
}

// psi_warm_point on U pairs of elements (k, k+1), k even and every array
// 16-byte aligned there: 16-byte loads and stores, all the loads of the U
// pairs before any store. ok[u] false skips pair u.
template <int U>
__device__ __forceinline__ void psi_warm_pairs(int mode, const WarmArrays& w,
                                               const long long (&k)[U], const bool (&ok)[U],
                                               bool hist, double rho)
{
    double2 a[U], s0[U], p1[U], d[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const double2 z = make_double2(0.0, 0.0);
        a[u] = ok[u] ? *(const double2*)(w.psi + k[u]) : z;
        s0[u] = ok[u] && mode >= 1 ? *(const double2*)(w.s0 + k[u]) : z;
        p1[u] = ok[u] && mode == 2 ? *(const double2*)(w.p1 + k[u]) : z;
        d[u] = ok[u] && mode == 0 && hist ? *(const double2*)(w.d1 + k[u])
             : (ok[u] && mode == 1 && hist ? *(const double2*)(w.d2 + k[u]) : z);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (!ok[u]) continue;
        const double2 A = a[u], S = s0[u], P = p1[u], D = d[u];
        if (mode == 0) {
            *(double2*)(w.s0 + k[u]) = A;
            if (hist) *(double2*)(w.psi + k[u]) = make_double2(A.x + rho * D.x, A.y + rho * D.y);
        } else if (mode == 1) {
            *(double2*)(w.p1 + k[u]) = A;
            double gx = S.x + 0.5 * (A.x - S.x), gy = S.y + 0.5 * (A.y - S.y);
            if (hist) {
                gx += 0.25 * rho * D.x;
                gy += 0.25 * rho * D.y;
            }
            *(double2*)(w.psi + k[u]) = make_double2(gx, gy);
        } else {
            *(double2*)(w.d1 + k[u]) = make_double2((4.0 * A.x - 3.0 * S.x) - P.x,
                                                    (4.0 * A.y - 3.0 * S.y) - P.y);
            *(double2*)(w.d2 + k[u]) = make_double2((4.0 * A.x - 2.0 * S.x) - 2.0 * P.x,
                                                    (4.0 * A.y - 2.0 * S.y) - 2.0 * P.y);
            *(double2*)(w.psi + k[u]) = make_double2(2.0 * A.x - S.x, 2.0 * A.y - S.y);
        }
    }
}

// the single-model form over n elements (every point; non-fluid points
// stay 0); mode 2 records dt_warm
int launch_psi_warm(int mode, const WarmArrays& w, long long n, DevScalars* sc,
                    cudaStream_t s);
// the failure-detection test switch of the stage kernels' TMA waits, one per
// translation unit (stage.cu, ensemble.cu)
int tma_wait_test_set_stage(int enabled, unsigned long long limit_ns);
int tma_wait_test_set_ensemble(int enabled, unsigned long long limit_ns);
int launch_pushforward(DevScalars* sc, cudaStream_t s);
size_t pt_grid_blocks(const Geom& g);
// euler pressure projection around the Neumann solve
int launch_euler_div(int prec, const void* ux, const void* uy, void* dv, double* rhs,
                     const uint32_t* code, double rdx2, double rdy2, double area,
                     const Geom& g, cudaStream_t s);
// qgrsw: the QG projection of a tendency (or of the state) around the
// Helmholtz solve (qg_projection, operators.py:176-211)
struct QgProj {
    const void *ux, *uy, *h;        // state in (the update's base)
    void *uxo, *uyo, *ho;           // state out
    void *cx, *cy, *ch;             // raw tendency (state form: the state, in place)
    void *sx, *sy, *sh;             // projected tendency out (if store)
    const void *d1x, *d1y, *d1h;    // earlier projected tendencies (RK) or the
    const void *d2x, *d2y, *d2h;    //   filtered previous state (LFRA, d1)
    void *px, *py, *ph;             // LFRA: filtered state out
    const void *fx, *fy, *fh;       // forcing terms added to the projected tendency
    double c2;                      // f0 * area / g (thickness_from_psi)
    double h0;                      // state mode: H * area - hb, else 0
    int mode;                       // 0: tendency + integrator update;
                                    // 1: project the state (cx.. in place);
                                    // 2: the projected tendency into sx.. only
    int store;                      // keep the projected tendency in sx..
};
int launch_qgrsw_pv(int prec, const void* ux, const void* uy, const void* h, double* pv,
                    const uint32_t* code, double cs, double h0, const Geom& g,
                    cudaStream_t s);
int launch_qgrsw_update(int prec, const QgProj& a, const double* psi, const uint32_t* code,
                        int stage, const Geom& g, DevScalars* sc, cudaStream_t s);
// Bulk diagnostics (diagnostics.py:39-57) appended to a device ring
struct BulkArgs {
    const void *ke, *omega, *Ux, *Uy;
    double* ring;      // records of {t, ke, ens, vort, angular}
    int* count;        // records in the ring
    int cap;
    double summsk, area, dx, dy;
};
int launch_bulk(int prec, const BulkArgs& a, const Geom& g, DevScalars* sc, double* partials,
                cudaStream_t s);
// a field as packed (NY, NX) float32 (the history's dtype "f", io.py:71)
int launch_to_f32(int prec, const void* in, float* out, const Geom& g, cudaStream_t s);
int launch_euler_project(int prec, void* ux, void* uy, const double* p, const uint32_t* code,
                         const Geom& g, cudaStream_t s);

}  // namespace f2d
