// Discrete adjoint of the eulerpsi time step (vorticity / streamfunction on
// a closed basin): vector-Jacobian products of the flux-form tendency
//
//   D(w) = -div( phi(U, w) U ) * msk        (divflux, operators.py:21-29)
//   U    = perpgrad( A^-1 c2v(w) )          (equations.py:73-86,
//                                             operators.py:126-149)
//
// and of the SSP-RK3 stage combinations (integrators.py:92-107), with the
// time step held fixed. Every factor is differentiated exactly, including
// the nonlinear WENO-Z smoothness weights (weno.py:75-100, 167-197); the
// upwind selection by the sign of U is piecewise constant, so the face value
// has no derivative with respect to U and dF/dU = phi. The Poisson factor is
// self-adjoint: its adjoint is the same masked solve (done by the caller).
//
// The adjoint arithmetic is FP64 whatever the forward precision; the stage
// states and face velocities it linearises about come from snapshots taken
// while the forward steps are recomputed from a checkpoint.
#include "adjoint.cuh"
#include "weno.cuh"

namespace f2d {

// ---- face values with their gradient w.r.t. the stencil ------------------
// weno5z (weno.py:167-197) on (a, b, c, d, e) = (qmm, qm, q0, qp, qpp) and its
// gradient, by reverse accumulation through the formula.
__device__ __forceinline__ double weno5z_grad(double a, double b, double c, double d,
                                              double e, double (&g)[5])
{
    const double eps = 1e-16;
    const double c13 = 1. / 3., c76 = 7. / 6., c116 = 11. / 6., c16 = 1. / 6., c56 = 5. / 6.;
    const double qi1 = (c13 * a - c76 * b) + c116 * c;
    const double qi2 = (-c16 * b + c56 * c) + c13 * d;
    const double qi3 = (c13 * c + c56 * d) - c16 * e;
    const double k1 = 13. / 12., k2 = 0.25;
    const double a1 = (a - 2 * b) + c, b1 = (a - 4 * b) + 3 * c;
    const double a2 = (b - 2 * c) + d, b2 = b - d;
    const double a3 = (c - 2 * d) + e, b3 = (3 * c - 4 * d) + e;
    const double be1 = k1 * (a1 * a1) + k2 * (b1 * b1);
    const double be2 = k1 * (a2 * a2) + k2 * (b2 * b2);
    const double be3 = k1 * (a3 * a3) + k2 * (b3 * b3);
    const double t13 = be1 - be3;
    const double tau = fabs(t13);
    const double d1 = be1 + eps, d2 = be2 + eps, d3 = be3 + eps;
    const double w1 = 0.1 * (1 + tau / d1), w2 = 0.6 * (1 + tau / d2),
                 w3 = 0.3 * (1 + tau / d3);
    const double S = (w1 + w2) + w3;
    const double phi = ((w1 * qi1 + w2 * qi2) + w3 * qi3) / S;
    // reverse sweep, phi_bar = 1
    const double iS = 1 / S;
    const double q1b = w1 * iS, q2b = w2 * iS, q3b = w3 * iS;
    const double w1b = (qi1 - phi) * iS, w2b = (qi2 - phi) * iS, w3b = (qi3 - phi) * iS;
    const double taub = w1b * 0.1 / d1 + w2b * 0.6 / d2 + w3b * 0.3 / d3;
    double be1b = -w1b * 0.1 * tau / (d1 * d1);
    const double be2b = -w2b * 0.6 * tau / (d2 * d2);
    double be3b = -w3b * 0.3 * tau / (d3 * d3);
    const double sg = t13 > 0 ? 1.0 : (t13 < 0 ? -1.0 : 0.0);
    be1b += sg * taub;
    be3b -= sg * taub;
    const double a1b = 2 * k1 * a1 * be1b, b1b = 2 * k2 * b1 * be1b;
    const double a2b = 2 * k1 * a2 * be2b, b2b = 2 * k2 * b2 * be2b;
    const double a3b = 2 * k1 * a3 * be3b, b3b = 2 * k2 * b3 * be3b;
    g[0] = c13 * q1b + a1b + b1b;
    g[1] = -c76 * q1b - c16 * q2b - 2 * a1b - 4 * b1b + a2b + b2b;
    g[2] = c116 * q1b + c56 * q2b + c13 * q3b + a1b + 3 * b1b - 2 * a2b + a3b + 3 * b3b;
    g[3] = c13 * q2b + c56 * q3b + a2b - b2b - 2 * a3b - 4 * b3b;
    g[4] = -c16 * q3b + a3b + b3b;
    return phi;
}

// weno3z (weno.py:75-100) on (a, b, c) = (qm, q0, qp) and its gradient
__device__ __forceinline__ double weno3z_grad(double a, double b, double c, double (&g)[3])
{
    const double eps = 1e-14;
    const double qi1 = -0.5 * a + 1.5 * b, qi2 = 0.5 * (b + c);
    const double e1 = b - a, e2 = c - b;
    const double be1 = e1 * e1, be2 = e2 * e2;
    const double t21 = be2 - be1;
    const double tau = fabs(t21);
    const double d1 = be1 + eps, d2 = be2 + eps;
    const double w1 = (1. / 3.) * (1 + tau / d1), w2 = (2. / 3.) * (1 + tau / d2);
    const double S = w1 + w2;
    const double phi = (w1 * qi1 + w2 * qi2) / S;
    const double iS = 1 / S;
    const double q1b = w1 * iS, q2b = w2 * iS;
    const double w1b = (qi1 - phi) * iS, w2b = (qi2 - phi) * iS;
    const double taub = w1b * (1. / 3.) / d1 + w2b * (2. / 3.) / d2;
    double be1b = -w1b * (1. / 3.) * tau / (d1 * d1);
    double be2b = -w2b * (2. / 3.) * tau / (d2 * d2);
    const double sg = t21 > 0 ? 1.0 : (t21 < 0 ? -1.0 : 0.0);
    be2b += sg * taub;
    be1b -= sg * taub;
    const double e1b = 2 * e1 * be1b, e2b = 2 * e2 * be2b;
    g[0] = -0.5 * q1b - e1b;
    g[1] = 1.5 * q1b + 0.5 * q2b + e1b - e2b;
    g[2] = 0.5 * q2b + e2b;
    return phi;
}

// Face value for order level L from the 6-point window q[0..5] (face between
// q[2] and q[3]) and its gradient g[0..5] w.r.t. the window; methods WENO
// and UPWIND (f1, f3, f5 of weno.py:303-343).
template <int M>
__device__ __forceinline__ double face_value_grad(int L, double U, const double (&q)[6],
                                                  double (&g)[6])
{
#pragma unroll
    for (int k = 0; k < 6; ++k) g[k] = 0.0;
    const bool up = U > 0;
    if (L == 3) {
        // upwind: (a..e) = q0..q4; otherwise the mirrored q5..q1
        const double a = up ? q[0] : q[5], b = up ? q[1] : q[4], c = up ? q[2] : q[3];
        const double d = up ? q[3] : q[2], e = up ? q[4] : q[1];
        double h[5];
        double phi;
        if (M == METHOD_WENO) {
            phi = weno5z_grad(a, b, c, d, e, h);
        } else {  // up5 (weno.py:40-43)
            phi = ((((2 * a - 13 * b) + 47 * c) + 27 * d) - 3 * e) / 60;
            h[0] = 2. / 60;
            h[1] = -13. / 60;
            h[2] = 47. / 60;
            h[3] = 27. / 60;
            h[4] = -3. / 60;
        }
        if (up) {
#pragma unroll
            for (int k = 0; k < 5; ++k) g[k] = h[k];
        } else {
#pragma unroll
            for (int k = 0; k < 5; ++k) g[5 - k] = h[k];
        }
        return phi;
    }
    if (L == 2) {
        const double a = up ? q[1] : q[4], b = up ? q[2] : q[3], c = up ? q[3] : q[2];
        double h[3];
        double phi;
        if (M == METHOD_WENO) {
            phi = weno3z_grad(a, b, c, h);
        } else {  // up3 (weno.py:36-38)
            phi = ((5 * b + 2 * c) - a) / 6;
            h[0] = -1. / 6;
            h[1] = 5. / 6;
            h[2] = 2. / 6;
        }
        if (up) {
            g[1] = h[0];
            g[2] = h[1];
            g[3] = h[2];
        } else {
            g[4] = h[0];
            g[3] = h[1];
            g[2] = h[2];
        }
        return phi;
    }
    if (L == 1) {
        g[up ? 2 : 3] = 1.0;
        return up ? q[2] : q[3];
    }
    return 0.0;
}

// ---- kernels ---------------------------------------------------------------
__device__ __forceinline__ bool pt(const Geom& g, int& j, int& i, long long& o)
{
    i = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    o = (long long)j * g.P + i;
    return j < g.NY && i < g.NX;
}

template <typename T>
__device__ __forceinline__ double ld(const T* a, const Geom& g, int j, int i)
{
    return (j >= 0 && j < g.NY && i >= 0 && i < g.NX) ? (double)a[(long long)j * g.P + i] : 0.0;
}

// Snapshot of (w, U.x, U.y) into slot *slot of the arena
template <typename T>
__global__ void k_adj_snap(const T* __restrict__ w, const T* __restrict__ ux,
                           const T* __restrict__ uy, T* __restrict__ arena, long long fsz,
                           const int* __restrict__ slot)
{
    const long long n = fsz;
    T* dst = arena + (long long)(*slot) * 3 * fsz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        dst[k] = w[k];
        dst[fsz + k] = ux[k];
        dst[2 * fsz + k] = uy[k];
    }
}

__global__ void k_adj_slot(int* slot, int delta) { *slot += delta; }

// The per-stage cache of the forward streamfunctions: store cache[*slot] =
// psi, or restore psi = cache[*slot] (fields of fsz FP64 elements).
__global__ void k_adj_psi(double* __restrict__ psi, double* __restrict__ cache, long long fsz,
                          const int* __restrict__ slot, int store)
{
    double* c = cache + (long long)(*slot) * fsz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < fsz;
         k += (long long)gridDim.x * blockDim.x) {
        if (store) c[k] = psi[k];
        else psi[k] = c[k];
    }
}

// RK3 combinations of the adjoint (integrators.py:92-107 reversed):
// mode 0: d3 = c3 y, d2 = c2 y, d1 = c1 y; mode 1: d1 += c1 y, d2 += c2 y;
// mode 2: d1 += c1 y
__global__ void k_adj_comb(Geom g, const double* __restrict__ yb, double* __restrict__ d1,
                           double* __restrict__ d2, double* __restrict__ d3, int mode,
                           double c1, double c2, double c3)
{
    int j, i;
    long long o;
    if (!pt(g, j, i, o)) return;
    const double y = yb[o];
    if (mode == 0) {
        d3[o] = c3 * y;
        d2[o] = c2 * y;
        d1[o] = c1 * y;
    } else if (mode == 1) {
        d1[o] += c1 * y;
        d2[o] += c2 * y;
    } else {
        d1[o] += c1 * y;
    }
}

// Faces: with mu = db * msk, the flux adjoint of face (j,i) of x is
// mu(j,i) - mu(j,i-1) (div, operators.py:104-107); its face-velocity adjoint
// is Fb * phi and the window cells get Fb * U * dphi/dq_k (plane k of gx).
// Same for the y-faces.
template <typename T, int M>
__global__ void k_adj_faces(Geom g, const uint32_t* __restrict__ code, const T* __restrict__ arena,
                            long long fsz, const int* __restrict__ slot, int soff,
                            const double* __restrict__ db, double* __restrict__ gx,
                            double* __restrict__ gy, double* __restrict__ ubx,
                            double* __restrict__ uby)
{
    int j, i;
    long long o;
    if (!pt(g, j, i, o)) return;
    const T* w = arena + (long long)(*slot + soff) * 3 * fsz;
    const T* Ux = w + fsz;
    const T* Uy = w + 2 * fsz;
    const uint32_t cd = code[o];
    const double mu = (cd & B_MSK) ? db[o] : 0.0;
    // x-face
    {
        const int L = lev(cd, SH_OCX);
        double ub = 0.0, gk[6] = {0, 0, 0, 0, 0, 0};
        if (L) {
            const double muL = (i >= 1 && (code[o - 1] & B_MSK)) ? db[o - 1] : 0.0;
            const double Fb = mu - muL;
            const double U = (double)Ux[o];
            double q[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) q[k] = ld(w, g, j, i - 3 + k);
            double dg[6];
            const double phi = face_value_grad<M>(L, U, q, dg);
            ub = Fb * phi;
#pragma unroll
            for (int k = 0; k < 6; ++k) gk[k] = Fb * U * dg[k];
        }
        ubx[o] = ub;
#pragma unroll
        for (int k = 0; k < 6; ++k) gx[k * fsz + o] = gk[k];
    }
    // y-face
    {
        const int L = lev(cd, SH_OCY);
        double ub = 0.0, gk[6] = {0, 0, 0, 0, 0, 0};
        if (L) {
            const double muS = (j >= 1 && (code[o - g.P] & B_MSK)) ? db[o - g.P] : 0.0;
            const double Fb = mu - muS;
            const double U = (double)Uy[o];
            double q[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) q[k] = ld(w, g, j - 3 + k, i);
            double dg[6];
            const double phi = face_value_grad<M>(L, U, q, dg);
            ub = Fb * phi;
#pragma unroll
            for (int k = 0; k < 6; ++k) gk[k] = Fb * U * dg[k];
        }
        uby[o] = ub;
#pragma unroll
        for (int k = 0; k < 6; ++k) gy[k * fsz + o] = gk[k];
    }
}

// Vertices: psi_bar = perpgrad^T (U_bar) (operators.py:144-149 transposed),
// kept at the fluid vertices of the Poisson problem (the right-hand side of
// the adjoint solve).
__global__ void k_adj_psib(Geom g, const uint32_t* __restrict__ code,
                           const double* __restrict__ ubx, const double* __restrict__ uby,
                           double rdx2, double rdy2, double* __restrict__ psib)
{
    int j, i;
    long long o;
    if (!pt(g, j, i, o)) return;
    const uint32_t cd = code[o];
    double v = 0.0;
    if (cd & B_GV) {
        // U.x(j,i) = -(psi(j+1,i) - psi(j,i)) mskx rdy2 for j <= NY-2
        if (j <= g.NY - 2 && (cd & B_MSKX)) v += ubx[o] * rdy2;
        if (j >= 1 && (code[o - g.P] & B_MSKX)) v -= ubx[o - g.P] * rdy2;
        // U.y(j,i) = (psi(j,i+1) - psi(j,i)) msky rdx2 for i <= NX-2
        if (i <= g.NX - 2 && (cd & B_MSKY)) v -= uby[o] * rdx2;
        if (i >= 1 && (code[o - 1] & B_MSKY)) v += uby[o - 1] * rdx2;
    }
    psib[o] = v;
}

// Cells: yb += the window gathers of the face gradients (a cell is window
// point k of the x-face i+3-k and of the y-face j+3-k) and c2v^T of the
// adjoint solution rb (operators.py:126-133 transposed).
__global__ void k_adj_cells(Geom g, const uint32_t* __restrict__ code,
                            const double* __restrict__ gx, const double* __restrict__ gy,
                            long long fsz, const double* __restrict__ rb,
                            double* __restrict__ yb)
{
    int j, i;
    long long o;
    if (!pt(g, j, i, o)) return;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int fi = i + 3 - k;
        if (fi >= 0 && fi < g.NX) acc += gx[k * fsz + o + (fi - i)];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const int fj = j + 3 - k;
        if (fj >= 0 && fj < g.NY) acc += gy[k * fsz + o + (long long)(fj - j) * g.P];
    }
    double v = 0.0;
#pragma unroll
    for (int dj = 0; dj < 2; ++dj)
#pragma unroll
        for (int di = 0; di < 2; ++di) {
            const int vj = j + dj, vi = i + di;
            if (vj >= 1 && vi >= 1 && vj < g.NY && vi < g.NX) {
                const long long ov = (long long)vj * g.P + vi;
                if (code[ov] & B_MSKV) v += rb[ov];
            }
        }
    yb[o] += acc + 0.25 * v;
}

// ---- launchers -----------------------------------------------------------------
static dim3 grid2(const Geom& g) { return dim3((g.NX + 31) / 32, (g.NY + 7) / 8); }

int launch_adj_snap(int prec, const void* w, const void* ux, const void* uy, void* arena,
                    long long fsz, const int* slot, cudaStream_t s)
{
    const int nb = (int)std::min<long long>((fsz + 255) / 256, 152 * 8);
    if (prec == 0)
        k_adj_snap<double><<<nb, 256, 0, s>>>((const double*)w, (const double*)ux,
                                              (const double*)uy, (double*)arena, fsz, slot);
    else
        k_adj_snap<float><<<nb, 256, 0, s>>>((const float*)w, (const float*)ux,
                                             (const float*)uy, (float*)arena, fsz, slot);
    return (int)cudaGetLastError();
}

int launch_adj_psi(double* psi, double* cache, long long fsz, const int* slot, int store,
                   cudaStream_t s)
{
    const int nb = (int)std::min<long long>((fsz + 255) / 256, 152 * 8);
    k_adj_psi<<<nb, 256, 0, s>>>(psi, cache, fsz, slot, store);
    return (int)cudaGetLastError();
}

int launch_adj_slot(int* slot, int delta, cudaStream_t s)
{
    k_adj_slot<<<1, 1, 0, s>>>(slot, delta);
    return (int)cudaGetLastError();
}

int launch_adj_comb(const Geom& g, const double* yb, double* d1, double* d2, double* d3,
                    int mode, double c1, double c2, double c3, cudaStream_t s)
{
    k_adj_comb<<<grid2(g), dim3(32, 8), 0, s>>>(g, yb, d1, d2, d3, mode, c1, c2, c3);
    return (int)cudaGetLastError();
}

int launch_adj_vjp_pre(int method, int prec, const Geom& g, const uint32_t* code,
                       const void* arena, long long fsz, const int* slot, int soff,
                       const double* db, double* gx, double* gy, double* ubx, double* uby,
                       double rdx2, double rdy2, double* psib, cudaStream_t s)
{
    const dim3 gr = grid2(g), bl(32, 8);
#define F2D_ADJ_FACES(T, M)                                                               \
    k_adj_faces<T, M><<<gr, bl, 0, s>>>(g, code, (const T*)arena, fsz, slot, soff, db, gx, gy, \
                                        ubx, uby)
    if (prec == 0) {
        if (method == METHOD_WENO) F2D_ADJ_FACES(double, METHOD_WENO);
        else F2D_ADJ_FACES(double, METHOD_UPWIND);
    } else {
        if (method == METHOD_WENO) F2D_ADJ_FACES(float, METHOD_WENO);
        else F2D_ADJ_FACES(float, METHOD_UPWIND);
    }
#undef F2D_ADJ_FACES
    k_adj_psib<<<gr, bl, 0, s>>>(g, code, ubx, uby, rdx2, rdy2, psib);
    return (int)cudaGetLastError();
}

int launch_adj_vjp_post(const Geom& g, const uint32_t* code, const double* gx, const double* gy,
                        long long fsz, const double* rb, double* yb, cudaStream_t s)
{
    k_adj_cells<<<grid2(g), dim3(32, 8), 0, s>>>(g, code, gx, gy, fsz, rb, yb);
    return (int)cudaGetLastError();
}

}  // namespace f2d
