// Interface reconstructions of the reference's flux methods, as device
// functions templated on the working precision (double or float).
//
// Each function states the reference function it computes
// (pvthinker/Fluids2d, src/fluids2d/weno.py). Operands are combined in the
// reference's order; the compiler may contract a*b+c into an FMA, which moves
// results by rounding only.
#pragma once
#include <cuda_runtime.h>

namespace f2d {

// Order levels: a stencil order o (int8 in the reference) selects the 6-, 4-
// or 2-point formula by o > 4, o > 2, o > 0 (weno.py:352-363). Kernels carry
// the level L = 3, 2, 1, 0 in two bits.
__host__ __device__ inline int order_level(int o)
{
    return o > 4 ? 3 : (o > 2 ? 2 : (o > 0 ? 1 : 0));
}

template <typename T> struct WenoConst;
template <> struct WenoConst<double> {
    static constexpr double eps5 = 1e-16;  // weno5z, weno.py:177
    static constexpr double eps3 = 1e-14;  // weno3z, weno.py:85
};
template <> struct WenoConst<float> {
    static constexpr float eps5 = 1e-16f;
    static constexpr float eps3 = 1e-14f;
};

// weno5z (weno.py:167-197): Borges et al. (2008) WENO-Z, 5th order,
// reconstruction at the face between q0 and qp, upwind side qmm..q0.
template <typename T>
__device__ __forceinline__ T weno5z(T qmm, T qm, T q0, T qp, T qpp)
{
    const T eps = WenoConst<T>::eps5;
    const T c13 = T(1.) / T(3.), c76 = T(7.) / T(6.), c116 = T(11.) / T(6.);
    const T c16 = T(1.) / T(6.), c56 = T(5.) / T(6.);
    T qi1 = (c13 * qmm - c76 * qm) + c116 * q0;
    T qi2 = (-c16 * qm + c56 * q0) + c13 * qp;
    T qi3 = (c13 * q0 + c56 * qp) - c16 * qpp;
    const T k1 = T(13.) / T(12.), k2 = T(0.25);
    T a1 = (qmm - T(2) * qm) + q0, b1 = (qmm - T(4) * qm) + T(3) * q0;
    T a2 = (qm - T(2) * q0) + qp, b2 = qm - qp;
    T a3 = (q0 - T(2) * qp) + qpp, b3 = (T(3) * q0 - T(4) * qp) + qpp;
    T beta1 = k1 * (a1 * a1) + k2 * (b1 * b1);
    T beta2 = k1 * (a2 * a2) + k2 * (b2 * b2);
    T beta3 = k1 * (a3 * a3) + k2 * (b3 * b3);
    T tau5 = fabs(beta1 - beta3);
    T w1 = T(0.1) * (T(1) + tau5 / (beta1 + eps));
    T w2 = T(0.6) * (T(1) + tau5 / (beta2 + eps));
    T w3 = T(0.3) * (T(1) + tau5 / (beta3 + eps));
    return ((w1 * qi1 + w2 * qi2) + w3 * qi3) / ((w1 + w2) + w3);
}

// FP64 form of weno5z with one division instead of four: the weights
// w_k = g_k (1 + tau/d_k), d_k = beta_k + eps, are scaled by d1 d2 d3, so
// W_k = g_k (d_k + tau) prod_{m != k} d_m and the reconstruction is
// sum W_k qi_k / sum W_k - the same value up to rounding. With d_k >= 1e-16
// the products stay far inside the double range (>= 1e-48). On GB300 the
// double divisions dominate the FP64 instruction count of the stencil.
template <>
__device__ __forceinline__ double weno5z<double>(double qmm, double qm, double q0,
                                                 double qp, double qpp)
{
    const double eps = WenoConst<double>::eps5;
    const double c13 = 1. / 3., c76 = 7. / 6., c116 = 11. / 6.;
    const double c16 = 1. / 6., c56 = 5. / 6.;
    const double qi1 = (c13 * qmm - c76 * qm) + c116 * q0;
    const double qi2 = (-c16 * qm + c56 * q0) + c13 * qp;
    const double qi3 = (c13 * q0 + c56 * qp) - c16 * qpp;
    const double k1 = 13. / 12., k2 = 0.25;
    const double a1 = (qmm - 2. * qm) + q0, b1 = (qmm - 4. * qm) + 3. * q0;
    const double a2 = (qm - 2. * q0) + qp, b2 = qm - qp;
    const double a3 = (q0 - 2. * qp) + qpp, b3 = (3. * q0 - 4. * qp) + qpp;
    const double beta1 = k1 * (a1 * a1) + k2 * (b1 * b1);
    const double beta2 = k1 * (a2 * a2) + k2 * (b2 * b2);
    const double beta3 = k1 * (a3 * a3) + k2 * (b3 * b3);
    const double tau5 = fabs(beta1 - beta3);
    const double d1 = beta1 + eps, d2 = beta2 + eps, d3 = beta3 + eps;
    const double W1 = (0.1 * (d1 + tau5)) * (d2 * d3);
    const double W2 = (0.6 * (d2 + tau5)) * (d1 * d3);
    const double W3 = (0.3 * (d3 + tau5)) * (d1 * d2);
    return ((W1 * qi1 + W2 * qi2) + W3 * qi3) / ((W1 + W2) + W3);
}

// FP32 form of weno5z: the three weight quotients tau/d_k and the final
// normalisation use the fast single-precision division (__fdividef, ~2 ulp;
// d_k >= 1e-16 and the denominator of the normalisation is >= 1, far inside
// its range). In FP32 the IEEE division sequences are a large share of the
// stencil's instructions; 2 ulp is within the FP32 form's own rounding.
template <>
__device__ __forceinline__ float weno5z<float>(float qmm, float qm, float q0, float qp,
                                               float qpp)
{
    const float eps = WenoConst<float>::eps5;
    const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f;
    const float c16 = 1.f / 6.f, c56 = 5.f / 6.f;
    const float qi1 = (c13 * qmm - c76 * qm) + c116 * q0;
    const float qi2 = (-c16 * qm + c56 * q0) + c13 * qp;
    const float qi3 = (c13 * q0 + c56 * qp) - c16 * qpp;
    const float k1 = 13.f / 12.f, k2 = 0.25f;
    const float a1 = (qmm - 2.f * qm) + q0, b1 = (qmm - 4.f * qm) + 3.f * q0;
    const float a2 = (qm - 2.f * q0) + qp, b2 = qm - qp;
    const float a3 = (q0 - 2.f * qp) + qpp, b3 = (3.f * q0 - 4.f * qp) + qpp;
    const float beta1 = k1 * (a1 * a1) + k2 * (b1 * b1);
    const float beta2 = k1 * (a2 * a2) + k2 * (b2 * b2);
    const float beta3 = k1 * (a3 * a3) + k2 * (b3 * b3);
    const float tau5 = fabsf(beta1 - beta3);
    const float w1 = 0.1f * (1.f + __fdividef(tau5, beta1 + eps));
    const float w2 = 0.6f * (1.f + __fdividef(tau5, beta2 + eps));
    const float w3 = 0.3f * (1.f + __fdividef(tau5, beta3 + eps));
    return __fdividef((w1 * qi1 + w2 * qi2) + w3 * qi3, (w1 + w2) + w3);
}

// weno3z (weno.py:75-100): WENO-Z, 3rd order.
template <typename T>
__device__ __forceinline__ T weno3z(T qm, T q0, T qp)
{
    const T eps = WenoConst<T>::eps3;
    T qi1 = T(-0.5) * qm + T(1.5) * q0;
    T qi2 = T(0.5) * (q0 + qp);
    T d1 = q0 - qm, d2 = qp - q0;
    T beta1 = d1 * d1, beta2 = d2 * d2;
    T tau = fabs(beta2 - beta1);
    T w1 = (T(1.) / T(3.)) * (T(1) + tau / (beta1 + eps));
    T w2 = (T(2.) / T(3.)) * (T(1) + tau / (beta2 + eps));
    return (w1 * qi1 + w2 * qi2) / (w1 + w2);
}

// FP32 form of weno3z with the fast division (see weno5z<float>).
template <>
__device__ __forceinline__ float weno3z<float>(float qm, float q0, float qp)
{
    const float eps = WenoConst<float>::eps3;
    const float qi1 = -0.5f * qm + 1.5f * q0;
    const float qi2 = 0.5f * (q0 + qp);
    const float d1 = q0 - qm, d2 = qp - q0;
    const float beta1 = d1 * d1, beta2 = d2 * d2;
    const float tau = fabsf(beta2 - beta1);
    const float w1 = (1.f / 3.f) * (1.f + __fdividef(tau, beta1 + eps));
    const float w2 = (2.f / 3.f) * (1.f + __fdividef(tau, beta2 + eps));
    return __fdividef(w1 * qi1 + w2 * qi2, w1 + w2);
}

// FP64 form of weno3z with one division (see weno5z<double>); d_k >= 1e-14.
template <>
__device__ __forceinline__ double weno3z<double>(double qm, double q0, double qp)
{
    const double eps = WenoConst<double>::eps3;
    const double qi1 = -0.5 * qm + 1.5 * q0;
    const double qi2 = 0.5 * (q0 + qp);
    const double e1 = q0 - qm, e2 = qp - q0;
    const double beta1 = e1 * e1, beta2 = e2 * e2;
    const double tau = fabs(beta2 - beta1);
    const double d1 = beta1 + eps, d2 = beta2 + eps;
    const double W1 = ((1. / 3.) * (d1 + tau)) * d2;
    const double W2 = ((2. / 3.) * (d2 + tau)) * d1;
    return (W1 * qi1 + W2 * qi2) / (W1 + W2);
}

// up3 / up5 (weno.py:36-43): linear upwind reconstructions.
template <typename T> __device__ __forceinline__ T up3(T qm, T q0, T qp)
{
    return ((T(5) * q0 + T(2) * qp) - qm) / T(6);
}
template <typename T>
__device__ __forceinline__ T up5(T qmmm, T qmm, T qm, T qp, T qpp)
{
    return ((((T(2) * qmmm - T(13) * qmm) + T(47) * qm) + T(27) * qp) -
            T(3) * qpp) / T(60);
}

// ce2 / ce4 / ce6 (weno.py:21-33): centred reconstructions.
template <typename T> __device__ __forceinline__ T ce2(T qm, T qp)
{
    return (qm + qp) * T(0.5);
}
template <typename T> __device__ __forceinline__ T ce4(T qmm, T qm, T qp, T qpp)
{
    return ((-qmm + T(7) * (qm + qp)) - qpp) / T(12);
}
template <typename T>
__device__ __forceinline__ T ce6(T qmmm, T qmm, T qm, T qp, T qpp, T qppp)
{
    return (((qmmm - T(8) * (qmm + qpp)) + T(37) * (qm + qp)) + qppp) / T(60);
}

// cweno3z (weno.py:103-134).
template <typename T>
__device__ __forceinline__ T cweno3z(T U, T qmm, T qm, T qp, T qpp)
{
    const T eps = WenoConst<T>::eps3;
    T qi1 = T(-0.5) * qmm + T(1.5) * qm;
    T qi2 = T(0.5) * (qm + qp);
    T qi3 = T(-0.5) * qpp + T(1.5) * qp;
    T beta1, beta2;
    if (U > T(0)) {
        T d1 = qm - qmm, d2 = qp - qm;
        beta1 = d1 * d1;
        beta2 = d2 * d2;
    } else {
        T d1 = qp - qpp, d2 = qp - qm;
        beta1 = d1 * d1;
        beta2 = d2 * d2;
    }
    T tau = fabs(beta2 - beta1);
    T w1 = (T(1.) / T(3.)) * (T(1) + tau / (beta1 + eps));
    T w2 = (T(2.) / T(3.)) * (T(1) + tau / (beta2 + eps));
    return (w1 * (qi1 + qi3) * T(0.5) + w2 * qi2) / (w1 + w2);
}

// cweno5z_v0 (weno.py:255-300).
template <typename T>
__device__ __forceinline__ T cweno5z(T qmmm, T qmm, T qm, T qp, T qpp, T qppp)
{
    const T eps = WenoConst<T>::eps5;
    const T c13 = T(1.) / T(3.), c76 = T(7.) / T(6.), c116 = T(11.) / T(6.);
    const T c16 = T(1.) / T(6.), c56 = T(5.) / T(6.);
    T qi1 = (c13 * qmmm - c76 * qmm) + c116 * qm;
    T qi2 = (-c16 * qmm + c56 * qm) + c13 * qp;
    T qi3 = (c13 * qm + c56 * qp) - c16 * qpp;
    T qi4 = (c13 * qp + c56 * qm) - c16 * qmm;
    T qi5 = (-c16 * qpp + c56 * qp) + c13 * qm;
    T qi6 = (c13 * qppp - c76 * qpp) + c116 * qp;
    const T k1 = T(13.) / T(12.), k2 = T(0.25);
    T a1 = (qmmm - T(2) * qmm) + qm, b1 = (qmmm - T(4) * qmm) + T(3) * qm;
    T a2 = (qmm - T(2) * qm) + qp, b2 = qmm - qp;
    T a3 = (qm - T(2) * qp) + qpp, b3 = (T(3) * qm - T(4) * qp) + qpp;
    T beta1 = k1 * (a1 * a1) + k2 * (b1 * b1);
    T beta2 = k1 * (a2 * a2) + k2 * (b2 * b2);
    T beta3 = k1 * (a3 * a3) + k2 * (b3 * b3);
    T tau5 = fabs(beta1 - beta3);
    T w1 = T(0.1) * (T(1) + tau5 / (beta1 + eps));
    T w2 = T(0.6) * (T(1) + tau5 / (beta2 + eps));
    T w3 = T(0.3) * (T(1) + tau5 / (beta3 + eps));
    return ((w1 * (qi1 + qi6) + w2 * (qi2 + qi5)) + w3 * (qi3 + qi4)) /
           (T(2) * ((w1 + w2) + w3));
}

enum { METHOD_WENO = 0, METHOD_UPWIND = 1, METHOD_CENTERED = 2,
       METHOD_CWENO = 3,
       METHOD_CLASSIC = 4 /* innerproduct only: the 4-point kinetic energy */ };

// The reference's (f1, f3, f5) triple of each method (weno.py:303-343).
// Stencil values are q[-3..+2] around the face for the 6-point formula
// (q0 = qmmm ... q5 = qppp); the face lies between q2 and q3.
template <int M, typename T>
__device__ __forceinline__ T flux6(T U, T q0, T q1, T q2, T q3, T q4, T q5)
{
    if (M == METHOD_CENTERED) return ce6<T>(q0, q1, q2, q3, q4, q5);
    if (M == METHOD_CWENO) return cweno5z<T>(q0, q1, q2, q3, q4, q5);
    // upwind side chosen by the sign of U, mirrored stencil otherwise; the
    // operands are selected first so that one reconstruction is evaluated
    const bool up = U > T(0);
    const T a = up ? q0 : q5, b = up ? q1 : q4, c = up ? q2 : q3;
    const T d = up ? q3 : q2, e = up ? q4 : q1;
    if (M == METHOD_WENO) return weno5z<T>(a, b, c, d, e);
    return up5<T>(a, b, c, d, e);
}

template <int M, typename T>
__device__ __forceinline__ T flux4(T U, T q1, T q2, T q3, T q4)
{
    if (M == METHOD_CENTERED) return ce4<T>(q1, q2, q3, q4);
    if (M == METHOD_CWENO) return cweno3z<T>(U, q1, q2, q3, q4);
    const bool up = U > T(0);
    const T a = up ? q1 : q4, b = up ? q2 : q3, c = up ? q3 : q2;
    if (M == METHOD_WENO) return weno3z<T>(a, b, c);
    return up3<T>(a, b, c);
}

template <int M, typename T> __device__ __forceinline__ T flux2(T U, T q2, T q3)
{
    if (M == METHOD_WENO || M == METHOD_UPWIND) return U > T(0) ? q2 : q3;
    return ce2<T>(q2, q3);
}

// Reconstructed value at a face for order level L from the 6-point window
// q0..q5 (face between q2 and q3). L = 0 returns 0.
template <int M, typename T>
__device__ __forceinline__ T face_value(int L, T U, T q0, T q1, T q2, T q3,
                                        T q4, T q5)
{
    if (L == 3) return flux6<M, T>(U, q0, q1, q2, q3, q4, q5);
    if (L == 2) return flux4<M, T>(U, q1, q2, q3, q4);
    if (L == 1) return flux2<M, T>(U, q2, q3);
    return T(0);
}

}  // namespace f2d
