/*
 * ORACLE - test infrastructure only. Included twice by sweeps.c with
 * different SQ()/SFX() definitions (see the comment there).
 *
 * Each function restates the reference function named beside it
 * (src/fluids2d/weno.py); operands are combined in the reference's order.
 */
#ifndef F2D_ORACLE_BODY
#error "include through sweeps.c"
#endif

/* ce2/ce4/ce6, weno.py:21-33 */
static inline double SFX(o_ce2)(double U, double qm, double qp)
{
    (void)U;
    return (qm + qp) * 0.5;
}
static inline double SFX(o_ce4)(double U, double qmm, double qm, double qp,
                                double qpp)
{
    (void)U;
    return ((-qmm + 7.0 * (qm + qp)) - qpp) / 12.0;
}
static inline double SFX(o_ce6)(double U, double qmmm, double qmm, double qm,
                                double qp, double qpp, double qppp)
{
    (void)U;
    return (((qmmm - 8.0 * (qmm + qpp)) + 37.0 * (qm + qp)) + qppp) / 60.0;
}

/* up3/up5, weno.py:36-43 */
static inline double SFX(o_up3)(double qm, double q0, double qp)
{
    return ((5.0 * q0 + 2.0 * qp) - qm) / 6.0;
}
static inline double SFX(o_up5)(double qmmm, double qmm, double qm, double qp,
                                double qpp)
{
    return ((((2.0 * qmmm - 13.0 * qmm) + 47.0 * qm) + 27.0 * qp) - 3.0 * qpp)
           / 60.0;
}

/* weno3z, weno.py:75-100 (Borges et al. 2008, 3rd order) */
static inline double SFX(o_weno3z)(double qm, double q0, double qp)
{
    const double eps = 1e-14;
    double qi1 = (-1. / 2.) * qm + (3. / 2.) * q0;
    double qi2 = (1. / 2.) * (q0 + qp);
    double beta1 = SQ(q0 - qm);
    double beta2 = SQ(qp - q0);
    double tau = fabs(beta2 - beta1);
    const double g1 = 1. / 3., g2 = 2. / 3.;
    double w1 = g1 * (1. + tau / (beta1 + eps));
    double w2 = g2 * (1. + tau / (beta2 + eps));
    return (w1 * qi1 + w2 * qi2) / (w1 + w2);
}

/* cweno3z, weno.py:103-134 */
static inline double SFX(o_cweno3z)(double U, double qmm, double qm, double qp,
                                    double qpp)
{
    const double eps = 1e-14;
    double qi1 = (-1. / 2.) * qmm + (3. / 2.) * qm;
    double qi2 = (1. / 2.) * (qm + qp);
    double qi3 = (-1. / 2.) * qpp + (3. / 2.) * qp;
    double beta1, beta2;
    if (U > 0) {
        beta1 = SQ(qm - qmm);
        beta2 = SQ(qp - qm);
    } else {
        beta1 = SQ(qp - qpp);
        beta2 = SQ(qp - qm);
    }
    double tau = fabs(beta2 - beta1);
    const double g1 = 1. / 3., g2 = 2. / 3.;
    double w1 = g1 * (1. + tau / (beta1 + eps));
    double w2 = g2 * (1. + tau / (beta2 + eps));
    return (w1 * (qi1 + qi3) * 0.5 + w2 * qi2) / (w1 + w2);
}

/* weno5z, weno.py:167-197 (Borges et al. 2008, 5th order) */
static inline double SFX(o_weno5z)(double qmm, double qm, double q0, double qp,
                                   double qpp)
{
    const double eps = 1e-16;
    double qi1 = ((1. / 3.) * qmm - (7. / 6.) * qm) + (11. / 6.) * q0;
    double qi2 = ((-1. / 6.) * qm + (5. / 6.) * q0) + (1. / 3.) * qp;
    double qi3 = ((1. / 3.) * q0 + (5. / 6.) * qp) - (1. / 6.) * qpp;
    const double k1 = 13. / 12., k2 = 0.25;
    double beta1 = k1 * SQ((qmm - 2.0 * qm) + q0)
                 + k2 * SQ((qmm - 4.0 * qm) + 3.0 * q0);
    double beta2 = k1 * SQ((qm - 2.0 * q0) + qp) + k2 * SQ(qm - qp);
    double beta3 = k1 * SQ((q0 - 2.0 * qp) + qpp)
                 + k2 * SQ((3.0 * q0 - 4.0 * qp) + qpp);
    double tau5 = fabs(beta1 - beta3);
    const double g1 = 0.1, g2 = 0.6, g3 = 0.3;
    double w1 = g1 * (1.0 + tau5 / (beta1 + eps));
    double w2 = g2 * (1.0 + tau5 / (beta2 + eps));
    double w3 = g3 * (1.0 + tau5 / (beta3 + eps));
    return ((w1 * qi1 + w2 * qi2) + w3 * qi3) / ((w1 + w2) + w3);
}

/* cweno5z_v0, weno.py:255-300 (the "cweno" 6-point flux) */
static inline double SFX(o_cweno5z_v0)(double U, double qmmm, double qmm,
                                       double qm, double qp, double qpp,
                                       double qppp)
{
    (void)U;
    const double eps = 1e-16;
    double qi1 = ((1. / 3.) * qmmm - (7. / 6.) * qmm) + (11. / 6.) * qm;
    double qi2 = ((-1. / 6.) * qmm + (5. / 6.) * qm) + (1. / 3.) * qp;
    double qi3 = ((1. / 3.) * qm + (5. / 6.) * qp) - (1. / 6.) * qpp;
    double qi4 = ((1. / 3.) * qp + (5. / 6.) * qm) - (1. / 6.) * qmm;
    double qi5 = ((-1. / 6.) * qpp + (5. / 6.) * qp) + (1. / 3.) * qm;
    double qi6 = ((1. / 3.) * qppp - (7. / 6.) * qpp) + (11. / 6.) * qp;
    const double k1 = 13. / 12., k2 = 0.25;
    /* both branches of the reference compute the same betas */
    double beta1 = k1 * SQ((qmmm - 2.0 * qmm) + qm)
                 + k2 * SQ((qmmm - 4.0 * qmm) + 3.0 * qm);
    double beta2 = k1 * SQ((qmm - 2.0 * qm) + qp) + k2 * SQ(qmm - qp);
    double beta3 = k1 * SQ((qm - 2.0 * qp) + qpp)
                 + k2 * SQ((3.0 * qm - 4.0 * qp) + qpp);
    double tau5 = fabs(beta1 - beta3);
    const double g1 = 0.1, g2 = 0.6, g3 = 0.3;
    double w1 = g1 * (1.0 + tau5 / (beta1 + eps));
    double w2 = g2 * (1.0 + tau5 / (beta2 + eps));
    double w3 = g3 * (1.0 + tau5 / (beta3 + eps));
    return ((w1 * (qi1 + qi6) + w2 * (qi2 + qi5)) + w3 * (qi3 + qi4))
           / (2.0 * ((w1 + w2) + w3));
}

/* f1 / f3 / f5 of each method (weno.py:303-343) */
static inline double SFX(o_f1)(int method, double U, double qm, double qp)
{
    if (method == 0 || method == 1) return U > 0 ? qm : qp; /* flx1 */
    return SFX(o_ce2)(U, qm, qp);                           /* ce2  */
}

static inline double SFX(o_f3)(int method, double U, double qmm, double qm,
                               double qp, double qpp)
{
    switch (method) {
    case 0: /* flx3 */
        return U > 0 ? SFX(o_weno3z)(qmm, qm, qp) : SFX(o_weno3z)(qpp, qp, qm);
    case 1: /* flxup3 */
        return U > 0 ? SFX(o_up3)(qmm, qm, qp) : SFX(o_up3)(qpp, qp, qm);
    case 2: /* ce4 */
        return SFX(o_ce4)(U, qmm, qm, qp, qpp);
    default: /* cflx3 */
        return SFX(o_cweno3z)(U, qmm, qm, qp, qpp);
    }
}

static inline double SFX(o_f5)(int method, double U, double qmmm, double qmm,
                               double qm, double qp, double qpp, double qppp)
{
    switch (method) {
    case 0: /* flx5 */
        return U > 0 ? SFX(o_weno5z)(qmmm, qmm, qm, qp, qpp)
                     : SFX(o_weno5z)(qppp, qpp, qp, qm, qmm);
    case 1: /* flxup5 */
        return U > 0 ? SFX(o_up5)(qmmm, qmm, qm, qp, qpp)
                     : SFX(o_up5)(qppp, qpp, qp, qm, qmm);
    case 2: /* ce6 */
        return SFX(o_ce6)(U, qmmm, qmm, qm, qp, qpp, qppp);
    default: /* cflx5 */
        return SFX(o_cweno5z_v0)(U, qmmm, qmm, qm, qp, qpp, qppp);
    }
}

/* compflux_on_interval, weno.py:349-363 */
void SFX(oracle_compflux)(int method, double *flx, const double *U,
                          const double *q, const int8_t *o, int64_t s,
                          int64_t i0, int64_t i1)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = i0; i < i1; i++) {
        if (o[i] > 4)
            flx[i] = SFX(o_f5)(method, U[i], q[i - 3 * s], q[i - 2 * s],
                               q[i - s], q[i], q[i + s], q[i + 2 * s]) * U[i];
        else if (o[i] > 2)
            flx[i] = SFX(o_f3)(method, U[i], q[i - 2 * s], q[i - s], q[i],
                               q[i + s]) * U[i];
        else if (o[i] > 0)
            flx[i] = SFX(o_f1)(method, U[i], q[i - s], q[i]) * U[i];
        else
            flx[i] = 0;
    }
}

/* vortexforce_on_interval, weno.py:370-384 */
void SFX(oracle_vortexforce)(int method, double *du, const double *V,
                             const double *q, const int8_t *o, int64_t s,
                             int64_t s2, int sign, int64_t i0, int64_t i1)
{
    const double sg = (double)sign;
#pragma omp parallel for schedule(static)
    for (int64_t i = i0; i < i1; i++) {
        if (o[i] > 0) {
            double Vm = 0.25 * (((V[i] + V[i + s]) + V[i - s2]) + V[i + s - s2]);
            double r;
            if (o[i] > 4)
                r = SFX(o_f5)(method, Vm, q[i - 2 * s], q[i - s], q[i],
                              q[i + s], q[i + 2 * s], q[i + 3 * s]);
            else if (o[i] > 2)
                r = SFX(o_f3)(method, Vm, q[i - s], q[i], q[i + s],
                              q[i + 2 * s]);
            else
                r = SFX(o_f1)(method, Vm, q[i], q[i + s]);
            du[i] = sg * r * Vm;
        } else {
            du[i] = 0;
        }
    }
}

/* innerproduct_on_interval, weno.py:391-403 */
void SFX(oracle_innerproduct)(int method, double *ke, const double *U,
                              const double *q, const int8_t *o, int64_t s,
                              int64_t i0, int64_t i1)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = i0; i < i1; i++) {
        if (o[i] > 0) {
            double Um = 0.5 * (U[i] + U[i + s]);
            double r;
            if (o[i] > 4)
                r = SFX(o_f5)(method, Um, q[i - 2 * s], q[i - s], q[i],
                              q[i + s], q[i + 2 * s], q[i + 3 * s]);
            else if (o[i] > 2)
                r = SFX(o_f3)(method, Um, q[i - s], q[i], q[i + s],
                              q[i + 2 * s]);
            else
                r = SFX(o_f1)(method, Um, q[i], q[i + s]);
            ke[i] += r * Um;
        }
    }
}
