/*
 * ORACLE - test infrastructure only. Not part of the product path.
 *
 * Plain-C restatement of the reference's flux reconstructions and flat-index
 * sweep kernels (pvthinker/Fluids2d, src/fluids2d/weno.py) and of its stencil
 * order builder (src/fluids2d/meshes.py:146-186). Only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load this library, and only
 * to check or to time the CUDA path against it.
 *
 * Arithmetic follows the reference expression by expression: the same
 * operation order, IEEE binary64, no FMA contraction (build with
 * -ffp-contract=off). The reference's `x**2` on Python floats is pow(x, 2.0),
 * which differs from x*x in the last bit for about 1 in 1000 arguments; the
 * "_py" entry points use pow so that they reproduce the reference run without
 * numba bit for bit. The entry points without the suffix use x*x, which is
 * what numba compiles `x**2` to, and are the ones timed as the CPU baseline.
 *
 * Methods: 0 = "weno", 1 = "upwind", 2 = "centered", 3 = "cweno"
 * (the `_fluxes` table of weno.py:338-343).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#define F2D_ORACLE_BODY 1

/* ---- first instantiation: square = x*x (numba semantics) ---- */
#define SQ(x) ((x) * (x))
#define SFX(name) name
#include "sweeps_body.h"
#undef SQ
#undef SFX

/* ---- second instantiation: square = pow(x, 2) (Python-float semantics) -- */
#define SQ(x) pow((x), 2.0)
#define SFX(name) name##_py
#include "sweeps_body.h"
#undef SQ
#undef SFX

/*
 * set_order (meshes.py:146-186): stencil order of every flat index from the
 * sums of the mask over 2, 4 and 6 neighbours along `shift` (positive: the
 * stencil leans towards lower indices; negative: towards higher indices),
 * capped at maxorder.
 */
void oracle_set_order(const int8_t *m, int64_t n, int64_t shift, int maxorder,
                      int8_t *o)
{
    for (int64_t i = 0; i < n; i++) {
        long s2, s4, s6;
        if (shift > 0) {
            s2 = (i - shift >= 0) ? (long)m[i - shift] + m[i] : 0;
            s4 = ((i - 2 * shift >= 0) && (i + shift < n))
                     ? (long)m[i - 2 * shift] + m[i + shift] + s2 : 0;
            s6 = ((i - 3 * shift >= 0) && (i + 2 * shift < n))
                     ? (long)m[i - 3 * shift] + m[i + 2 * shift] + s4 : 0;
        } else {
            s2 = (i - shift < n) ? (long)m[i - shift] + m[i] : 0;
            s4 = ((i - 2 * shift < n) && (i + shift >= 0))
                     ? (long)m[i - 2 * shift] + m[i + shift] + s2 : 0;
            s6 = ((i - 3 * shift < n) && (i + 2 * shift >= 0))
                     ? (long)m[i - 3 * shift] + m[i + 2 * shift] + s4 : 0;
        }
        int v = (s6 == 6) ? 6 : ((s4 == 4) ? 4 : ((s2 == 2) ? 2 : 0));
        if (v > maxorder) v = maxorder;
        o[i] = (int8_t)v;
    }
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
