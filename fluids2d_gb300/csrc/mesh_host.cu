// Host-side mesh construction: the reference's derived masks, slip
// coefficients, stencil orders and fluid-point index, computed once per mask
// and packed into per-point code words for the kernels. Integer results are
// identical to the reference's (checked against its outputs in the tests).
#include <cstring>
#include <string>
#include <vector>

#include "mesh_host.h"
#include "weno.cuh"

namespace f2d {

// set_order (meshes.py:146-186): neighbour sums of the flattened mask over
// 2, 4 and 6 points along `shift`; order 6/4/2/0 where all are fluid, capped
// at maxorder. Indices are flat, so x-stencils run across row ends exactly
// as in the reference.
void set_order_host(const int8_t* m, int64_t n, int64_t shift, int maxorder, int8_t* o)
{
    const int64_t s = shift;
    for (int64_t i = 0; i < n; ++i) {
        long a2 = 0, a4 = 0, a6 = 0;
        bool ok2, ok4, ok6;
        if (s > 0) {
            ok2 = i - s >= 0;
            ok4 = (i - 2 * s >= 0) && (i + s < n);
            ok6 = (i - 3 * s >= 0) && (i + 2 * s < n);
        } else {
            ok2 = i - s < n;
            ok4 = (i - 2 * s < n) && (i + s >= 0);
            ok6 = (i - 3 * s < n) && (i + 2 * s >= 0);
        }
        if (ok2) a2 = (long)m[i - s] + m[i];
        if (ok4) a4 = (long)m[i - 2 * s] + m[i + s] + a2;
        if (ok6) a6 = (long)m[i - 3 * s] + m[i + 2 * s] + a4;
        int v = a6 == 6 ? 6 : (a4 == 4 ? 4 : (a2 == 2 ? 2 : 0));
        o[i] = (int8_t)(v < maxorder ? v : maxorder);
    }
}

int mesh_build_host(const f2d_params& p, const int8_t* msk_in, MeshHost& M,
                    std::string& err)
{
    if (p.halowidth != 3) {
        err = "halowidth must be 3";
        return 1;
    }
    if (p.yperiodic) {
        err = "yperiodic is not supported (the reference never fills y halos "
              "and its Poisson operator ignores y periodicity)";
        return 1;
    }
    if (p.nx < 6 || p.ny < 6) {
        err = "nx and ny must be at least 6";
        return 1;
    }
    const int h = 3;
    const int NY = p.ny + 2 * h, NX = p.nx + 2 * h;
    const size_t N = (size_t)NY * NX;
    M.NY = NY;
    M.NX = NX;
    M.msk.assign(N, 0);
    if (msk_in) {
        for (size_t k = 0; k < N; ++k) M.msk[k] = msk_in[k] ? 1 : 0;
    } else {
        // set_default_mask (meshes.py:70-75)
        for (int j = h; j < NY - h; ++j)
            for (int i = 0; i < NX; ++i)
                if (p.xperiodic || (i >= h && i < NX - h)) M.msk[(size_t)j * NX + i] = 1;
    }
    const int8_t* m = M.msk.data();

    // set_masks (meshes.py:77-86)
    M.mskx.assign(N, 0);
    M.msky.assign(N, 0);
    M.mskv.assign(N, 0);
    for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) {
            const size_t k = (size_t)j * NX + i;
            if (i >= 1) M.mskx[k] = m[k] * m[k - 1];
            if (j >= 1) M.msky[k] = m[k] * m[k - NX];
            if (i >= 1 && j >= 1)
                M.mskv[k] = m[k - NX] * m[k - NX - 1] * m[k] * m[k - 1];
        }

    // get_slipcoef (noslip.py:4-36): count of fluid cells around a vertex
    M.slip.assign(N, 0.0);
    std::vector<int> cnt(N, 0);
    for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) {
            const size_t k = (size_t)j * NX + i;
            int c = m[k];
            if (i >= 1) c += m[k - 1];
            if (j >= 1) c += m[k - NX];
            if (i >= 1 && j >= 1) c += m[k - NX - 1];
            cnt[k] = c;
            M.slip[k] = (c == 4) ? 1.0 : 0.0;  // free slip
        }
    auto noslip_at = [&](size_t k) { M.slip[k] = cnt[k] < 1 ? (double)cnt[k] : 1.0; };
    if (p.noslip == F2D_SLIP_NOSLIP) {
        for (size_t k = 0; k < N; ++k) noslip_at(k);
    } else if (p.noslip == F2D_SLIP_SIDES) {
        if (p.noslip_sides & F2D_SIDE_LEFT)
            for (int j = 0; j < NY; ++j) noslip_at((size_t)j * NX + h);
        if (p.noslip_sides & F2D_SIDE_RIGHT)
            for (int j = 0; j < NY; ++j) noslip_at((size_t)j * NX + (NX - h));
        if (p.noslip_sides & F2D_SIDE_BOTTOM)
            for (int i = 0; i < NX; ++i) noslip_at((size_t)h * NX + i);
        if (p.noslip_sides & F2D_SIDE_TOP)
            for (int i = 0; i < NX; ++i) noslip_at((size_t)(NY - h) * NX + i);
    }

    // set_stencils (meshes.py:88-104)
    const int mo = p.maxorder;
    for (int k = 0; k < 6; ++k) M.ord[k].assign(N, 0);
    set_order_host(m, (int64_t)N, 1, mo, M.ord[0].data());    // oc.x
    set_order_host(m, (int64_t)N, NX, mo, M.ord[1].data());   // oc.y
    std::vector<int8_t> mv(N);
    for (size_t k = 0; k < N; ++k) mv[k] = M.slip[k] > 0 ? 1 : 0;
    set_order_host(mv.data(), (int64_t)N, -1, mo, M.ord[2].data());   // ov.x
    set_order_host(mv.data(), (int64_t)N, -NX, mo, M.ord[3].data());  // ov.y
    for (size_t k = 0; k < N; ++k) {
        M.ord[2][k] = (int8_t)(M.ord[2][k] * M.msky[k]);
        M.ord[3][k] = (int8_t)(M.ord[3][k] * M.mskx[k]);
    }
    set_order_host(M.mskx.data(), (int64_t)N, -1, mo, M.ord[4].data());   // ok.x
    set_order_host(M.msky.data(), (int64_t)N, -NX, mo, M.ord[5].data());  // ok.y

    // Poisson2D "v" fluid index (elliptic.py:102-111, 198-203)
    M.gv.assign(N, -1);
    int32_t next = 0;
    for (int j = 0; j < NY; ++j)
        for (int i = 0; i < NX; ++i) {
            const size_t k = (size_t)j * NX + i;
            bool f = M.mskv[k] == 1;
            if (p.xperiodic && (i < h || i >= NX - h)) f = false;
            if (f) M.gv[k] = next++;
        }
    M.nfluid_v = next;

    // packed codes
    M.code.assign(N, 0);
    for (size_t k = 0; k < N; ++k) {
        uint32_t c = 0;
        c |= (uint32_t)order_level(M.ord[0][k]) << SH_OCX;
        c |= (uint32_t)order_level(M.ord[1][k]) << SH_OCY;
        c |= (uint32_t)order_level(M.ord[2][k]) << SH_OVX;
        c |= (uint32_t)order_level(M.ord[3][k]) << SH_OVY;
        c |= (uint32_t)order_level(M.ord[4][k]) << SH_OKX;
        c |= (uint32_t)order_level(M.ord[5][k]) << SH_OKY;
        if (m[k]) c |= B_MSK;
        if (M.mskx[k]) c |= B_MSKX;
        if (M.msky[k]) c |= B_MSKY;
        if (M.mskv[k]) c |= B_MSKV;
        if (M.slip[k] != 0.0) c |= B_SLIP;
        if (M.gv[k] >= 0) c |= B_GV;
        M.code[k] = c;
    }
    return 0;
}

}  // namespace f2d
