// Host-side mesh construction (mesh_host.cpp).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fluids2d_gb300.h"
#include "common.cuh"

namespace f2d {

struct MeshHost {
    int NY = 0, NX = 0;
    std::vector<int8_t> msk, mskx, msky, mskv;
    std::vector<int8_t> ord[6];  // oc.x, oc.y, ov.x, ov.y, ok.x, ok.y
    std::vector<double> slip;
    std::vector<int32_t> gv;
    std::vector<uint32_t> code;
    int nfluid_v = 0;
};

void set_order_host(const int8_t* m, int64_t n, int64_t shift, int maxorder, int8_t* o);
int mesh_build_host(const f2d_params& p, const int8_t* msk, MeshHost& M, std::string& err);

}  // namespace f2d
