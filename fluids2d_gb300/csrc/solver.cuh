// Batched multigrid-preconditioned solver for the masked vertex
// Poisson/Helmholtz operator of one or many models (a single model is a
// batch of one). See solver.cu.
#pragma once
#include <vector>

#include "mg.cuh"

namespace f2d {

constexpr int BS_LMAX = 16;           // levels per member
constexpr int BS_RING = 32;           // inner iterations per refinement round, at most
constexpr int BS_TW = 32;  // node tile: 32 columns x 32 or 64 rows, 32 x 8 threads

struct BSInfo {
    int nl, ltail, ksweeps;  // levels, first tail level, coarsest sweeps
    int n0, nn;              // range of the member in the level-0 tile table
    int pad2;
    // the member's range in the level-0 table of the multigrid level kernels
    // (the tile totals of <r, z> written by the level-0 up leg); mnn = 0 when
    // level 0 is in the member's tail
    int mn0, mnn, pad0, pad1;
};

struct BSGlobals {
    unsigned int ticket[4];
    int active_out, active_in;  // members still iterating (outer / inner)
    int status, pad;
    long long loops_out, loops_in;  // loop iterations (all members together)
};

// Arena base pointers; members are told apart by the offsets inside their
// level-0 descriptors (node (J, I) of member b at off0_b + J*pitch_b + I).
struct BSVecs {
    void* x64;  // solution (FP64, the model's psi)
    void* b64;  // right-hand side (FP64)
    void* r64;  // FP64 residual
    void* p;    // CG direction (FP64 form: double; refinement: float)
    void* p2;   // second CG direction buffer (p alternates between the two)
    void* q;    // A p (same precision as p)
    void* z;    // preconditioned residual, multigrid precision
    void* za;   // level-0 multigrid x after the pre-smoothing (as z)
    void* rin;  // inner residual of the refinement form (float), multigrid rhs
    long long nelem;  // elements of each arena vector (the direction ring's stride)
};

struct BSMemberDesc {
    int nyn, nxn;
    long long pitch, off0;  // level-0 node layout inside the arenas
    int per;
    const uint8_t* hmask;   // host fluid mask, node (J,I) at hoff0 + J*pitch + I
    long long hoff0;
    double cx, cy, maindiag;
    // hmask holds the whole rows of the level-0 arrays (in-row bytes outside
    // the node columns included); when not (a rebuild from the dense level
    // masks), win_ok carries the first build's check of those bytes
    int hwin = 1;
    int win_ok = 0;
};

struct BatchSolver {
    int n = 0;
    int mode = 0;  // 0: FP64 multigrid-PCG; 1: FP32 inner PCG + FP64 refinement
    std::vector<MGHost> mg;
    MGLevel* dlevs = nullptr;
    BSInfo* dinfo = nullptr;
    BSGlobals* eg = nullptr;
    DevScalars* scs = nullptr;  // one per member, owned by the caller
    double* partials = nullptr;
    std::vector<int4*> tiles;  // node tiles per level (members reaching it)
    std::vector<int> ntiles;
    std::vector<int4*> mtiles; // tiles of the multigrid level kernels per level
    std::vector<int> nmtiles;
    double* mpartials = nullptr;  // <r, z> tile totals of the level-0 up leg (per mtiles[0])
    // pipelined FP32 level kernels (mg_pipe.cuh): used when the level arrays
    // pass bs_build's layout checks; TMA maps per member and level, grid sizes
    bool pipe = false;
    void* mmaps = nullptr;     // CUtensorMap[n][BS_LMAX][MP_NMAP]
    int pipe_gdown = 0, pipe_gup = 0;
    int4* rtiles = nullptr;    // level-0 tiles of the Krylov kernels
    int nrtiles = 0;
    int maxl = 0;
    size_t tail_smem = 0;
    int tail_threads = 1024;  // block size of k_bs_tail (bs_build)
    bool helm = false, unit = false;  // FP64 residual variant (bs_build)
    // refinement form: the inner iterations' directions p_0 .. p_{k-1}, one
    // float arena each (p_i at pring + i * nelem), so the round's correction
    // sum alpha_i p_i is formed once, by k_bs_correct, instead of an x
    // update in every iteration; inner iterations are capped at BS_RING
    float* pring = nullptr;
    BSVecs v;
    double tol = 1e-12, tol_in = 1e-6;
    int maxit = 200, maxit_in = 30, maxouter = 20;
    int nu = 2;  // red-black sweeps before and after each coarse correction (1 or 2)
    int th = 32;  // tile rows (32 or 64), chosen by bs_build
    int th_force = 0;  // tile rows set by the autotuner (0: bs_build's rule)
    std::vector<BSMemberDesc> descs;  // as built (host mask pointers stale)
    const uint8_t* dmask = nullptr;
    int body_launches = 0;
    cudaStream_t s3 = nullptr;  // capture stream of the inner loop body (own per solver)
    std::vector<void*> owned;
};

int bs_build(BatchSolver& s, const std::vector<BSMemberDesc>& members,
             const uint8_t* dmask, int mode, const BSVecs& v, DevScalars* scs);
void bs_free(BatchSolver& s);

// Autotuner of the multigrid schedule: tile rows (32, 64) x sweeps per leg
// (1, 2) x, in the FP32 refinement form, inner tolerance (1e-8 .. 1e-4).
// Each candidate's solve is captured as a graph and timed over `reps` solves
// of the current right-hand side b from the warm start 0.999 x* (x* = the
// current solution in x, FP64, xbytes); candidates that stop short of the
// tolerance are discarded. The fastest is applied (the solver rebuilt for
// its tile rows) and x is restored. The caller drops graphs that captured
// the solver before.
struct BSTune {
    int th, nu;
    double tol_in, ms;
    int ncand;
};
int bs_autotune(BatchSolver& s, cudaStream_t st, cudaStream_t st2, void* x, const void* b,
                size_t xbytes, int reps, BSTune* out);
// Set the schedule directly (tile rows 32/64, sweeps per leg 1/2, inner
// tolerance of the refinement form in (0, 1)); rebuilds the tile tables when
// the tile rows change. The caller drops graphs that captured the solver.
int bs_set_schedule(BatchSolver& s, int th, int nu, double tol_in);
// measurement hook: mean ms of the level-0 down kernel over `reps` launches
int bs_time_down(BatchSolver& s, cudaStream_t st, int reps, int flush_l2, double* avg_ms,
                 long long* nodes, int* es);
// Record one solve of every member on `st`: eagerly (host-driven loops, a
// profiling aid) or, under stream capture, as conditional WHILE nodes whose
// bodies are captured on `st2`.
int bs_record(BatchSolver& s, cudaStream_t st, cudaStream_t st2, int* launches);

}  // namespace f2d
