// Stage 3 of PaMO: safe projection of the simplified mesh back onto the source ("GT") mesh — a Newton
// solver over distance-to-GT, StVK membrane, hinge bending and an IPC log-barrier between nearby
// point-triangle and edge-edge pairs, with Jacobi-preconditioned CG, a per-vertex step clamp, additive CCD
// and a backtracking line search (simp_cuda/safe_project/src/pamo_safe_project/system.py:411-470).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "lbvh.cuh"
#include "pamo_common.cuh"

namespace pamo {

// Stage3Config defaults (pamo_safe_project/config.py:6-73)
struct Stage3Params {
    int n_newton_iters = 10;
    int n_cg_iters = 40;
    int n_line_search_iters = 10;
    float d_hat = 1e-3f;
    float coll_stiffness = 1e2f;
    float contact_detection_radius = 1e-2f;
    float ee_classify_thres = 1e-3f;
    float ccd_slackness = 0.7f;
    float ccd_thickness = 1e-6f;
    int ccd_max_iters = 100;
    int ccd_fp64 = 2;  // the precision mode's CCD: 2 double-float (FP32 pipes), 1 float64; 0 float32 as Warp's kernels
    int spd_max_iters = 3;
    float elas_young_modulus = 0.1f;
    float elas_poisson_ratio = 0.0f;
    float hinge_stiffness = 1e-2f;
    float mesh2gt_dist_stiffness = 1e3f;
    float min_angle_thres = 0.0f;  // degrees
    long long max_blocks = 1ll << 25;
};

// Device scalars of the solver. Kernels of a Newton iteration read their sizes and coefficients from here,
// so that one captured CUDA graph serves every iteration of a run.
struct SolverScalars {
    float energy, energy_prev, v_A_v, z_r, z_r_last, ccd_step;
    float radius;         // contact detection radius (halved when contacts exceed max_blocks)
    int barrier_extra;    // test knob: arrivals a grid barrier waits for beyond its grid (0; 1 makes every wait run out)
    int n_contacts, n_contacts_raw, accepted, status;
    int abort;            // 0 running; 1 contact list full, 3 candidate list full (grow, redo the iteration);
                          // 2 contacts above max_blocks (halve the radius, redo)
    int iters_done;       // Newton iterations completed in this run
    int red_count;        // arrival counter of the grid-wide sums
    int max_contacts;
    int rebuild;          // candidate lists are rebuilt in this iteration
    int n_cand_pt, n_cand_ee;  // candidate pairs (true counts, may exceed the capacities)
    int n_cand_all;            // n_cand_pt + n_cand_ee of this iteration's contact filter
    int n_rebuilds;
    long long total_contacts;
};

struct Stage3Stats {
    int n_particles = 0, n_triangles = 0, n_edges = 0, n_hinges = 0;
    int steps = 0, newton_iters = 0, max_contacts = 0, radius_halvings = 0;
    int do_nothing = 0;
    double last_energy = 0.0;
    long long total_contacts = 0;  // summed over Newton iterations
    int candidate_rebuilds = 0;    // Newton iterations that rebuilt the contact candidate lists
    int barrier_reruns = 0;        // 1: a grid barrier gave up and the run was made again without cooperative kernels
};

// The call's unique edges (v * n_points + u, ascending: trimesh's edges_unique order) and hinges, on the host
int stage3_topology(const int* triangles, int n_points, int n_tris, std::vector<long long>& ukeys,
                    std::vector<int4>& hinges);

struct EnergyArgs;  // arguments of the energy kernels (safe_project.cu)

class Stage3 {
public:
    Stage3() = default;
    ~Stage3();
    // Runs process(gt_V, gt_F, V, F, n_iters) on device buffers; out_points receives float64 positions in
    // the input frame. Returns a pamo_status code; err holds the message. A cooperative kernel's grid barrier
    // needs all the kernel's blocks running at once, which other work sharing the GPU from other streams can
    // prevent; when one gives up (its wait is bounded), the run is made again with the PCG as two ordinary launches
    // per iteration and the line search as a launch pair per trial, which give the bits of cg_mode 0 / ls_mode 1.
    int run(const double* gt_points, const int* gt_tris, int n_gt_points, int n_gt_tris, const double* points,
            const int* tris, int n_points, int n_tris, int n_iters, double* out_points, cudaStream_t s);
    Stage3Params params;
    Stage3Stats stats;
    std::string err;
    bool use_graph = true;  // capture one Newton iteration as a CUDA graph and replay it
    int cg_mode = 0;        // PCG kernel: 0/1 grid-wide cooperative, 128 threads; 3: 256 threads; 2: one cluster
    int ls_mode = 1;        // line search: 1 one cooperative launch, 0 a launch pair per trial
    int test_barrier_extra = 0;  // copied to SolverScalars::barrier_extra at each run (tests of the bounded waits)
    int cluster_size = 1;   // CTAs of the cluster kernel (device limit, at most 16)

private:
    int run_once(const double* gt_points, const int* gt_tris, int n_gt_points, int n_gt_tris, const double* points,
                 const int* tris, int n_points, int n_tris, int n_iters, double* out_points, cudaStream_t s);
    bool barrier_gave_up = false;  // the last run_once failed because a grid barrier's bounded wait ran out
    template <typename T>
    int grow(T*& p, size_t& cap, size_t n);
    int dalloc(void** p, size_t bytes);
    void dfree(void* p);
    cudaMemPool_t pool = nullptr;  // the solver's stream-ordered pool for the size-dependent buffers
    int fail(int code, const std::string& m) {
        err = m;
        return code;
    }
    int ensure(int np, int nt, int ne, int nh, int ngp, int ngt);
    int ensure_contacts(size_t n);
    int ensure_candidates(size_t npt, size_t nee);
    int ensure_slots();
    void release();
    void drop_graph();

    // problem sizes
    int NP = 0, NT = 0, NE = 0, NH = 0, NGP = 0, NGT = 0;
    // capacities
    size_t cap_v = 0, cap_t = 0, cap_e = 0, cap_h = 0, cap_gp = 0, cap_gt = 0, cap_c = 0;
    // GT mesh and its LBVH
    float4* gt_pos = nullptr;
    int4* gt_tri = nullptr;
    BvhBuffers gt_bvh{};
    char* gt_bvh_mem = nullptr;
    size_t gt_bvh_cap = 0;
    RoundCounters* gt_rc = nullptr;
    // simulated mesh
    float4 *q = nullptr, *q_rest = nullptr, *q_prev_newton = nullptr, *p = nullptr;
    float4* q_ref = nullptr;  // positions at the last build of the candidate lists
    float4 *target = nullptr, *grad = nullptr, *hdiag = nullptr, *r = nullptr, *z = nullptr;
    float4* v[2] = {nullptr, nullptr};  // CG search directions, ping-pong
    float* vweight = nullptr;  // Voronoi area
    int4* tri = nullptr;
    int4* edge4 = nullptr;     // edges as (u, v, v, 0) for the edge LBVH
    float* el_area = nullptr;
    float4* el_invDm = nullptr;
    int4* hinge = nullptr;
    float2* hinge_rest = nullptr;  // (rest angle, rest edge length)
    float* hinge_blocks = nullptr; // packed symmetric 9x9 Hessian part per hinge (48 floats)
    // contacts
    int4* c_idx = nullptr;
    int2* c_type = nullptr;
    float* c_d = nullptr;
    float4* c_dd = nullptr;    // 4 per contact
    // candidate pairs within the detection reach plus a skin, kept while no vertex moved more than half the
    // skin (point-triangle: (vertex, triangle); edge-edge: (edge, edge))
    int2* cand_pt = nullptr;
    int2* cand_ee = nullptr;
    size_t cap_cpt = 0, cap_cee = 0;
    int* cand_cnt = nullptr;  // per query: candidates of the counting pass (points, then edges)
    int* cand_off = nullptr;  // their exclusive prefix sums (where each query writes)
    size_t cap_cq = 0;
    // the contact filter's per-candidate results (flag, prefix sums = contact index, ids, type)
    int* cflag = nullptr;
    int* cpos = nullptr;
    int4* cid = nullptr;
    int2* cty = nullptr;
    size_t cap_cf = 0;
    // per-vertex sums in a fixed order: the per-corner parts (triangle corners 3f + c, hinge slots 3 NT + 4h + a,
    // contact corners 4b + k) in slot arrays at their positions in their vertex's range (the static ranges first,
    // the contact ranges after cbase = 3 NT + 4 NH), each range summed in order
    std::vector<int> vs_host_off, vs_host_list;  // the static ranges as built on the host
    int* vs_off = nullptr;   // static ranges (triangle corners and hinge slots per vertex), NP + 1 offsets
    int* inv_vs = nullptr;   // 3 NT + 4 NH: the position of each static code in its vertex's range
    size_t cap_vs = 0, cap_vso = 0;
    int* c_cnt = nullptr;    // contact corners per vertex (NP + 1), their offsets and fill cursors
    int* c_off = nullptr;
    int* c_cur = nullptr;
    int* c_tmp = nullptr;    // 4 per contact: the codes filled per vertex, then ranked
    int* c_inv = nullptr;    // 4 per contact: the position of each contact code in its vertex's range
    float4 *gslot = nullptr, *hslot = nullptr, *aslot = nullptr;
    size_t cap_slot = 0;
    int* scan_scratch = nullptr;  // two scan scratches (exclusive_scans with two jobs)
    float2* partial = nullptr;  // block partials of the grid-wide sums
    void* cg_bar = nullptr;     // grid-barrier state of the cooperative CG kernel
    int coop_max_blocks = 1, n_sm = 1;
    int ls_coop_max_blocks = 0;  // co-resident blocks of the cooperative line search
    // LBVHs over the current triangles and edges (built at registration, refitted at every detection)
    BvhBuffers tri_bvh{}, edge_bvh{};
    char *tri_bvh_mem = nullptr, *edge_bvh_mem = nullptr;
    size_t tri_bvh_cap = 0, edge_bvh_cap = 0;
    RoundCounters *tri_rc = nullptr, *edge_rc = nullptr;
    SolverScalars* sc = nullptr;
    SolverScalars* h_sc = nullptr;
    double* d_norm = nullptr;  // [0..2] centre, [3] scale, [4..6] offset t, [16..] per-block partials
    cudaStream_t stream = nullptr;  // private stream the solver runs on (capturable)
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    // captured Newton iteration
    cudaGraphExec_t graph = nullptr;
    long long graph_kernels = 0;
    int graph_key[6] = {0, 0, 0, 0, 0, 0};

    void newton_iteration();  // enqueue one Newton iteration (system.py:425-459)
    void launch_energy(const float4* x, int ls_n = -1);
    EnergyArgs energy_args() const;
    int energy_grid() const;  // blocks of the energy sum (k_energy and the line search)
};

}  // namespace pamo
