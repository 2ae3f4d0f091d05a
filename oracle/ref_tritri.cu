// Harness that evaluates the reference's per-pair self-intersection decision with the reference's own
// code, compiled for the host from simp_cuda/src/bvh (tri_tri_3d.cuh, math.cuh, self_intersect.cuh).
// The steps of the __device__-only lambda in self_intersect.cuh:233-377 (coordinate translation by the
// floored mean, shared-index count, then the calls below) are restated here; is_coplanar,
// detect_shared_edge_coord, isect_tri_tri_v3 and largest_distance are the reference's functions.
//
// Input (stdin, binary): int32 n, then n records of {float cur[9], float qry[9], int32 cur_ids[3],
// int32 qry_ids[3]}. Output (stdout, binary): n int32 decisions (1 = the pair counts as intersecting).
// Built by oracle/build_ref.py into oracle/_ref/; test infrastructure only.
#include <cstdio>
#include <cstdint>
#include <cmath>
#include <vector>
#include "cusimp_free.h"
#include "bvh/self_intersect.cuh"

static int floor_mean_h(float v1, float v2, float v3, float v4, float v5, float v6) {
    float mean = (v1 + v2 + v3 + v4 + v5 + v6) / 6.0f;
    return (int)floorf(mean);
}

static int decide(const float* c, const float* q, const int* ci, const int* qi, float epsilon) {
    float3 p1 = make_float3(c[0], c[1], c[2]), q1 = make_float3(c[3], c[4], c[5]), r1 = make_float3(c[6], c[7], c[8]);
    float3 p2 = make_float3(q[0], q[1], q[2]), q2 = make_float3(q[3], q[4], q[5]), r2 = make_float3(q[6], q[7], q[8]);
    int mx = floor_mean_h(p1.x, q1.x, r1.x, p2.x, q2.x, r2.x);
    int my = floor_mean_h(p1.y, q1.y, r1.y, p2.y, q2.y, r2.y);
    int mz = floor_mean_h(p1.z, q1.z, r1.z, p2.z, q2.z, r2.z);
    float3* pts[6] = {&p1, &q1, &r1, &p2, &q2, &r2};
    for (float3* p : pts) { p->x -= mx; p->y -= my; p->z -= mz; }
    int num_count = 0;
    for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++)
            if (ci[j] == qi[k]) num_count++;
    float tri_a[3][3], tri_b[3][3];
    copy_v3_v3_float_float3(tri_a[0], p1);
    copy_v3_v3_float_float3(tri_a[1], q1);
    copy_v3_v3_float_float3(tri_a[2], r1);
    copy_v3_v3_float_float3(tri_b[0], p2);
    copy_v3_v3_float_float3(tri_b[1], q2);
    copy_v3_v3_float_float3(tri_b[2], r2);
    if (is_coplanar(tri_a, tri_b)) return 0;
    if (num_count == 2) return 0;
    if (selfx::detect_shared_edge_coord(p1, q1, r1, p2, q2, r2)) return 0;
    float r_i1[3], r_i2[3];
    if (!isect_tri_tri_v3(p1, q1, r1, p2, q2, r2, r_i1, r_i2)) return 0;
    float3 source, target;
    copy_v3_v3_float3_float(source, r_i1);
    copy_v3_v3_float3_float(target, r_i2);
    float dist = largest_distance(source, target);
    if (dist < epsilon && num_count == 1) return 0;
    return 1;
}

int main() {
    int32_t n = 0;
    if (fread(&n, 4, 1, stdin) != 1) return 1;
    std::vector<int32_t> out(n);
    for (int i = 0; i < n; ++i) {
        float c[9], q[9];
        int32_t ci[3], qi[3];
        if (fread(c, 4, 9, stdin) != 9 || fread(q, 4, 9, stdin) != 9 || fread(ci, 4, 3, stdin) != 3 ||
            fread(qi, 4, 3, stdin) != 3)
            return 2;
        out[i] = decide(c, q, ci, qi, 1e-3f);
    }
    fwrite(out.data(), 4, n, stdout);
    return 0;
}
