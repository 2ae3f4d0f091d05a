// Float64 oracle of the stage-2 edge cost, the reference for the precision figures of the CUDA path's precision
// modes. Test infrastructure: loaded by tests/ and the precision leg of bench.py only.
//
// For each given edge (u, v) of a mesh it evaluates the reference's cost formula (cusimp_free.cu:337-585) in
// double: face planes with unit normals, vertex quadrics Q = sum p p^T over the incident faces, the mean length of
// the edges the two rings list (the same per-face edge mask as the reference's ring loops), the edge length, the
// skinny term over both rings with the moving vertex at the placement (the reference's operator precedence), the
// quadric error v^T (Qu + Qv) v, and cost = qem / s^2 + len + 5 * qa / ntri * threshold, without clamp or
// quantisation. The placement is the midpoint, or with optimal != 0 the minimiser of v^T (Qu + Qv) v (the adjugate
// solve when the determinant is above 1e-10 of the cube of the largest diagonal entry, else the midpoint). Validity
// (link condition, normal flips) is not decided here: callers compare the edges the GPU found valid.
#include <cmath>
#include <cstdint>
#include <vector>

#include <omp.h>

namespace {

struct D3 {
    double x, y, z;
};
inline D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double dnorm(D3 a) { return std::sqrt(ddot(a, a)); }

}  // namespace

extern "C" int oracle_cost_fp64(const float* points, const int* tris, int n_points, int n_tris, const int* edges,
                                int n_edges, double scale, double tres, int optimal, int threads, double* out_cost,
                                double* out_place) {
    std::vector<D3> P(n_points);
    for (int i = 0; i < n_points; ++i) P[i] = {points[3 * i], points[3 * i + 1], points[3 * i + 2]};
    // vertex -> faces
    std::vector<int> off(n_points + 1, 0), adj(3 * (size_t)n_tris);
    for (int f = 0; f < n_tris; ++f)
        for (int k = 0; k < 3; ++k) {
            const int v = tris[3 * f + k];
            if (v < 0 || v >= n_points) return 1;
            off[v + 1]++;
        }
    for (int v = 0; v < n_points; ++v) off[v + 1] += off[v];
    {
        std::vector<int> cur(off.begin(), off.end() - 1);
        for (int f = 0; f < n_tris; ++f)
            for (int k = 0; k < 3; ++k) adj[cur[tris[3 * f + k]]++] = f;
    }
    // face planes (unit normal, offset) and the quadric of every vertex
    std::vector<double> plane(4 * (size_t)n_tris);
    for (int f = 0; f < n_tris; ++f) {
        const D3 a = P[tris[3 * f]], b = P[tris[3 * f + 1]], c = P[tris[3 * f + 2]];
        D3 n = dcross(dsub(b, a), dsub(c, a));
        const double l = dnorm(n);
        n = {n.x / l, n.y / l, n.z / l};
        plane[4 * f] = n.x;
        plane[4 * f + 1] = n.y;
        plane[4 * f + 2] = n.z;
        plane[4 * f + 3] = -ddot(n, a);
    }
    std::vector<double> Q(10 * (size_t)n_points, 0.0);
    for (int v = 0; v < n_points; ++v) {
        double* q = &Q[10 * (size_t)v];
        for (int s = off[v]; s < off[v + 1]; ++s) {
            const double* p = &plane[4 * (size_t)adj[s]];
            q[0] += p[0] * p[0]; q[1] += p[0] * p[1]; q[2] += p[0] * p[2]; q[3] += p[0] * p[3];
            q[4] += p[1] * p[1]; q[5] += p[1] * p[2]; q[6] += p[1] * p[3];
            q[7] += p[2] * p[2]; q[8] += p[2] * p[3]; q[9] += p[3] * p[3];
        }
    }
    const double k4s3 = 4.0 * std::sqrt(3.0);
    omp_set_num_threads(threads > 0 ? threads : 1);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int e = 0; e < n_edges; ++e) {
        const int u = edges[2 * e], v = edges[2 * e + 1];
        // mean length of the edges the two rings list (an edge i > j of each face, as the reference's loops)
        double len = 0.0;
        int cnt = 0;
        for (int w : {u, v})
            for (int s = off[w]; s < off[w + 1]; ++s) {
                const int* t = &tris[3 * (size_t)adj[s]];
                if (t[0] > t[1]) { len += dnorm(dsub(P[t[0]], P[t[1]])); cnt++; }
                if (t[1] > t[2]) { len += dnorm(dsub(P[t[1]], P[t[2]])); cnt++; }
                if (t[2] > t[0]) { len += dnorm(dsub(P[t[2]], P[t[0]])); cnt++; }
            }
        len = len / cnt / scale * tres + dnorm(dsub(P[u], P[v])) / scale * tres;
        double m[10];
        for (int i = 0; i < 10; ++i) m[i] = Q[10 * (size_t)u + i] + Q[10 * (size_t)v + i];
        D3 x = {(P[u].x + P[v].x) / 2, (P[u].y + P[v].y) / 2, (P[u].z + P[v].z) / 2};
        if (optimal) {
            const double nrm = std::fmax(std::fabs(m[0]), std::fmax(std::fabs(m[4]), std::fabs(m[7])));
            const double c00 = m[4] * m[7] - m[5] * m[5], c01 = m[2] * m[5] - m[1] * m[7], c02 = m[1] * m[5] - m[4] * m[2];
            const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
            if (nrm > 0 && std::fabs(det) > 1e-10 * nrm * nrm * nrm) {
                const double c11 = m[0] * m[7] - m[2] * m[2], c12 = m[1] * m[2] - m[0] * m[5],
                             c22 = m[0] * m[4] - m[1] * m[1];
                x = {-(c00 * m[3] + c01 * m[6] + c02 * m[8]) / det, -(c01 * m[3] + c11 * m[6] + c12 * m[8]) / det,
                     -(c02 * m[3] + c12 * m[6] + c22 * m[8]) / det};
            }
        }
        // skinny term over both rings, the moving vertex at x, faces holding both endpoints skipped
        double qa = 0.0;
        int ntri = 0;
        for (int side = 0; side < 2; ++side) {
            const int w = side ? v : u, other = side ? u : v;
            for (int s = off[w]; s < off[w + 1]; ++s) {
                const int* t = &tris[3 * (size_t)adj[s]];
                if (t[0] == other || t[1] == other || t[2] == other) continue;
                const D3 n0 = t[0] == w ? x : P[t[0]], n1 = t[1] == w ? x : P[t[1]], n2 = t[2] == w ? x : P[t[2]];
                const double l01 = dnorm(dsub(n0, n1)), l12 = dnorm(dsub(n1, n2)), l20 = dnorm(dsub(n2, n0));
                const double sh = (l01 + l12 + l20) / 2;
                const double area = std::sqrt(std::fmax(0.0, sh * (sh - l01) * (sh - l12) * (sh - l20)));
                const double sum = k4s3 * area / (l01 * l01) + l12 * l12 + l20 * l20 + 1e-7;
                qa += 1.0 - std::fmin(std::fmax(sum, 0.0), 1.0);
                ntri++;
            }
        }
        const double vv[4] = {x.x, x.y, x.z, 1.0};
        const int row[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
        double qem = 0.0;
        for (int r = 0; r < 4; ++r) {
            double c = 0.0;
            for (int k = 0; k < 4; ++k) c += m[row[r][k]] * vv[k];
            qem += c * vv[r];
        }
        out_cost[e] = qem / (scale * scale) + len + 5.0 * qa / ntri * tres;
        if (out_place) {
            out_place[3 * (size_t)e] = x.x;
            out_place[3 * (size_t)e + 1] = x.y;
            out_place[3 * (size_t)e + 2] = x.z;
        }
    }
    return 0;
}
