// PaMO stage-2 oracle: a CPU restatement of the reference's parallel QEM edge-collapse round and of the
// PaMO.run round loop (stage 1 and stage 3 off).
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: it is linked by tests/, by __graft_entry__.smoke()
// and by bench.py's CPU-baseline leg. The product library (pamo_gb300/) never loads it.
//
// Reference files followed (paths inside the reference project):
//   simp_cuda/src/cusimp_free.cu   round kernels and CUSimp_Free::forward (:208-1048)
//   simp_cuda/src/cusimp_free.h    Vertex/Mat4x4 arithmetic (:24-182)
//   simp_cuda/src/bvh/self_intersect.cuh  candidate query + tri-tri filter (:25-392)
//   simp_cuda/src/bvh/tri_tri_3d.cuh      is_coplanar / isect_tri_tri_v3_ex (:20-297)
//   simp_cuda/src/bvh/math.cuh            largest_distance (:42-51)
//   simp_cuda/pamo/__init__.py            PaMO.run loop, centring and compaction (:60-72, :95-163)
//   CCCL 3.0.1 thrust/system/detail/generic/shuffle.inl  feistel_bijection + shuffle_copy (third-party,
//                                          used by thrust::shuffle at cusimp_free.cu:937-941)
//
// Determinism: the reference fills the vertex->face lists with atomics, so the order of faces around a
// vertex (and with it the float summation order of quadrics and ring lengths) varies run to run. This
// restatement fixes that order to ascending face index. Every other step follows the reference's
// arithmetic operation for operation (compile with -ffp-contract=off to mirror nvcc --fmad=false).
//
// The reference's LBVH is only a candidate filter: a pair (query f, hit g) reaches the tri-tri test iff
// both faces are live, f != g and their closed AABBs overlap. This restatement enumerates the same
// candidate set with a uniform grid.
//
// Memory the reference reads before writing (fresh cudaMalloc blocks) is modelled as zero-filled.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct P3 {
    float x, y, z;
};
struct F3 {
    int i, j, k;
};

// ---- Vertex<float> arithmetic (cusimp_free.h:31-97) ----
inline P3 vsub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 vadd(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float vdot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 vcross(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float vnorm(P3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline P3 vdiv(P3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }

// min/max/clamp templates of cusimp_free.cu:29-34 (NaN goes to the upper bound)
inline float rmin(float a, float b) { return a < b ? a : b; }
inline float rmax(float a, float b) { return a > b ? a : b; }
inline float rclamp(float x, float a, float b) { return rmin(rmax(a, x), b); }

// float -> uint32 as the GPU converts it (cvt.rzi.u32.f32 saturates)
inline uint32_t f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

inline bool killed(const F3& t) { return t.i == -1 && t.j == -1 && t.k == -1; }

constexpr float COST_RANGE = 10.0f;                 // cusimp_free.cu:15
constexpr float UINT32_MAX_F = 4294967296.0f;       // (float)UINT32_MAX
constexpr int MAX_EXTRA_UNDO_PASSES = 5;            // cusimp_free.cu:1039
constexpr float TRI_EPS = 1e-3f;                    // cusimp_free.cu:893

// ---- 4x4 quadric (cusimp_free.h:114-182) ----
struct Q44 {
    float m[16];
};

inline void plane_of(const P3* pts, F3 t, float p[4]) {  // tri2plane, cusimp_free.cu:337-346
    P3 v0 = pts[t.i], v1 = pts[t.j], v2 = pts[t.k];
    P3 n = vcross(vsub(v1, v0), vsub(v2, v0));
    n = vdiv(n, vnorm(n));
    float off = -vdot(n, v0);
    p[0] = n.x; p[1] = n.y; p[2] = n.z; p[3] = off;
}

inline float vTMv(const Q44& q, const float v[4]) {  // cusimp_free.h:145-152
    float c[4];
    for (int j = 0; j < 4; ++j) c[j] = q.m[0 * 4 + j] * v[0] + q.m[1 * 4 + j] * v[1] + q.m[2 * 4 + j] * v[2] + q.m[3 * 4 + j] * v[3];
    return c[0] * v[0] + c[1] * v[1] + c[2] * v[2] + c[3] * v[3];
}

inline float tri_area(P3 p0, P3 p1, P3 p2) {  // cusimp_free.cu:368-375
    float a = vnorm(vsub(p0, p1));
    float b = vnorm(vsub(p1, p2));
    float c = vnorm(vsub(p2, p0));
    float s = (a + b + c) / 2;
    return std::sqrt(s * (s - a) * (s - b) * (s - c));
}

// is_skinny_triangle, cusimp_free.cu:617-637 (threshold evaluated in double: the literal 1e-6 is double)
inline bool is_skinny(P3 p, P3 q, P3 r) {
    P3 pq = vsub(q, p), pr = vsub(r, p), qr = vsub(r, q);
    float lpq = std::sqrt(vdot(pq, pq));
    float lpr = std::sqrt(vdot(pr, pr));
    float lqr = std::sqrt(vdot(qr, qr));
    float maxl = std::fmax(lpq, std::fmax(lpr, lqr));
    P3 c = {pq.y * pr.z - pq.z * pr.y, pq.z * pr.x - pq.x * pr.z, pq.x * pr.y - pq.y * pr.x};
    float thr = (float)(1e-6 * (double)maxl * (double)maxl);
    float area = 0.5f * std::sqrt(c.x * c.x + c.y * c.y + c.z * c.z);
    return area < thr;
}

inline int next_after(F3 t, int v) {  // edge i-j; j-k; k-i  (cusimp_free.cu:410-417)
    if (t.i == v) return t.j;
    if (t.j == v) return t.k;
    if (t.k == v) return t.i;
    return -1;
}

// ---------------------------------------------------------------------------------------------------
// thrust::shuffle(first, last, default_random_engine()) permutation, restated from the published CCCL
// 3.0.1 algorithm: a 24-round Feistel bijection over [0, 2^bits) keyed by minstd_rand, followed by a
// stable compaction of the keys that fall inside [0, m). out[r] = in[perm[r]].
// ---------------------------------------------------------------------------------------------------
void shuffle_perm(uint64_t m, std::vector<int>& perm) {
    perm.clear();
    if (m == 0) return;
    uint64_t bits;
    if (m <= 16) {
        bits = 4;
    } else {
        bits = 0;
        uint64_t t = m - 1;
        while (t) { ++bits; t >>= 1; }
    }
    const uint64_t lbits = bits / 2, rbits = bits - lbits;
    const uint64_t lmask = (1ull << lbits) - 1, rmask = (1ull << rbits) - 1;
    uint32_t key[24];
    uint64_t x = 1;  // minstd_rand default seed
    for (int r = 0; r < 24; ++r) {
        x = (x * 48271ull) % 2147483647ull;
        key[r] = (uint32_t)x;
    }
    const uint64_t n = 1ull << bits;
    perm.reserve(m);
    for (uint64_t idx = 0; idx < n; ++idx) {
        uint32_t s0 = (uint32_t)(idx >> rbits), s1 = (uint32_t)(idx & rmask);
        for (int r = 0; r < 24; ++r) {
            uint64_t prod = 0xD2B74407B1CE6E93ull * (uint64_t)s0;
            uint32_t hi = (uint32_t)(prod >> 32), lo = (uint32_t)prod;
            lo = (lo << (rbits - lbits)) | (s1 >> lbits);
            s0 = ((hi ^ key[r]) ^ s1) & (uint32_t)lmask;
            s1 = lo & (uint32_t)rmask;
        }
        uint64_t g = ((uint64_t)s0 << rbits) | (uint64_t)s1;
        if (g < m) perm.push_back((int)g);
    }
}

// ---------------------------------------------------------------------------------------------------
// Triangle-triangle test of the reference (self_intersect.cuh:129-149, 229-378; tri_tri_3d.cuh)
// ---------------------------------------------------------------------------------------------------
struct F3f {
    float x, y, z;
};

inline int floor_mean6(float a, float b, float c, float d, float e, float f) {
    float mean = (a + b + c + d + e + f) / 6.0f;
    return (int)std::floor(mean);
}

inline bool same_eps(const float a[3], const float b[3], float eps) {
    return std::fabs(a[0] - b[0]) < eps && std::fabs(a[1] - b[1]) < eps && std::fabs(a[2] - b[2]) < eps;
}

inline bool shared_edge_coord(const float A[3][3], const float B[3][3]) {  // self_intersect.cuh:38-48
    const float eps = 1e-6f;
    int s = 0;
    for (int i = 0; i < 3; ++i) s += (same_eps(A[i], B[0], eps) || same_eps(A[i], B[1], eps) || same_eps(A[i], B[2], eps)) ? 1 : 0;
    return s >= 2;
}

inline void plane_db(const float T[3][3], double pl[4]) {
    double ba[3] = {(double)T[0][0] - (double)T[1][0], (double)T[0][1] - (double)T[1][1], (double)T[0][2] - (double)T[1][2]};
    double bc[3] = {(double)T[2][0] - (double)T[1][0], (double)T[2][1] - (double)T[1][1], (double)T[2][2] - (double)T[1][2]};
    pl[0] = ba[1] * bc[2] - ba[2] * bc[1];
    pl[1] = ba[2] * bc[0] - ba[0] * bc[2];
    pl[2] = ba[0] * bc[1] - ba[1] * bc[0];
    pl[3] = -(pl[0] * (double)T[1][0] + pl[1] * (double)T[1][1] + pl[2] * (double)T[1][2]);
}

inline double dot_dbfl(const double a[3], const float b[3]) { return a[0] * (double)b[0] + a[1] * (double)b[1] + a[2] * (double)b[2]; }

bool coplanar(const float A[3][3], const float B[3][3]) {  // tri_tri_3d.cuh:99-129
    float scale = 0.0f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) scale = std::fmax(scale, std::fabs(A[i][j]));
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) scale = std::fmax(scale, std::fabs(B[i][j]));
    double pa[4];
    plane_db(A, pa);
    double s0 = dot_dbfl(pa, B[0]) + pa[3];
    double s1 = dot_dbfl(pa, B[1]) + pa[3];
    double s2 = dot_dbfl(pa, B[2]) + pa[3];
    double eps = (double)scale * 1e-6;
    return std::fabs(s0) <= eps && std::fabs(s1) <= eps && std::fabs(s2) <= eps;
}

inline void lerp3(float r[3], const float a[3], const float b[3], float t) {
    const float s = 1.0f - t;
    r[0] = s * a[0] + t * b[0];
    r[1] = s * a[1] + t * b[1];
    r[2] = s * a[2] + t * b[2];
}

// isect_tri_tri_v3_ex (tri_tri_3d.cuh:130-276): the segment shared by the two triangles, if any
bool isect_tri_tri(const float A[3][3], const float B[3][3], float r1[3], float r2[3]) {
    struct Range {
        float mn, mx;
        float loc[2][3];
    } range[2];
    float side[2][3];
    double pa[4], pb[4];
    plane_db(A, pa);
    side[1][0] = (float)(dot_dbfl(pa, B[0]) + pa[3]);
    side[1][1] = (float)(dot_dbfl(pa, B[1]) + pa[3]);
    side[1][2] = (float)(dot_dbfl(pa, B[2]) + pa[3]);
    if (side[1][0] == 0.0f && side[1][1] == 0.0f && side[1][2] == 0.0f) return false;
    if ((side[1][0] != 0.0f && side[1][1] != 0.0f && side[1][2] != 0.0f) && (side[1][0] < 0.0f) == (side[1][1] < 0.0f) &&
        (side[1][0] < 0.0f) == (side[1][2] < 0.0f))
        return false;
    plane_db(B, pb);
    side[0][0] = (float)(dot_dbfl(pb, A[0]) + pb[3]);
    side[0][1] = (float)(dot_dbfl(pb, A[1]) + pb[3]);
    side[0][2] = (float)(dot_dbfl(pb, A[2]) + pb[3]);
    if ((side[0][0] != 0.0f && side[0][1] != 0.0f && side[0][2] != 0.0f) && (side[0][0] < 0.0f) == (side[0][1] < 0.0f) &&
        (side[0][0] < 0.0f) == (side[0][2] < 0.0f))
        return false;
    double dir[3] = {pa[1] * pb[2] - pa[2] * pb[1], pa[2] * pb[0] - pa[0] * pb[2], pa[0] * pb[1] - pa[1] * pb[0]};
    for (int i = 0; i < 2; ++i) {
        const float(*T)[3] = (i == 0) ? A : B;
        const float* s = side[i];
        int ti[3];
        if ((s[0] != 0.0f && s[1] != 0.0f) && (s[0] < 0.0f) == (s[1] < 0.0f)) {
            ti[0] = 1; ti[1] = 2; ti[2] = 0;
        } else if ((s[1] != 0.0f && s[2] != 0.0f) && (s[1] < 0.0f) == (s[2] < 0.0f)) {
            ti[0] = 2; ti[1] = 0; ti[2] = 1;
        } else if (s[1] == 0.0f && (s[2] < 0.0f) != (s[0] < 0.0f)) {
            ti[0] = 1; ti[1] = 2; ti[2] = 0;
        } else {
            ti[0] = 0; ti[1] = 1; ti[2] = 2;
        }
        double dot_b = dot_dbfl(dir, T[ti[1]]);
        float sidec = s[ti[1]];
        if (sidec != 0.0f) {
            double dot_a = dot_dbfl(dir, T[ti[0]]);
            double dot_c = dot_dbfl(dir, T[ti[2]]);
            float fac0 = sidec / (sidec - s[ti[0]]);
            float fac1 = sidec / (sidec - s[ti[2]]);
            double off0 = (double)fac0 * (dot_a - dot_b);
            double off1 = (double)fac1 * (dot_c - dot_b);
            if (off0 > off1) {
                std::swap(off0, off1);
                std::swap(fac0, fac1);
                std::swap(ti[0], ti[2]);
            }
            range[i].mn = (float)(dot_b + off0);
            range[i].mx = (float)(dot_b + off1);
            lerp3(range[i].loc[0], T[ti[1]], T[ti[0]], fac0);
            lerp3(range[i].loc[1], T[ti[1]], T[ti[2]], fac1);
        } else {
            range[i].mn = range[i].mx = (float)dot_b;
            std::memcpy(range[i].loc[0], T[ti[1]], sizeof(float) * 3);
            std::memcpy(range[i].loc[1], T[ti[1]], sizeof(float) * 3);
        }
    }
    if ((range[0].mx > range[1].mn) && (range[0].mn < range[1].mx)) {
        if (range[0].mn >= range[1].mn) {
            std::memcpy(r1, range[0].loc[0], sizeof(float) * 3);
            if (range[0].mx <= range[1].mx)
                std::memcpy(r2, range[0].loc[1], sizeof(float) * 3);
            else
                std::memcpy(r2, range[1].loc[1], sizeof(float) * 3);
        } else {
            if (range[0].mx <= range[1].mx) {
                std::memcpy(r1, range[0].loc[1], sizeof(float) * 3);
                std::memcpy(r2, range[1].loc[0], sizeof(float) * 3);
            } else {
                std::memcpy(r1, range[1].loc[0], sizeof(float) * 3);
                std::memcpy(r2, range[1].loc[1], sizeof(float) * 3);
            }
        }
        return true;
    }
    return false;
}

// The per-pair decision of the reference's tri-tri lambda (self_intersect.cuh:233-377):
// "current" is the BVH hit, "query" the face that issued the query.
bool pair_intersects(const P3* pts, F3 cur, F3 qry, float eps) {
    float A[3][3] = {{pts[cur.i].x, pts[cur.i].y, pts[cur.i].z}, {pts[cur.j].x, pts[cur.j].y, pts[cur.j].z}, {pts[cur.k].x, pts[cur.k].y, pts[cur.k].z}};
    float B[3][3] = {{pts[qry.i].x, pts[qry.i].y, pts[qry.i].z}, {pts[qry.j].x, pts[qry.j].y, pts[qry.j].z}, {pts[qry.k].x, pts[qry.k].y, pts[qry.k].z}};
    int mx = floor_mean6(A[0][0], A[1][0], A[2][0], B[0][0], B[1][0], B[2][0]);
    int my = floor_mean6(A[0][1], A[1][1], A[2][1], B[0][1], B[1][1], B[2][1]);
    int mz = floor_mean6(A[0][2], A[1][2], A[2][2], B[0][2], B[1][2], B[2][2]);
    for (int v = 0; v < 3; ++v) {
        A[v][0] -= mx; A[v][1] -= my; A[v][2] -= mz;
        B[v][0] -= mx; B[v][1] -= my; B[v][2] -= mz;
    }
    int vc[3] = {cur.i, cur.j, cur.k}, vq[3] = {qry.i, qry.j, qry.k};
    int shared = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) shared += (vc[a] == vq[b]);
    if (coplanar(A, B)) return false;  // the coplanar branch returns before testing (Q5)
    if (shared == 2) return false;
    if (shared_edge_coord(A, B)) return false;
    float r1[3], r2[3];
    if (!isect_tri_tri(A, B, r1, r2)) return false;
    float dx = std::fabs(r2[0] - r1[0]), dy = std::fabs(r2[1] - r1[1]), dz = std::fabs(r2[2] - r1[2]);
    float d = -std::numeric_limits<float>::infinity();
    if (dx > d) d = dx;
    if (dy > d) d = dy;
    if (dz > d) d = dz;
    if (d < eps && shared == 1) return false;
    return true;
}

// ---------------------------------------------------------------------------------------------------
// Uniform-grid enumeration of AABB-overlapping live face pairs
// ---------------------------------------------------------------------------------------------------
struct Box {
    float lo[3], hi[3];
};

inline Box box_of(const P3* pts, F3 t) {
    P3 a = pts[t.i], b = pts[t.j], c = pts[t.k];
    Box bx;
    bx.lo[0] = std::fmin(a.x, std::fmin(b.x, c.x));
    bx.lo[1] = std::fmin(a.y, std::fmin(b.y, c.y));
    bx.lo[2] = std::fmin(a.z, std::fmin(b.z, c.z));
    bx.hi[0] = std::fmax(a.x, std::fmax(b.x, c.x));
    bx.hi[1] = std::fmax(a.y, std::fmax(b.y, c.y));
    bx.hi[2] = std::fmax(a.z, std::fmax(b.z, c.z));
    return bx;
}

inline bool overlap(const Box& a, const Box& b) {  // aabb.cuh:154-162
    for (int d = 0; d < 3; ++d)
        if (a.hi[d] < b.lo[d] || b.hi[d] < a.lo[d]) return false;
    return true;
}

struct Grid {
    float org[3];
    float cell;
    int dim[3];
    std::vector<int> start, items;
    int cell_coord(float v, int d) const {
        int c = (int)std::floor((v - org[d]) / cell);
        return c < 0 ? 0 : (c >= dim[d] ? dim[d] - 1 : c);
    }
    void build(const std::vector<Box>& boxes, const std::vector<int>& ids) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        std::vector<float> ext;
        ext.reserve(ids.size());
        for (int f : ids) {
            const Box& b = boxes[f];
            float e = 0;
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], (double)b.lo[d]);
                hi[d] = std::max(hi[d], (double)b.hi[d]);
                e = std::max(e, b.hi[d] - b.lo[d]);
            }
            ext.push_back(e);
        }
        if (ids.empty()) {
            for (int d = 0; d < 3; ++d) { org[d] = 0; dim[d] = 1; }
            cell = 1;
            start.assign(2, 0);
            items.clear();
            return;
        }
        std::nth_element(ext.begin(), ext.begin() + ext.size() / 2, ext.end());
        double c = std::max((double)ext[ext.size() / 2] * 2.0, 1e-12);
        double span = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
        c = std::max(c, span / 256.0);
        cell = (float)c;
        for (int d = 0; d < 3; ++d) {
            org[d] = (float)lo[d];
            dim[d] = std::max(1, std::min(1024, (int)std::ceil((hi[d] - lo[d]) / c) + 1));
        }
        size_t ncell = (size_t)dim[0] * dim[1] * dim[2];
        start.assign(ncell + 1, 0);
        for (int f : ids) {
            const Box& b = boxes[f];
            int a0 = cell_coord(b.lo[0], 0), a1 = cell_coord(b.hi[0], 0);
            int b0 = cell_coord(b.lo[1], 1), b1 = cell_coord(b.hi[1], 1);
            int c0 = cell_coord(b.lo[2], 2), c1 = cell_coord(b.hi[2], 2);
            for (int x = a0; x <= a1; ++x)
                for (int y = b0; y <= b1; ++y)
                    for (int z = c0; z <= c1; ++z) start[((size_t)x * dim[1] + y) * dim[2] + z + 1]++;
        }
        for (size_t i = 0; i < ncell; ++i) start[i + 1] += start[i];
        items.assign(start[ncell], 0);
        std::vector<int> cur(start.begin(), start.end() - 1);
        for (int f : ids) {
            const Box& b = boxes[f];
            int a0 = cell_coord(b.lo[0], 0), a1 = cell_coord(b.hi[0], 0);
            int b0 = cell_coord(b.lo[1], 1), b1 = cell_coord(b.hi[1], 1);
            int c0 = cell_coord(b.lo[2], 2), c1 = cell_coord(b.hi[2], 2);
            for (int x = a0; x <= a1; ++x)
                for (int y = b0; y <= b1; ++y)
                    for (int z = c0; z <= c1; ++z) items[cur[((size_t)x * dim[1] + y) * dim[2] + z]++] = f;
        }
    }
};

// ---------------------------------------------------------------------------------------------------
// The oracle context: the reference's CUSimp_Free state that survives between forward() calls
// ---------------------------------------------------------------------------------------------------
struct Oracle {
    int threads = 1;
    // grow-only capacities (cusimp_free.cu:36-206: new size = n + n/5, buffers hold size+1 entries)
    size_t cap_pts = 0, cap_edge_cost = 0;
    std::vector<uint32_t> edge_cost;   // survives between calls (stale reads, Q1)
    std::vector<uint8_t> invalid_tab;  // vertices_invalid_table (Q2)
    std::vector<int> pts_map;          // previous call's compaction map (Q3)
    std::vector<int> undo_list;        // vertices_undo_list, its tail survives between calls
    std::vector<int> tmp_undo;         // tmp_vertices_undo_list

    // working arrays of the current call
    std::vector<P3> points, orig_points;
    std::vector<F3> tris, orig_tris;
    std::vector<int> occ;
    std::vector<int> nt_off, nt;  // vertex -> incident faces (CSR, ascending face index)
    std::vector<int> eu, ev;      // edges
    std::vector<Q44> vq;
    std::vector<uint64_t> tri_min;
    std::vector<int> collapsed;   // collapsed edge list (regular winners in ascending edge order, then line collapses)
    std::vector<uint8_t> face_hit;

    // results / diagnostics of the last call
    int n_pts = 0, n_tris = 0, n_edges = 0, n_vertices_undo = 0;
    int n_collapsed_regular = 0, n_collapsed_total = 0, n_considered = 0;
    int n_undo_passes = 0;  // self-intersection checks run (1 + extra passes)
    long long n_intersect_first = 0;
    std::vector<int> undo_per_pass;
    int status = 0;

    // bounded accessors for the undo lists: the reference writes past their capacity in extreme cases,
    // this restatement records a capacity status instead
    void put(std::vector<int>& a, long long i, int x) {
        if (i >= 0 && (size_t)i < a.size()) a[i] = x;
        else status = 3;
    }
    int get(const std::vector<int>& a, long long i) const { return (i >= 0 && (size_t)i < a.size()) ? a[i] : 0; }
    int mapped(int x) const { return (x >= 0 && (size_t)x < pts_map.size()) ? pts_map[x] : 0; }

    void ensure_pts(size_t n) {
        if (n > cap_pts) {
            cap_pts = n + n / 5;
            invalid_tab.assign(cap_pts + 1, 0);
            pts_map.assign(cap_pts + 1, 0);
            undo_list.assign(cap_pts + 1, 0);
            tmp_undo.assign(cap_pts + 1, 0);
        }
    }
    void ensure_edge_cost(size_t n) {
        if (n > cap_edge_cost) {
            cap_edge_cost = n + n / 5;
            edge_cost.assign(cap_edge_cost + 1, 0u);
        }
    }

    // ---- kernels ----
    void build_csr() {
        nt_off.assign(n_pts + 1, 0);
        for (int f = 0; f < n_tris; ++f) {
            const F3& t = tris[f];
            if (killed(t)) continue;
            nt_off[t.i + 1]++; nt_off[t.j + 1]++; nt_off[t.k + 1]++;
        }
        for (int v = 0; v < n_pts; ++v) nt_off[v + 1] += nt_off[v];
        nt.assign(nt_off[n_pts], 0);
        std::vector<int> cur(nt_off.begin(), nt_off.end() - 1);
        for (int f = 0; f < n_tris; ++f) {
            const F3& t = tris[f];
            if (killed(t)) continue;
            nt[cur[t.i]++] = f; nt[cur[t.j]++] = f; nt[cur[t.k]++] = f;
        }
    }

    void build_edges() {  // count_edge_kernel / create_edge_kernel, cusimp_free.cu:306-335
        eu.clear(); ev.clear();
        for (int f = 0; f < n_tris; ++f) {
            const F3& t = tris[f];
            if (killed(t)) continue;
            if (t.i > t.j) { eu.push_back(t.j); ev.push_back(t.i); }
            if (t.j > t.k) { eu.push_back(t.k); ev.push_back(t.j); }
            if (t.k > t.i) { eu.push_back(t.i); ev.push_back(t.k); }
        }
        n_edges = (int)eu.size();
    }

    void compute_quadrics() {  // compute_vert_Q_kernel, cusimp_free.cu:348-366
        vq.assign(n_pts, Q44{});
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int v = 0; v < n_pts; ++v) {
            Q44 K;
            for (int a = 0; a < 16; ++a) K.m[a] = 0.0f;
            for (int s = nt_off[v]; s < nt_off[v + 1]; ++s) {
                float p[4];
                plane_of(points.data(), tris[nt[s]], p);
                for (int r = 0; r < 4; ++r)
                    for (int c = 0; c < 4; ++c) K.m[r * 4 + c] += p[r] * p[c];
            }
            vq[v] = K;
        }
    }

    // ring edge-length accumulation of compute_edge_cost_kernel (cusimp_free.cu:449-484)
    inline void ring_len(int w, float& len, int& cnt) const {
        for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) {
            const F3& t = tris[nt[s]];
            if (t.i > t.j) { len += vnorm(vsub(points[t.i], points[t.j])); cnt++; }
            if (t.j > t.k) { len += vnorm(vsub(points[t.j], points[t.k])); cnt++; }
            if (t.k > t.i) { len += vnorm(vsub(points[t.k], points[t.i])); cnt++; }
        }
    }

    // normal-flip test and skinny term over the ring of w, with w moved to vm, skipping faces that
    // contain `other` (cusimp_free.cu:497-575). Returns false when a normal flips. The reference squares the
    // lengths with the device's pow(float, int); this restatement multiplies (the device function differs from
    // x * x by one ulp for a few floats in a million, which the GPU tests find to change no result). legacy: the
    // legacy round's sum runs in double (cusimp.cu:423,463: `4.0f * sqrt(3)` takes the integer overload).
    inline bool ring_skinny(int w, int other, P3 vm, float& qa, int& ntri, bool legacy = false) const {
        const float k4s3 = 4.0f * std::sqrt(3.0f);
        for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) {
            const F3& t = tris[nt[s]];
            if (t.i == other || t.j == other || t.k == other) continue;
            P3 o0 = points[t.i], o1 = points[t.j], o2 = points[t.k];
            P3 n0 = o0, n1 = o1, n2 = o2;
            if (t.i == w) n0 = vm;
            if (t.j == w) n1 = vm;
            if (t.k == w) n2 = vm;
            P3 on = vcross(vsub(o1, o0), vsub(o2, o0));
            on = vdiv(on, vnorm(on));
            P3 nn = vcross(vsub(n1, n0), vsub(n2, n0));
            nn = vdiv(nn, vnorm(nn));
            if (vdot(on, nn) < 0) return false;
            float l01 = vnorm(vsub(n0, n1)), l12 = vnorm(vsub(n1, n2)), l20 = vnorm(vsub(n2, n0));
            // operator precedence of the reference (Q4): only the first squared length divides
            float e;
            if (legacy)
                e = (float)((double)4.0f * std::sqrt(3.0) * (double)tri_area(n0, n1, n2) / (double)(l01 * l01) +
                            (double)(l12 * l12) + (double)(l20 * l20) + (double)0.0000001f);
            else
                e = k4s3 * tri_area(n0, n1, n2) / (l01 * l01) + l12 * l12 + l20 * l20 + 0.0000001f;
            qa += 1.0f - rclamp(e, 0.0f, 1.0f);
            ntri++;
        }
        return true;
    }

    uint32_t edge_cost_of(int e, float scale, float tres, bool& write) const {
        const int u = eu[e], v = ev[e];
        write = true;
        if (invalid_tab[u] && invalid_tab[v]) return 0xFFFFFFFFu;
        // link condition (cusimp_free.cu:405-444)
        int dup = 0;
        for (int a = nt_off[u]; a < nt_off[u + 1]; ++a) {
            int iu = next_after(tris[nt[a]], u);
            for (int b = nt_off[v]; b < nt_off[v + 1]; ++b) {
                int iv = next_after(tris[nt[b]], v);
                if (iu == iv) dup++;
                if (dup > 2) return 0xFFFFFFFFu;
            }
        }
        if (dup != 2) { write = false; return 0; }
        float len = 0.0f;
        int cnt = 0;
        ring_len(u, len, cnt);
        ring_len(v, len, cnt);
        P3 v0 = points[u], v1 = points[v];
        len = len / (float)cnt / scale * tres;
        len = len + vnorm(vsub(v0, v1)) / scale * tres;
        P3 vm = vdiv(vadd(v0, v1), 2.0f);
        float qa = 0.0f;
        int ntri = 0;
        if (!ring_skinny(u, v, vm, qa, ntri)) return 0xFFFFFFFFu;
        if (!ring_skinny(v, u, vm, qa, ntri)) return 0xFFFFFFFFu;
        qa = 5.0f * qa;  // SKINNY_TRIANGLE_PENALTY
        Q44 Q;
        for (int a = 0; a < 16; ++a) Q.m[a] = vq[u].m[a] + vq[v].m[a];
        float v4[4] = {vm.x, vm.y, vm.z, 1.0f};
        float cost = vTMv(Q, v4) / (scale * scale);
        float tot = cost + len + qa / (float)ntri * tres;
        return f2u_sat(rclamp(tot, 0.0f, COST_RANGE) / COST_RANGE * UINT32_MAX_F);
    }

    // compute_edge_cost_kernel of the legacy CUSimp (cusimp.cu:270-471): the same link condition, rings and
    // flip test; `edge_len += edge_len + |e|/s*t` counts the mean ring length twice; no skinny penalty factor;
    // no invalid table
    uint32_t edge_cost_legacy(int e, float scale, float tres, bool& write) const {
        const int u = eu[e], v = ev[e];
        write = true;
        int dup = 0;
        for (int a = nt_off[u]; a < nt_off[u + 1]; ++a) {
            int iu = next_after(tris[nt[a]], u);
            for (int b = nt_off[v]; b < nt_off[v + 1]; ++b) {
                int iv = next_after(tris[nt[b]], v);
                if (iu == iv) dup++;
                if (dup > 2) return 0xFFFFFFFFu;
            }
        }
        if (dup != 2) { write = false; return 0; }
        float len = 0.0f;
        int cnt = 0;
        ring_len(u, len, cnt);
        ring_len(v, len, cnt);
        P3 v0 = points[u], v1 = points[v];
        len = len / (float)cnt / scale * tres;
        len += len + vnorm(vsub(v0, v1)) / scale * tres;
        P3 vm = vdiv(vadd(v0, v1), 2.0f);
        float qa = 0.0f;
        int ntri = 0;
        if (!ring_skinny(u, v, vm, qa, ntri, true)) return 0xFFFFFFFFu;
        if (!ring_skinny(v, u, vm, qa, ntri, true)) return 0xFFFFFFFFu;
        Q44 Q;
        for (int a = 0; a < 16; ++a) Q.m[a] = vq[u].m[a] + vq[v].m[a];
        float v4[4] = {vm.x, vm.y, vm.z, 1.0f};
        float cost = vTMv(Q, v4) / (scale * scale);
        float tot = cost + len + qa / (float)ntri * tres;
        return f2u_sat(rclamp(tot, 0.0f, COST_RANGE) / COST_RANGE * UINT32_MAX_F);
    }

    void compute_costs(float scale, float tres, bool is_stuck) {  // cusimp_free.cu:382-585
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads)
        for (int e = 0; e < n_edges; ++e) {
            const int u = eu[e], v = ev[e];
            if (invalid_tab[u] && invalid_tab[v]) { edge_cost[e] = 0xFFFFFFFFu; continue; }
            if (is_stuck) continue;
            bool write;
            uint32_t c = edge_cost_of(e, scale, tres, write);
            if (write) edge_cost[e] = c;
        }
    }

    void propagate() {  // propagate_edge_cost_kernel, cusimp_free.cu:587-610
        tri_min.assign(n_tris, ~0ull);
        for (int e = 0; e < n_edges; ++e) {
            uint64_t key = ((uint64_t)edge_cost[e] << 32) | (uint32_t)e;
            for (int w : {eu[e], ev[e]})
                for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) tri_min[nt[s]] = std::min(tri_min[nt[s]], key);
        }
    }

    void restore_ring(int w) {
        for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) tris[nt[s]] = orig_tris[nt[s]];
    }

    // kill the faces around u that contain v; rewire v -> u around v (cusimp_free.cu:691-715, 249-273)
    void rewire(int u, int v) {
        for (int s = nt_off[u]; s < nt_off[u + 1]; ++s) {
            F3& t = tris[nt[s]];
            if (t.i == v || t.j == v || t.k == v) t = {-1, -1, -1};
        }
        for (int s = nt_off[v]; s < nt_off[v + 1]; ++s) {
            F3& t = tris[nt[s]];
            if (t.i == u || t.j == u || t.k == u)
                t = {-1, -1, -1};
            else if (t.i == v)
                t.i = u;
            else if (t.j == v)
                t.j = u;
            else if (t.k == v)
                t.k = u;
        }
    }

    bool ring_has_skinny(int w) const {
        for (int s = nt_off[w]; s < nt_off[w + 1]; ++s) {
            const F3& t = tris[nt[s]];
            if (t.i == -1) continue;
            if (is_skinny(points[t.i], points[t.j], points[t.k])) return true;
        }
        return false;
    }

    void collapse(uint32_t collapse_t, bool restore = true) {  // collapse_edge_kernel, cusimp_free.cu:639-774
        std::vector<uint8_t> win(n_edges, 0);
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads)
        for (int e = 0; e < n_edges; ++e) {
            if (edge_cost[e] > collapse_t) continue;
            uint64_t key = ((uint64_t)edge_cost[e] << 32) | (uint32_t)e;
            bool ok = true;
            for (int w : {eu[e], ev[e]}) {
                for (int s = nt_off[w]; s < nt_off[w + 1] && ok; ++s)
                    if (tri_min[nt[s]] != key) ok = false;
            }
            win[e] = ok;
        }
        collapsed.clear();
        for (int e = 0; e < n_edges; ++e)
            if (win[e]) collapsed.push_back(e);
        n_collapsed_regular = (int)collapsed.size();
        // winners own disjoint face rings, so their updates commute
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
        for (int c = 0; c < n_collapsed_regular; ++c) {
            const int e = collapsed[c], u = eu[e], v = ev[e];
            P3 v0 = points[u], v1 = points[v];
            points[u] = vdiv(vadd(v0, v1), 2.0f);
            points[v] = {0, 0, 0};
            occ[v] = 0;
            rewire(u, v);
            if (!restore) continue;  // the legacy collapse (cusimp.cu:512-585) keeps every winner
            bool sk = ring_has_skinny(u);
            if (!sk) sk = ring_has_skinny(v);
            if (sk) {
                occ[v] = 1;
                points[u] = orig_points[u];
                points[v] = orig_points[v];
                restore_ring(u);
                restore_ring(v);
            }
        }
    }

    void remove_invalid_faces() {  // cusimp_free.cu:218-232
        for (int f = 0; f < n_tris; ++f) {
            F3& t = tris[f];
            if (killed(t)) continue;
            if (t.i == t.j || t.j == t.k || t.k == t.i) t = {-1, -1, -1};
        }
    }

    void remove_line_edges() {  // remove_line_edge_collapse, cusimp_free.cu:234-274 (applied in edge order)
        for (int e = 0; e < n_edges; ++e) {
            const int u = eu[e], v = ev[e];
            P3 p = points[u], q = points[v];
            if (!(p.x == q.x && p.y == q.y && p.z == q.z)) continue;
            collapsed.push_back(e);
            points[v] = {0, 0, 0};
            occ[v] = 0;
            rewire(u, v);
        }
        n_collapsed_total = (int)collapsed.size();
    }

    // self_intersect(): flags every live face that takes part in an intersecting (query, hit) pair
    long long self_intersect() {
        std::vector<Box> boxes(n_tris);
        std::vector<int> live;
        live.reserve(n_tris);
        for (int f = 0; f < n_tris; ++f)
            if (tris[f].i != -1) {
                boxes[f] = box_of(points.data(), tris[f]);
                live.push_back(f);
            }
        Grid g;
        g.build(boxes, live);
        face_hit.assign(n_tris, 0);
        long long hits = 0;
        const int nl = (int)live.size();
#pragma omp parallel num_threads(threads) reduction(+ : hits)
        {
            std::vector<int> stamp(n_tris, -1);
#pragma omp for schedule(dynamic, 256)
            for (int li = 0; li < nl; ++li) {
                const int f = live[li];
                const Box& b = boxes[f];
                int a0 = g.cell_coord(b.lo[0], 0), a1 = g.cell_coord(b.hi[0], 0);
                int b0 = g.cell_coord(b.lo[1], 1), b1 = g.cell_coord(b.hi[1], 1);
                int c0 = g.cell_coord(b.lo[2], 2), c1 = g.cell_coord(b.hi[2], 2);
                for (int x = a0; x <= a1; ++x)
                    for (int y = b0; y <= b1; ++y)
                        for (int z = c0; z <= c1; ++z) {
                            size_t cidx = ((size_t)x * g.dim[1] + y) * g.dim[2] + z;
                            for (int s = g.start[cidx]; s < g.start[cidx + 1]; ++s) {
                                int h = g.items[s];
                                if (h == f || stamp[h] == f) continue;
                                stamp[h] = f;
                                if (!overlap(b, boxes[h])) continue;
                                if (pair_intersects(points.data(), tris[h], tris[f], TRI_EPS)) {
                                    hits++;
                                    face_hit[f] = 1;  // both indices of the pair land in the list
                                    face_hit[h] = 1;
                                }
                            }
                        }
            }
        }
        return hits;
    }

    // get_undo_candidate_kernel, cusimp_free.cu:776-827
    int undo_candidates(std::vector<int>& undo_edges) {
        undo_edges.clear();
        for (int c = 0; c < n_considered; ++c) {
            const int e = collapsed[c];
            bool hit = false;
            for (int w : {eu[e], ev[e]}) {
                for (int s = nt_off[w]; s < nt_off[w + 1] && !hit; ++s)
                    if (face_hit[nt[s]]) hit = true;
                if (hit) break;
            }
            if (hit) undo_edges.push_back(e);
        }
        return (int)undo_edges.size();
    }

    void undo(const std::vector<int>& undo_edges) {  // undo_collapse_kernel, cusimp_free.cu:829-867
        for (int e : undo_edges) {
            const int u = eu[e], v = ev[e];
            occ[v] = 1;
            points[u] = orig_points[u];
            points[v] = orig_points[v];
            restore_ring(u);
            restore_ring(v);
        }
    }

    // CUSimp::forward (cusimp.cu:587-720): one legacy round, no rollback; the compaction map over nP + 1 entries
    int forward_legacy(const float* pts, const int* tris_in, int nP, int nT, float scale, float threshold, bool init) {
        status = 0;
        n_vertices_undo = 0;
        const float tres = threshold;
        const uint32_t collapse_t = f2u_sat(rclamp(threshold, 0.0f, COST_RANGE) / COST_RANGE * UINT32_MAX_F);
        n_pts = nP;
        n_tris = nT;
        ensure_pts(nP);
        points.assign((const P3*)pts, (const P3*)pts + nP);
        occ.assign(nP + 1, 1);
        occ[nP] = 0;
        tris.assign((const F3*)tris_in, (const F3*)tris_in + nT);
        if (init) {
            std::vector<int> perm;
            shuffle_perm((uint64_t)nT, perm);
            std::vector<F3> t2(nT);
            for (int r = 0; r < nT; ++r) t2[r] = tris[perm[r]];
            tris.swap(t2);
        }
        orig_points = points;
        orig_tris = tris;
        build_csr();
        build_edges();
        compute_quadrics();
        ensure_edge_cost(n_edges);
#pragma omp parallel for schedule(dynamic, 1024) num_threads(threads)
        for (int e = 0; e < n_edges; ++e) {
            bool write;
            uint32_t c = edge_cost_legacy(e, scale, tres, write);
            if (write) edge_cost[e] = c;
        }
        propagate();
        collapse(collapse_t, false);
        n_collapsed_total = n_collapsed_regular;
        n_considered = 0;
        n_undo_passes = 0;
        int acc = 0;
        for (int v = 0; v <= nP; ++v) {
            pts_map[v] = acc;
            acc += occ[v];
        }
        return status;
    }

    int forward(const float* pts, const int* tris_in, const int* verts_undo, int nU, int nP, int nT, float scale,
                float threshold, bool is_stuck, bool init) {
        status = 0;
        // undo-list bookkeeping (cusimp_free.cu:895-918); pts_map still holds the previous call's map
        n_vertices_undo = 0;
        int first = 0;
        if (is_stuck) {
            for (int a = 0; a < nU; ++a) put(tmp_undo, a, verts_undo[a]);
            n_vertices_undo = nU;
            for (int a = 0; a < nU; ++a) put(undo_list, a, mapped(get(tmp_undo, a)));
            first = nU;
        } else if (nU != 0) {
            std::fill(invalid_tab.begin(), invalid_tab.end(), 0);
        }
        for (int a = 0; a < nU; ++a) {
            int x = verts_undo[a];
            if (x >= 0 && (size_t)x < invalid_tab.size()) invalid_tab[x] = 1;
        }
        const float tres = threshold;
        const uint32_t collapse_t = f2u_sat(rclamp(threshold, 0.0f, COST_RANGE) / COST_RANGE * UINT32_MAX_F);

        n_pts = nP;
        n_tris = nT;
        ensure_pts(nP);
        points.assign((const P3*)pts, (const P3*)pts + nP);
        occ.assign(nP + 1, 1);
        occ[nP] = 0;
        tris.assign((const F3*)tris_in, (const F3*)tris_in + nT);
        if (init) {
            std::vector<int> perm;
            shuffle_perm((uint64_t)nT, perm);
            std::vector<F3> t2(nT);
            for (int r = 0; r < nT; ++r) t2[r] = tris[perm[r]];
            tris.swap(t2);
        }
        orig_points = points;
        orig_tris = tris;

        build_csr();
        build_edges();
        compute_quadrics();
        ensure_edge_cost(n_edges);
        compute_costs(scale, tres, is_stuck);
        propagate();
        collapse(collapse_t);
        const int h = n_collapsed_regular;
        remove_invalid_faces();
        remove_line_edges();
        // the reference sizes the undo-candidate grid from the regular count only (cusimp_free.cu:1016)
        n_considered = (h == 0) ? 0 : std::min(n_collapsed_total, ((h + 511) / 512) * 512);

        undo_per_pass.clear();
        std::vector<int> ue;
        n_intersect_first = self_intersect();
        n_undo_passes = 1;
        int nue = undo_candidates(ue);
        undo_per_pass.push_back(nue);
        n_vertices_undo += 2 * nue;
        int pass = 0;
        while (nue != 0) {
            ++pass;
            undo(ue);
            // rearrange_index_of_undo_vertices maps through the previous call's pts_map (Q3)
            for (int a = 0; a < nue; ++a) {
                put(tmp_undo, 2 * a, eu[ue[a]]);
                put(tmp_undo, 2 * a + 1, ev[ue[a]]);
            }
            for (int a = 0; a < n_vertices_undo - first; ++a) put(undo_list, first + a, mapped(get(tmp_undo, a)));
            first += 2 * nue;
            self_intersect();
            ++n_undo_passes;
            nue = undo_candidates(ue);
            undo_per_pass.push_back(nue);
            n_vertices_undo += 2 * nue;
            if (pass == MAX_EXTRA_UNDO_PASSES) break;
        }
        // compaction map (cusimp_free.cu:1042-1045)
        int acc = 0;
        for (int v = 0; v <= nP; ++v) {
            pts_map[v] = acc;
            acc += occ[v];
        }
        return status;
    }
};

// numpy float32 semantics of preprocess_mesh's centring (pamo/__init__.py:61-64):
// tris.mean(axis=1) = ((a+b)+c)/3 per face, then .mean(axis=0) = sequential float32 sum / F
void tris_mean_numpy(const float* pts, const int* tris, int nT, float out[3]) {
    float s[3] = {0, 0, 0};
    for (int f = 0; f < nT; ++f) {
        const int* t = tris + 3 * f;
        for (int d = 0; d < 3; ++d) {
            float m = ((pts[3 * t[0] + d] + pts[3 * t[1] + d]) + pts[3 * t[2] + d]) / 3.0f;
            s[d] += m;
        }
    }
    for (int d = 0; d < 3; ++d) out[d] = s[d] / (float)nT;
}

struct RunState {
    std::vector<float> verts;
    std::vector<int> faces;
    int rounds = 0;
    std::vector<int> faces_per_round;
    std::vector<double> round_seconds;  // wall time of each round (the forward call and the compaction)
};

}  // namespace

extern "C" {

struct pamo_oracle_handle {
    Oracle o;
    RunState run;
};

void* oracle_create(void) { return new pamo_oracle_handle(); }
void oracle_destroy(void* h) { delete (pamo_oracle_handle*)h; }

int oracle_set_threads(void* h, int n) {
    auto* H = (pamo_oracle_handle*)h;
    H->o.threads = n < 1 ? 1 : n;
    return H->o.threads;
}

int oracle_forward(void* h, const float* pts, const int* tris, const int* verts_undo, int n_verts_undo, int nP, int nT,
                   float scale, float threshold, int is_stuck, int init) {
    return ((pamo_oracle_handle*)h)->o.forward(pts, tris, verts_undo, n_verts_undo, nP, nT, scale, threshold, is_stuck != 0, init != 0);
}

int oracle_forward_legacy(void* h, const float* pts, const int* tris, int nP, int nT, float scale, float threshold,
                          int init) {
    return ((pamo_oracle_handle*)h)->o.forward_legacy(pts, tris, nP, nT, scale, threshold, init != 0);
}

// counts[0..9] = n_pts, n_tris, n_vertices_undo, n_edges, n_collapsed_regular, n_collapsed_total, n_considered,
//                n_undo_passes, n_intersect_first (pairs), status
void oracle_counts(void* h, long long* c) {
    Oracle& o = ((pamo_oracle_handle*)h)->o;
    c[0] = o.n_pts; c[1] = o.n_tris; c[2] = o.n_vertices_undo; c[3] = o.n_edges; c[4] = o.n_collapsed_regular;
    c[5] = o.n_collapsed_total; c[6] = o.n_considered; c[7] = o.n_undo_passes; c[8] = o.n_intersect_first; c[9] = o.status;
}

void oracle_outputs(void* h, float* verts, int* tris, int* occ, int* map, int* undo) {
    Oracle& o = ((pamo_oracle_handle*)h)->o;
    std::memcpy(verts, o.points.data(), sizeof(float) * 3 * o.n_pts);
    std::memcpy(tris, o.tris.data(), sizeof(int) * 3 * o.n_tris);
    std::memcpy(occ, o.occ.data(), sizeof(int) * o.n_pts);
    std::memcpy(map, o.pts_map.data(), sizeof(int) * o.n_pts);
    for (int a = 0; a < o.n_vertices_undo; ++a) undo[a] = (a < (int)o.undo_list.size()) ? o.undo_list[a] : 0;
}

void oracle_collapsed(void* h, int* out) {
    Oracle& o = ((pamo_oracle_handle*)h)->o;
    std::memcpy(out, o.collapsed.data(), sizeof(int) * o.collapsed.size());
}

void oracle_edge_costs(void* h, unsigned* out) {
    Oracle& o = ((pamo_oracle_handle*)h)->o;
    std::memcpy(out, o.edge_cost.data(), sizeof(unsigned) * o.n_edges);
}

void oracle_edges(void* h, int* out) {
    Oracle& o = ((pamo_oracle_handle*)h)->o;
    for (int e = 0; e < o.n_edges; ++e) { out[2 * e] = o.eu[e]; out[2 * e + 1] = o.ev[e]; }
}

void oracle_shuffle_perm(long long m, int* perm) {
    std::vector<int> p;
    shuffle_perm((uint64_t)m, p);
    std::memcpy(perm, p.data(), sizeof(int) * p.size());
}

int oracle_pair_intersects(const float* pts, const int* cur, const int* qry, float eps) {
    return pair_intersects((const P3*)pts, F3{cur[0], cur[1], cur[2]}, F3{qry[0], qry[1], qry[2]}, eps) ? 1 : 0;
}

void oracle_tris_mean(const float* pts, const int* tris, int nT, float* out) { tris_mean_numpy(pts, tris, nT, out); }

// selfx::self_intersect (self_intersect.cuh:151-392) on a whole mesh: out[f] = 1 iff face f belongs to a
// (query, hit) pair the reference records. Returns the number of intersecting (query, hit) tests.
long long oracle_self_intersect(void* h, const float* pts, const int* tris, int nP, int nT, unsigned char* out) {
    Oracle& o = ((pamo_oracle_handle*)h)->o;
    o.points.assign((const P3*)pts, (const P3*)pts + nP);
    o.tris.assign((const F3*)tris, (const F3*)tris + nT);
    o.n_pts = nP;
    o.n_tris = nT;
    long long hits = o.self_intersect();
    std::memcpy(out, o.face_hit.data(), nT);
    return hits;
}

// The stage-2 round loop of PaMO.run (pamo/__init__.py:95-163) with stage 1 and stage 3 off.
// Returns the number of rounds; the result is read with oracle_run_result.
// The round loop. PaMO.run (pamo/__init__.py:95-163): centring by tris_mean, stop at the target face count or
// at 10 faces, tolerance compared with ==. Blender entry (pamo_blender/cusimpinterface.cu:57-161, blender=true):
// no centring, no target, stop when >= tolerance rounds in a row removed no face.
static int run_loop(void* h, const float* pts, const int* tris, int nP, int nT, long long target, int tolerance,
                    float threshold, int iters, bool blender, int* out_nP, int* out_nT) {
    auto* H = (pamo_oracle_handle*)h;
    Oracle& o = H->o;
    RunState& R = H->run;
    float mean[3] = {0.f, 0.f, 0.f};
    if (!blender) tris_mean_numpy(pts, tris, nT, mean);
    std::vector<float> verts(pts, pts + 3 * (size_t)nP);
    if (!blender)
        for (int v = 0; v < nP; ++v)
            for (int d = 0; d < 3; ++d) verts[3 * v + d] = verts[3 * v + d] - mean[d];
    std::vector<int> faces(tris, tris + 3 * (size_t)nT);
    float ext[3];
    for (int d = 0; d < 3; ++d) {
        float lo = verts[d], hi = verts[d];
        for (int v = 1; v < nP; ++v) { lo = std::min(lo, verts[3 * v + d]); hi = std::max(hi, verts[3 * v + d]); }
        ext[d] = hi - lo;
    }
    float scale = std::max(std::max(ext[0], ext[1]), ext[2]);
    std::vector<int> undo;
    int count = 0;
    bool stuck = false, init = true;
    R.faces_per_round.clear();
    R.round_seconds.clear();
    int rounds = 0;
    for (int it = 0; it < iters; ++it) {
        const auto t0 = std::chrono::steady_clock::now();
        const int nf_prev = (int)(faces.size() / 3);
        const int np = (int)(verts.size() / 3);
        o.forward(verts.data(), faces.data(), undo.data(), (int)undo.size(), np, nf_prev, scale, threshold, stuck, init);
        ++rounds;
        init = false;
        undo.assign(o.n_vertices_undo, 0);
        for (int a = 0; a < o.n_vertices_undo; ++a) undo[a] = o.undo_list[a];
        // compaction (pamo/__init__.py:136-140)
        std::vector<float> nv;
        nv.reserve(verts.size());
        for (int v = 0; v < np; ++v)
            if (o.occ[v]) { nv.push_back(o.points[v].x); nv.push_back(o.points[v].y); nv.push_back(o.points[v].z); }
        std::vector<int> nf;
        nf.reserve(faces.size());
        for (int f = 0; f < nf_prev; ++f) {
            const F3& t = o.tris[f];
            if (t.i >= 0) { nf.push_back(o.pts_map[t.i]); nf.push_back(o.pts_map[t.j]); nf.push_back(o.pts_map[t.k]); }
        }
        verts.swap(nv);
        faces.swap(nf);
        const int nf_cur = (int)(faces.size() / 3);
        R.faces_per_round.push_back(nf_cur);
        R.round_seconds.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
        if (!blender && (nf_cur <= target || nf_cur <= 10)) break;
        if (nf_cur == nf_prev) {
            count++;
        } else {
            count = 0;
            stuck = false;
        }
        if (count >= 2) stuck = true;
        if (blender ? count >= tolerance : count == tolerance) break;
    }
    if (!blender)
        for (size_t v = 0; v < verts.size() / 3; ++v)
            for (int d = 0; d < 3; ++d) verts[3 * v + d] = verts[3 * v + d] + mean[d];
    R.verts.swap(verts);
    R.faces.swap(faces);
    R.rounds = rounds;
    *out_nP = (int)(R.verts.size() / 3);
    *out_nT = (int)(R.faces.size() / 3);
    return rounds;
}

int oracle_run(void* h, const float* pts, const int* tris, int nP, int nT, double ratio, int tolerance, float threshold,
               int iters, long long min_verts, int* out_nP, int* out_nT) {
    const long long target = std::max((long long)(ratio * (double)nT), min_verts);
    return run_loop(h, pts, tris, nP, nT, target, tolerance, threshold, iters, false, out_nP, out_nT);
}

// wall time of each round of the last run (seconds); returns the number of rounds
int oracle_run_round_seconds(void* h, double* out, int cap) {
    const RunState& R = ((pamo_oracle_handle*)h)->run;
    const int n = (int)R.round_seconds.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = R.round_seconds[i];
    return n;
}

// pamo_simplify of the Blender add-on: scale from the host bounding box of the raw vertices
// (cusimpinterface.cu:62-75), tolerance 4, 1000000 rounds at most
int oracle_run_blender(void* h, const float* pts, const int* tris, int nP, int nT, float threshold, int* out_nP,
                       int* out_nT) {
    return run_loop(h, pts, tris, nP, nT, -1, 4, threshold, 1000000, true, out_nP, out_nT);
}

void oracle_run_result(void* h, float* verts, int* faces, int* faces_per_round) {
    RunState& R = ((pamo_oracle_handle*)h)->run;
    std::memcpy(verts, R.verts.data(), sizeof(float) * R.verts.size());
    std::memcpy(faces, R.faces.data(), sizeof(int) * R.faces.size());
    if (faces_per_round) std::memcpy(faces_per_round, R.faces_per_round.data(), sizeof(int) * R.faces_per_round.size());
}

}  // extern "C"
