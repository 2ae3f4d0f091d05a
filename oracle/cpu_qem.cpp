// A conventional sequential QEM simplifier (Garland & Heckbert, "Surface simplification using quadric error
// metrics", 1997): plane quadrics summed per vertex, edge collapses in cost order from a priority queue, the
// merged vertex at the edge midpoint with cost v^T (Q_u + Q_v) v, a collapse rejected when the two endpoints
// share more than two neighbours (link condition) or when a surviving face would flip its normal.
//
// BASELINE ONLY: bench.py times it on the GPU machine's host cores (one thread) as the CPU QEM baseline of the
// measurement plan. It is not a restatement of the reference's parallel algorithm (that is pamo_oracle.cpp) and
// its output is not compared with anything.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <queue>
#include <vector>

namespace {

struct Q {
    double m[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // a2 ab ac ad b2 bc bd c2 cd d2
    void add_plane(double a, double b, double c, double d) {
        m[0] += a * a; m[1] += a * b; m[2] += a * c; m[3] += a * d; m[4] += b * b;
        m[5] += b * c; m[6] += b * d; m[7] += c * c; m[8] += c * d; m[9] += d * d;
    }
    void add(const Q& o) {
        for (int i = 0; i < 10; ++i) m[i] += o.m[i];
    }
    double eval(double x, double y, double z) const {
        return m[0] * x * x + 2 * m[1] * x * y + 2 * m[2] * x * z + 2 * m[3] * x + m[4] * y * y + 2 * m[5] * y * z +
               2 * m[6] * y + m[7] * z * z + 2 * m[8] * z + m[9];
    }
};

struct Mesh {
    std::vector<double> p;               // 3 per vertex
    std::vector<int> f;                  // 3 per face, -1 when removed
    std::vector<std::vector<int>> vf;    // vertex -> faces
    std::vector<Q> q;
    std::vector<int> ver;                // vertex version (stale queue entries)
    std::vector<char> alive;
    long long live_faces = 0;

    void normal(int fi, double n[3]) const {
        const int* t = &f[3 * fi];
        const double* a = &p[3 * t[0]];
        const double* b = &p[3 * t[1]];
        const double* c = &p[3 * t[2]];
        const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        n[0] = u[1] * w[2] - u[2] * w[1];
        n[1] = u[2] * w[0] - u[0] * w[2];
        n[2] = u[0] * w[1] - u[1] * w[0];
    }
    void neighbours(int v, std::vector<int>& out) const {
        out.clear();
        for (int fi : vf[v]) {
            if (f[3 * fi] < 0) continue;
            for (int k = 0; k < 3; ++k)
                if (f[3 * fi + k] != v) out.push_back(f[3 * fi + k]);
        }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
};

struct Entry {
    double cost;
    int u, v, vu, vv;
    bool operator<(const Entry& o) const { return cost > o.cost; }  // min-heap
};

double edge_cost(const Mesh& m, int u, int v) {
    Q s = m.q[u];
    s.add(m.q[v]);
    const double x = 0.5 * (m.p[3 * u] + m.p[3 * v]), y = 0.5 * (m.p[3 * u + 1] + m.p[3 * v + 1]),
                 z = 0.5 * (m.p[3 * u + 2] + m.p[3 * v + 2]);
    return s.eval(x, y, z);
}

// true when collapsing v into u at the midpoint keeps the link condition and flips no surviving face
bool collapse_ok(Mesh& m, int u, int v, std::vector<int>& nu, std::vector<int>& nv) {
    m.neighbours(u, nu);
    m.neighbours(v, nv);
    int common = 0;
    for (size_t i = 0, j = 0; i < nu.size() && j < nv.size();) {
        if (nu[i] < nv[j]) ++i;
        else if (nu[i] > nv[j]) ++j;
        else {
            ++common;
            ++i;
            ++j;
        }
    }
    if (common > 2) return false;
    const double mid[3] = {0.5 * (m.p[3 * u] + m.p[3 * v]), 0.5 * (m.p[3 * u + 1] + m.p[3 * v + 1]),
                           0.5 * (m.p[3 * u + 2] + m.p[3 * v + 2])};
    for (int w : {u, v}) {
        const int other = w == u ? v : u;
        for (int fi : m.vf[w]) {
            const int* t = &m.f[3 * fi];
            if (t[0] < 0 || t[0] == other || t[1] == other || t[2] == other) continue;
            double n0[3];
            m.normal(fi, n0);
            double save[3];
            for (int k = 0; k < 3; ++k) save[k] = m.p[3 * w + k];
            for (int k = 0; k < 3; ++k) m.p[3 * w + k] = mid[k];
            double n1[3];
            m.normal(fi, n1);
            for (int k = 0; k < 3; ++k) m.p[3 * w + k] = save[k];
            if (n0[0] * n1[0] + n0[1] * n1[1] + n0[2] * n1[2] <= 0.0) return false;
        }
    }
    return true;
}

}  // namespace

extern "C" {

// Simplify to at most target faces (or until no edge can collapse, or time_budget_s elapses; <= 0: no limit);
// returns the number of collapses; *out_faces = live faces at the end.
long long cpu_qem_simplify(const float* pts, int nv, const int* tris, int nf, long long target, double time_budget_s,
                           long long* out_faces) {
    Mesh m;
    m.p.resize(3 * (size_t)nv);
    for (size_t i = 0; i < 3 * (size_t)nv; ++i) m.p[i] = pts[i];
    m.f.assign(tris, tris + 3 * (size_t)nf);
    m.vf.assign(nv, {});
    m.q.assign(nv, Q());
    m.ver.assign(nv, 0);
    m.alive.assign(nv, 1);
    m.live_faces = nf;
    for (int fi = 0; fi < nf; ++fi) {
        double n[3];
        m.normal(fi, n);
        const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; ++k) m.vf[m.f[3 * fi + k]].push_back(fi);
        if (l <= 0) continue;
        const double a = n[0] / l, b = n[1] / l, c = n[2] / l;
        const double d = -(a * m.p[3 * m.f[3 * fi]] + b * m.p[3 * m.f[3 * fi] + 1] + c * m.p[3 * m.f[3 * fi] + 2]);
        for (int k = 0; k < 3; ++k) m.q[m.f[3 * fi + k]].add_plane(a, b, c, d);
    }
    std::priority_queue<Entry> pq;
    for (int fi = 0; fi < nf; ++fi)
        for (int k = 0; k < 3; ++k) {
            const int a = m.f[3 * fi + k], b = m.f[3 * fi + (k + 1) % 3];
            if (a < b) pq.push({edge_cost(m, a, b), a, b, 0, 0});
        }
    const auto t0 = std::chrono::steady_clock::now();
    long long collapses = 0;
    std::vector<int> nu, nvv;
    while (!pq.empty() && m.live_faces > target) {
        if (time_budget_s > 0 && (collapses & 1023) == 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > time_budget_s)
            break;
        const Entry e = pq.top();
        pq.pop();
        if (!m.alive[e.u] || !m.alive[e.v] || m.ver[e.u] != e.vu || m.ver[e.v] != e.vv) continue;
        if (!collapse_ok(m, e.u, e.v, nu, nvv)) continue;
        const int u = e.u, v = e.v;
        for (int k = 0; k < 3; ++k) m.p[3 * u + k] = 0.5 * (m.p[3 * u + k] + m.p[3 * v + k]);
        m.q[u].add(m.q[v]);
        for (int fi : m.vf[v]) {
            int* t = &m.f[3 * fi];
            if (t[0] < 0) continue;
            if (t[0] == u || t[1] == u || t[2] == u) {
                t[0] = t[1] = t[2] = -1;
                --m.live_faces;
            } else {
                for (int k = 0; k < 3; ++k)
                    if (t[k] == v) t[k] = u;
                m.vf[u].push_back(fi);
            }
        }
        m.vf[v].clear();
        m.alive[v] = 0;
        ++m.ver[u];
        ++collapses;
        m.neighbours(u, nu);
        for (int w : nu) {
            const int a = std::min(u, w), b = std::max(u, w);
            pq.push({edge_cost(m, a, b), a, b, m.ver[a], m.ver[b]});
        }
    }
    if (out_faces) *out_faces = m.live_faces;
    return collapses;
}

}  // extern "C"
