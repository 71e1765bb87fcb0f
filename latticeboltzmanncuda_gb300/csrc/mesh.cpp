// Geometry front end for D3Q27_REF (host side, no GPU): a closed triangle mesh turned into the
// cell flags and the reflection tables that the reference derives with CGAL.
//
//   Model::importModel / isModelClosed / checkError   Model.cpp:22-49     OBJ reader, closedness
//   Model::isPointInsideModel                         Model.cpp:51-63     ray parity, boundary = inside
//   Model::reflectionVector                           Model.cpp:75-91     first hit, face normal, rotation
//   rotateVectorAroundAxis                            Geometry.cpp:22-42  quaternion rotation
//   Lattice::insertModel                              Lattice.cpp:228-260
//   Lattice::distributeVector                         Lattice.cpp:262-321
//   Lattice::preProcessModel                          Lattice.cpp:323-426
//
// The reference runs these on CGAL 5/6 (Surface_mesh, AABB_tree, Side_of_triangle_mesh,
// Polygon_mesh_processing::compute_face_normal) with the Simple_cartesian<float> kernel.  CGAL is
// not part of this build; the published algorithms are restated here:
//   * point in mesh: outside the bounding box is outside; a point on a face is on the boundary,
//     which counts as inside; otherwise a ray is cast (first along +-z, towards the nearer bounding
//     box face, then in pseudo-random directions while a ray grazes an edge, a vertex or a face
//     plane) and the parity of its crossings decides;
//   * first intersection: the face hit closest to the ray's source (edges and vertices included;
//     among faces hit at the same distance the lowest face index);
//   * face normal: the sum of 0.5 (p_k p_k+1 x p_k p_0) over the face's fan triangles, divided by
//     its length, in float.
// Predicates are evaluated in double on the float coordinates.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "lbm_capi.h"
#include "lbm_internal.h"

namespace lbm {
lbm_status set_thread_error(lbm_status s, const std::string &msg);
}

namespace {

struct V3 {
    double x, y, z;
};
inline V3 sub(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(const V3 &a, const V3 &b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct Tri {
    V3 a, b, c;
    int32_t face;  // index of the (possibly polygonal) face this triangle belongs to
};

struct Box {
    double lo[3], hi[3];
    void grow(const V3 &p) {
        const double v[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], v[k]);
            hi[k] = std::max(hi[k], v[k]);
        }
    }
    static Box empty() { return {{HUGE_VAL, HUGE_VAL, HUGE_VAL}, {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}}; }
};

// Bounding volume hierarchy over the triangles: median split on the longest axis, leaves of <= 4.
struct BVH {
    struct Node {
        Box box;
        int32_t left, right;  // children, or -1 for a leaf
        int32_t first, count; // leaf triangle range in `order`
    };
    std::vector<Node> nodes;
    std::vector<int32_t> order;

    void build(const std::vector<Tri> &tris) {
        nodes.clear();
        order.resize(tris.size());
        for (size_t i = 0; i < tris.size(); ++i) order[i] = (int32_t)i;
        if (!tris.empty()) make(tris, 0, (int32_t)tris.size());
    }

    int32_t make(const std::vector<Tri> &tris, int32_t first, int32_t count) {
        Box b = Box::empty();
        for (int32_t i = first; i < first + count; ++i) {
            const Tri &t = tris[(size_t)order[(size_t)i]];
            b.grow(t.a), b.grow(t.b), b.grow(t.c);
        }
        const int32_t id = (int32_t)nodes.size();
        nodes.push_back({b, -1, -1, first, count});
        if (count <= 4) return id;
        int axis = 0;
        double ext = -1;
        for (int k = 0; k < 3; ++k)
            if (b.hi[k] - b.lo[k] > ext) ext = b.hi[k] - b.lo[k], axis = k;
        auto key = [&](int32_t i) {
            const Tri &t = tris[(size_t)i];
            const double c[3] = {t.a.x + t.b.x + t.c.x, t.a.y + t.b.y + t.c.y, t.a.z + t.b.z + t.c.z};
            return c[axis];
        };
        const int32_t mid = first + count / 2;
        std::nth_element(order.begin() + first, order.begin() + mid, order.begin() + first + count,
                         [&](int32_t p, int32_t q) { return key(p) < key(q) || (key(p) == key(q) && p < q); });
        const int32_t l = make(tris, first, count / 2);
        const int32_t r = make(tris, mid, count - count / 2);
        nodes[(size_t)id].left = l;
        nodes[(size_t)id].right = r;
        return id;
    }

    // visit the triangles of every leaf whose box passes `test`
    template <class BoxTest, class Visit>
    void walk(BoxTest &&test, Visit &&visit) const {
        if (nodes.empty()) return;
        int32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const Node &n = nodes[(size_t)stack[--sp]];
            if (!test(n.box)) continue;
            if (n.left < 0) {
                for (int32_t i = n.first; i < n.first + n.count; ++i) visit(order[(size_t)i]);
            } else if (sp + 2 <= 128) {
                stack[sp++] = n.left;
                stack[sp++] = n.right;
            }
        }
    }
};

// slab test of the ray o + t d, t >= 0, against a box widened by eps
bool ray_box(const V3 &o, const V3 &d, const Box &b, double eps) {
    double t0 = 0.0, t1 = HUGE_VAL;
    const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; ++k) {
        const double lo = b.lo[k] - eps, hi = b.hi[k] + eps;
        if (dd[k] == 0.0) {
            if (oo[k] < lo || oo[k] > hi) return false;
            continue;
        }
        double a = (lo - oo[k]) / dd[k], c = (hi - oo[k]) / dd[k];
        if (a > c) std::swap(a, c);
        t0 = std::max(t0, a);
        t1 = std::min(t1, c);
        if (t0 > t1) return false;
    }
    return true;
}

}  // namespace

struct lbm_mesh {
    std::vector<float> xyz;                 // 3 per vertex
    std::vector<std::vector<int32_t>> faces;
    std::vector<Tri> tris;                  // fan triangulation of every face
    BVH bvh;
    Box box = Box::empty();
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    bool triangle_mesh = false, closed = false;
    double scale = 1.0;                     // bounding-box diagonal, for the boundary tolerance

    bool valid() const { return triangle_mesh && closed && !faces.empty(); }

    V3 vertex(int32_t i) const {
        return {(double)xyz[3 * (size_t)i], (double)xyz[3 * (size_t)i + 1], (double)xyz[3 * (size_t)i + 2]};
    }
};

namespace {

lbm_status finish_mesh(lbm_mesh *m) {
    const int64_t nv = (int64_t)(m->xyz.size() / 3);
    m->triangle_mesh = !m->faces.empty();
    for (const auto &f : m->faces) {
        if (f.size() < 3) return lbm::set_thread_error(LBM_ERR_INVALID, "mesh face with fewer than 3 vertices");
        for (int32_t v : f)
            if (v < 0 || v >= nv) return lbm::set_thread_error(LBM_ERR_INVALID, "mesh face index out of range");
        if (f.size() != 3) m->triangle_mesh = false;
    }
    // closed: every directed edge a->b of a face has its opposite b->a in another face
    std::map<std::pair<int32_t, int32_t>, int32_t> edges;
    for (const auto &f : m->faces)
        for (size_t k = 0; k < f.size(); ++k) ++edges[{f[k], f[(k + 1) % f.size()]}];
    m->closed = !m->faces.empty();
    for (const auto &e : edges) {
        auto it = edges.find({e.first.second, e.first.first});
        if (it == edges.end() || it->second != e.second) {
            m->closed = false;
            break;
        }
    }
    m->box = Box::empty();
    for (int64_t i = 0; i < nv; ++i) m->box.grow(m->vertex((int32_t)i));
    if (nv > 0) {
        for (int k = 0; k < 3; ++k) m->bmin[k] = m->bmax[k] = m->xyz[(size_t)k];
        for (int64_t i = 0; i < nv; ++i)
            for (int k = 0; k < 3; ++k) {
                m->bmin[k] = std::min(m->bmin[k], m->xyz[3 * (size_t)i + k]);
                m->bmax[k] = std::max(m->bmax[k], m->xyz[3 * (size_t)i + k]);
            }
        const double dx = m->box.hi[0] - m->box.lo[0], dy = m->box.hi[1] - m->box.lo[1], dz = m->box.hi[2] - m->box.lo[2];
        m->scale = std::max(1e-30, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    m->tris.clear();
    for (size_t fi = 0; fi < m->faces.size(); ++fi) {
        const auto &f = m->faces[fi];
        for (size_t k = 1; k + 1 < f.size(); ++k)
            m->tris.push_back({m->vertex(f[0]), m->vertex(f[k]), m->vertex(f[k + 1]), (int32_t)fi});
    }
    m->bvh.build(m->tris);
    return LBM_OK;
}

// Relation of the ray o + t d (t > 0) to one triangle.
enum class Hit { None, Cross, Degenerate, Source };

Hit classify(const Tri &t, const V3 &o, const V3 &d, double eps_vol) {
    const V3 a = sub(t.a, o), b = sub(t.b, o), c = sub(t.c, o);
    // signed volumes of the ray line against the three edges
    const double u = dot(d, cross(b, c)), v = dot(d, cross(c, a)), w = dot(d, cross(a, b));
    const bool neg = u < -eps_vol || v < -eps_vol || w < -eps_vol;
    const bool pos = u > eps_vol || v > eps_vol || w > eps_vol;
    if (neg && pos) return Hit::None;  // the line misses the triangle
    const V3 n = cross(sub(t.b, t.a), sub(t.c, t.a));
    const double dn = dot(d, n);
    const double num = dot(a, n);  // t * dn
    if (!neg && !pos) return Hit::Degenerate;  // the line lies in the triangle's plane or grazes a vertex
    const bool on_edge = std::fabs(u) <= eps_vol || std::fabs(v) <= eps_vol || std::fabs(w) <= eps_vol;
    if (dn == 0.0) return Hit::Degenerate;
    const double tt = num / dn;
    if (std::fabs(num) <= 1e-12 * std::sqrt(dot(n, n)) * std::sqrt(dot(a, a) + 1e-300)) return Hit::Source;
    if (tt < 0.0) return Hit::None;
    return on_edge ? Hit::Degenerate : Hit::Cross;
}

// point-triangle distance test for the boundary case
bool on_triangle(const Tri &t, const V3 &p, double eps) {
    const V3 ab = sub(t.b, t.a), ac = sub(t.c, t.a), ap = sub(p, t.a);
    const V3 n = cross(ab, ac);
    const double nn = dot(n, n);
    if (nn == 0.0) return false;
    const double dist = dot(ap, n) / std::sqrt(nn);
    if (std::fabs(dist) > eps) return false;
    // barycentric coordinates of the projection, with a tolerance of eps along the edges
    const V3 q = {p.x - dist * n.x / std::sqrt(nn), p.y - dist * n.y / std::sqrt(nn), p.z - dist * n.z / std::sqrt(nn)};
    const V3 e[3] = {sub(t.b, t.a), sub(t.c, t.b), sub(t.a, t.c)};
    const V3 s[3] = {sub(q, t.a), sub(q, t.b), sub(q, t.c)};
    for (int k = 0; k < 3; ++k) {
        const double side = dot(cross(e[k], s[k]), n) / std::sqrt(nn);  // distance-scaled edge test
        const double len = std::sqrt(dot(e[k], e[k]));
        if (len > 0 && side / len < -eps) return false;
    }
    return true;
}

struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

bool point_inside(const lbm_mesh &m, const float pf[3]) {
    if (!m.valid()) return false;
    const V3 p = {(double)pf[0], (double)pf[1], (double)pf[2]};
    if (p.x < m.box.lo[0] || p.x > m.box.hi[0] || p.y < m.box.lo[1] || p.y > m.box.hi[1] || p.z < m.box.lo[2] ||
        p.z > m.box.hi[2])
        return false;
    const double eps = 1e-7 * m.scale;
    bool boundary = false;
    m.bvh.walk(
        [&](const Box &b) {
            return !boundary && p.x >= b.lo[0] - eps && p.x <= b.hi[0] + eps && p.y >= b.lo[1] - eps &&
                   p.y <= b.hi[1] + eps && p.z >= b.lo[2] - eps && p.z <= b.hi[2] + eps;
        },
        [&](int32_t i) {
            if (!boundary && on_triangle(m.tris[(size_t)i], p, eps)) boundary = true;
        });
    if (boundary) return true;
    // first a vertical ray towards the nearer z face of the box, then pseudo-random directions
    V3 d = {0.0, 0.0, 2.0 * p.z < m.box.lo[2] + m.box.hi[2] ? -1.0 : 1.0};
    Rng rng{0x243F6A8885A308D3ull ^ ((uint64_t)(uint32_t)(int32_t)std::lround(p.x * 1e6) * 0x100000001B3ull) ^
            ((uint64_t)(uint32_t)(int32_t)std::lround(p.y * 1e6) << 21) ^ (uint64_t)(uint32_t)(int32_t)std::lround(p.z * 1e6)};
    for (int attempt = 0; attempt < 256; ++attempt) {
        int crossings = 0;
        bool degenerate = false, source = false;
        const double eps_vol = 1e-13 * m.scale * m.scale;
        m.bvh.walk([&](const Box &b) { return !degenerate && ray_box(p, d, b, eps); },
                   [&](int32_t i) {
                       if (degenerate) return;
                       switch (classify(m.tris[(size_t)i], p, d, eps_vol)) {
                           case Hit::Cross: ++crossings; break;
                           case Hit::Degenerate: degenerate = true; break;
                           case Hit::Source: source = true; break;
                           default: break;
                       }
                   });
        if (source) return true;
        if (!degenerate) return (crossings & 1) != 0;
        // uniform direction on the sphere (Marsaglia 1972)
        double x1, x2, s2;
        do {
            x1 = 2.0 * rng.u01() - 1.0;
            x2 = 2.0 * rng.u01() - 1.0;
            s2 = x1 * x1 + x2 * x2;
        } while (s2 >= 1.0 || s2 == 0.0);
        const double r = 2.0 * std::sqrt(1.0 - s2);
        d = {x1 * r, x2 * r, 1.0 - 2.0 * s2};
    }
    return false;
}

// closest face hit by the ray from p1 through p2 (edges included), -1 if none
int32_t first_hit(const lbm_mesh &m, const V3 &o, const V3 &d) {
    double best = HUGE_VAL;
    int32_t face = -1;
    const double eps = 1e-7 * m.scale;
    const double eps_vol = 1e-13 * m.scale * m.scale * std::sqrt(dot(d, d));
    m.bvh.walk([&](const Box &b) { return ray_box(o, d, b, eps); },
               [&](int32_t i) {
                   const Tri &t = m.tris[(size_t)i];
                   const V3 a = sub(t.a, o), b = sub(t.b, o), c = sub(t.c, o);
                   const double u = dot(d, cross(b, c)), v = dot(d, cross(c, a)), w = dot(d, cross(a, b));
                   const bool neg = u < -eps_vol || v < -eps_vol || w < -eps_vol;
                   const bool pos = u > eps_vol || v > eps_vol || w > eps_vol;
                   if (neg && pos) return;
                   const V3 n = cross(sub(t.b, t.a), sub(t.c, t.a));
                   const double dn = dot(d, n);
                   if (dn == 0.0) return;  // parallel to the face plane
                   const double tt = dot(a, n) / dn;
                   if (tt < 0.0) return;
                   if (tt < best || (tt == best && t.face < face)) {
                       best = tt;
                       face = t.face;
                   }
               });
    return face;
}

// face normal in float: the sum of 0.5 * (p_k p_k+1 x p_k p_0) over the fan triangles
// (p_0, p_k, p_k+1) of the face, divided by its length
void face_normal(const lbm_mesh &m, int32_t fi, float out[3]) {
    const auto &f = m.faces[(size_t)fi];
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    const float *p0 = &m.xyz[3 * (size_t)f[0]];
    for (size_t k = 1; k + 1 < f.size(); ++k) {
        const float *p1 = &m.xyz[3 * (size_t)f[k]];
        const float *p2 = &m.xyz[3 * (size_t)f[k + 1]];
        const float ax = p2[0] - p1[0], ay = p2[1] - p1[1], az = p2[2] - p1[2];
        const float bx = p0[0] - p1[0], by = p0[1] - p1[1], bz = p0[2] - p1[2];
        const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        nx = nx + cx * 0.5f;
        ny = ny + cy * 0.5f;
        nz = nz + cz * 0.5f;
    }
    const float sq = nx * nx + ny * ny + nz * nz;
    if (sq != 0.0f) {
        const float len = std::sqrt(sq);
        nx = nx / len;
        ny = ny / len;
        nz = nz / len;
    }
    out[0] = nx, out[1] = ny, out[2] = nz;
}

// Hamilton product of quaternions (w, x, y, z)
void qmul(const float a[4], const float b[4], float r[4]) {
    r[0] = (a[0] * b[0]) - (a[1] * b[1]) - (a[2] * b[2]) - (a[3] * b[3]);
    r[1] = (a[0] * b[1]) + (a[1] * b[0]) + (a[2] * b[3]) - (a[3] * b[2]);
    r[2] = (a[0] * b[2]) - (a[1] * b[3]) + (a[2] * b[0]) + (a[3] * b[1]);
    r[3] = (a[0] * b[3]) + (a[1] * b[2]) - (a[2] * b[1]) + (a[3] * b[0]);
}

void rotate(const float axis_in[3], const float v[3], float angle, float out[3]) {
    const float mag = std::sqrt((axis_in[0] * axis_in[0]) + (axis_in[1] * axis_in[1]) + (axis_in[2] * axis_in[2]));
    const float ax = axis_in[0] / mag, ay = axis_in[1] / mag, az = axis_in[2] / mag;
    const float h = (float)((double)angle / 2.0);
    const float c = std::cos(h), s = std::sin(h), cn = std::cos(-h), sn = std::sin(-h);
    const float q[4] = {c, s * ax, s * ay, s * az};
    const float qi[4] = {cn, sn * ax, sn * ay, sn * az};
    const float pt[4] = {0.0f, v[0], v[1], v[2]};
    float t[4], r[4];
    qmul(q, pt, t);
    qmul(t, qi, r);
    out[0] = r[1], out[1] = r[2], out[2] = r[3];
}

void reflection_vector(const lbm_mesh &m, const float p1[3], const float p2[3], float out[3]) {
    const V3 o = {(double)p1[0], (double)p1[1], (double)p1[2]};
    const V3 d = {(double)p2[0] - o.x, (double)p2[1] - o.y, (double)p2[2] - o.z};
    float v[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
    const float norm = std::sqrt((v[0] * v[0]) + (v[1] * v[1]) + (v[2] * v[2]));
    v[0] /= norm, v[1] /= norm, v[2] /= norm;
    const int32_t f = (d.x == 0.0 && d.y == 0.0 && d.z == 0.0) ? -1 : first_hit(m, o, d);
    if (f < 0) {
        out[0] = out[1] = out[2] = 0.0f;
        return;
    }
    float n[3];
    face_normal(m, f, n);
    rotate(n, v, (float)M_PI, out);
}

// unit D3Q27 directions in float, each c_q / |c_q| rounded once from double
struct UnitDirs {
    float u[27][3];
    UnitDirs() {
        for (int q = 0; q < 27; ++q) {
            const int l2 = lbm::kD3Q27[q][0] * lbm::kD3Q27[q][0] + lbm::kD3Q27[q][1] * lbm::kD3Q27[q][1] +
                           lbm::kD3Q27[q][2] * lbm::kD3Q27[q][2];
            const double len = l2 ? std::sqrt((double)l2) : 1.0;
            for (int k = 0; k < 3; ++k) u[q][k] = l2 ? (float)((double)lbm::kD3Q27[q][k] / len) : 0.0f;
        }
    }
};
const UnitDirs &unit_dirs() {
    static const UnitDirs u;
    return u;
}

void distribute(const float v[3], float score[27], int32_t dir[27]) {
    const UnitDirs &U = unit_dirs();
    std::pair<float, int> s[27];
    for (int q = 0; q < 27; ++q) {
        const float dx = v[0] - U.u[q][0], dy = v[1] - U.u[q][1], dz = v[2] - U.u[q][2];
        const float len = std::sqrt(((dx * dx) + (dy * dy)) + (dz * dz));
        s[q] = {(float)(2.0 - (double)len), q};
    }
    // descending by score, equal scores by the larger direction index first
    std::sort(s, s + 27, [](const std::pair<float, int> &a, const std::pair<float, int> &b) { return b < a; });
    for (int i = 0; i < 27; ++i) score[i] = s[i].first, dir[i] = s[i].second;
}

void set_refl_dir(lbm::ReflRecord &r, int s, int dir) {
    const uint32_t shift = 5u * (uint32_t)(s % 6);
    uint32_t word = (uint32_t)r.dirs[s / 6];
    word = (word & ~(31u << shift)) | ((uint32_t)dir << shift);
    r.dirs[s / 6] = (int32_t)word;
}

bool check_dims(int32_t X, int32_t Y, int32_t Z, float spacing) {
    return X >= 1 && Y >= 1 && Z >= 1 && (int64_t)X * Y * Z <= INT32_MAX && spacing > 0.0f && std::isfinite(spacing);
}

}  // namespace

extern "C" {

LBM_API lbm_status lbm_mesh_load_obj(const char *path, lbm_mesh **out) {
    if (!path || !out) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_load_obj: null argument");
    *out = nullptr;
    std::ifstream in(path);
    if (!in) return lbm::set_thread_error(LBM_ERR_INVALID, std::string("lbm_mesh_load_obj: cannot open ") + path);
    std::unique_ptr<lbm_mesh> m(new lbm_mesh());
    std::string line;
    int64_t lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag)) continue;
        if (tag == "v") {
            std::string sx, sy, sz;
            if (!(ls >> sx >> sy >> sz))
                return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_load_obj: bad vertex on line " + std::to_string(lineno));
            for (const std::string *t : {&sx, &sy, &sz}) {
                char *end = nullptr;
                const double val = std::strtod(t->c_str(), &end);
                if (end == t->c_str() || *end)
                    return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_load_obj: bad number on line " + std::to_string(lineno));
                m->xyz.push_back((float)val);
            }
        } else if (tag == "f") {
            std::vector<int32_t> f;
            std::string tok;
            const int64_t nv = (int64_t)(m->xyz.size() / 3);
            while (ls >> tok) {
                const std::string idx = tok.substr(0, tok.find('/'));
                char *end = nullptr;
                const long v = std::strtol(idx.c_str(), &end, 10);
                if (end == idx.c_str() || *end || v == 0)
                    return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_load_obj: bad face index on line " + std::to_string(lineno));
                f.push_back((int32_t)(v > 0 ? v - 1 : nv + v));  // negative indices count back from the last vertex
            }
            m->faces.push_back(std::move(f));
        }
    }
    const lbm_status st = finish_mesh(m.get());
    if (st != LBM_OK) return st;
    *out = m.release();
    return LBM_OK;
}

LBM_API lbm_status lbm_mesh_create(const float *vertices, int64_t nv, const int32_t *face_sizes, int64_t nf,
                                   const int32_t *face_indices, lbm_mesh **out) {
    if (!out || nv < 0 || nf < 0 || (nv && !vertices) || (nf && (!face_sizes || !face_indices)))
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_create: bad argument");
    *out = nullptr;
    std::unique_ptr<lbm_mesh> m(new lbm_mesh());
    m->xyz.assign(vertices, vertices + 3 * nv);
    int64_t at = 0;
    for (int64_t i = 0; i < nf; ++i) {
        if (face_sizes[i] < 3) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_create: face with fewer than 3 vertices");
        m->faces.emplace_back(face_indices + at, face_indices + at + face_sizes[i]);
        at += face_sizes[i];
    }
    const lbm_status st = finish_mesh(m.get());
    if (st != LBM_OK) return st;
    *out = m.release();
    return LBM_OK;
}

LBM_API void lbm_mesh_destroy(lbm_mesh *m) { delete m; }

LBM_API lbm_status lbm_mesh_get_info(const lbm_mesh *m, lbm_mesh_info *out) {
    if (!m || !out) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_get_info: null argument");
    std::memset(out, 0, sizeof(*out));
    out->vertices = (int64_t)(m->xyz.size() / 3);
    out->faces = (int64_t)m->faces.size();
    out->triangle_mesh = m->triangle_mesh;
    out->closed = m->closed;
    out->valid = m->valid();
    for (int k = 0; k < 3; ++k) out->bbox_min[k] = m->bmin[k], out->bbox_max[k] = m->bmax[k];
    return LBM_OK;
}

LBM_API lbm_status lbm_mesh_point_inside(const lbm_mesh *m, const float point[3], int32_t *inside) {
    if (!m || !point || !inside) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_point_inside: null argument");
    *inside = point_inside(*m, point) ? 1 : 0;
    return LBM_OK;
}

LBM_API lbm_status lbm_mesh_reflection_vector(const lbm_mesh *m, const float p1[3], const float p2[3], float out[3]) {
    if (!m || !p1 || !p2 || !out) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_reflection_vector: null argument");
    reflection_vector(*m, p1, p2, out);
    return LBM_OK;
}

LBM_API void lbm_rotate_vector(const float axis[3], const float v[3], float angle, float out[3]) {
    if (axis && v && out) rotate(axis, v, angle, out);
}

LBM_API void lbm_distribute_vector(const float v[3], float score_out[27], int32_t dir_out[27]) {
    if (v && score_out && dir_out) distribute(v, score_out, dir_out);
}

LBM_API lbm_status lbm_mesh_rasterize(const lbm_mesh *m, int32_t X, int32_t Y, int32_t Z, float spacing,
                                      uint8_t *host_flags, int32_t *applied) {
    if (!m || !host_flags) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_rasterize: null argument");
    if (!check_dims(X, Y, Z, spacing)) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_rasterize: bad lattice size or spacing");
    if (applied) *applied = 0;
    // a model that does not fit the lattice leaves the flags alone (Lattice.cpp:236-244)
    if (m->bmin[0] < 0.0f || m->bmin[1] < 0.0f || m->bmin[2] < 0.0f || m->bmax[0] > (float)X * spacing ||
        m->bmax[1] > (float)Y * spacing || m->bmax[2] > (float)Z * spacing)
        return LBM_OK;
    const unsigned hw = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    const int32_t nthreads = (int32_t)std::min<int64_t>(hw, X);
    auto work = [&](int32_t t) {
        for (int32_t x = t; x < X; x += nthreads)
            for (int32_t y = 0; y < Y; ++y)
                for (int32_t z = 0; z < Z; ++z) {
                    const float p[3] = {(float)x * spacing, (float)y * spacing, (float)z * spacing};
                    uint8_t &f = host_flags[(size_t)z + (size_t)Z * ((size_t)y + (size_t)Y * (size_t)x)];
                    f = point_inside(*m, p) ? (uint8_t)(f | LBM_INTERNAL) : (uint8_t)(f & ~LBM_INTERNAL);
                }
    };
    std::vector<std::thread> pool;
    for (int32_t t = 1; t < nthreads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
    if (applied) *applied = 1;
    return LBM_OK;
}

LBM_API lbm_status lbm_mesh_reflection_tables(const lbm_mesh *m, int32_t X, int32_t Y, int32_t Z, float spacing,
                                              uint8_t *host_flags, int64_t capacity, int32_t *host_cells,
                                              void *host_records, int64_t *count) {
    if (!m || !host_flags || !count) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_reflection_tables: null argument");
    if (!check_dims(X, Y, Z, spacing)) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_reflection_tables: bad lattice size or spacing");
    const int64_t cells = (int64_t)X * Y * Z;
    auto internal = [&](int64_t i) { return i >= 0 && i < cells && (host_flags[i] & LBM_INTERNAL); };
    std::vector<int32_t> out_cells;
    std::vector<lbm::ReflRecord> out_recs;
    for (int32_t x = 0; x < X; ++x)
        for (int32_t y = 0; y < Y; ++y)
            for (int32_t z = 0; z < Z; ++z) {
                const int64_t c = (int64_t)z + (int64_t)Z * ((int64_t)y + (int64_t)Y * x);
                if (!(host_flags[c] & LBM_INTERNAL)) continue;
                int64_t rec = -1;
                for (int d = 0; d < 27; ++d) {
                    const int32_t nx = x + lbm::kD3Q27[d][0], ny = y + lbm::kD3Q27[d][1], nz = z + lbm::kD3Q27[d][2];
                    if (nx < 0 || ny < 0 || nz < 0 || nx >= X || ny >= Y || nz >= Z) continue;
                    if (internal((int64_t)nz + (int64_t)Z * ((int64_t)ny + (int64_t)Y * nx))) continue;
                    const float p1[3] = {spacing * (float)nx, spacing * (float)ny, spacing * (float)nz};
                    const float p2[3] = {spacing * (float)x, spacing * (float)y, spacing * (float)z};
                    float rv[3];
                    reflection_vector(*m, p1, p2, rv);
                    float score[27];
                    int32_t dir[27];
                    distribute(rv, score, dir);
                    const int base = lbm::d3q27_inverse(d) * 3;
                    int counter = 0;
                    float norm = 0.0f;
                    for (int i = 0; i < 27 && counter < 3; ++i) {
                        // the neighbour in direction dir[i], by the reference's linear index (no range check
                        // there; an index outside the lattice counts as not internal here)
                        const int64_t nb = ((int64_t)z + lbm::kD3Q27[dir[i]][2]) + (int64_t)Z * ((int64_t)y + lbm::kD3Q27[dir[i]][1]) +
                                           (int64_t)Z * Y * ((int64_t)x + lbm::kD3Q27[dir[i]][0]);
                        if (internal(nb)) continue;
                        if (rec < 0) {
                            rec = (int64_t)out_recs.size();
                            out_recs.emplace_back();
                            std::memset(&out_recs.back(), 0, sizeof(lbm::ReflRecord));
                            out_cells.push_back((int32_t)c);
                        }
                        set_refl_dir(out_recs[(size_t)rec], base + counter, dir[i]);
                        out_recs[(size_t)rec].w[base + counter] = score[i];
                        norm += score[i];
                        ++counter;
                    }
                    if (norm != 0.0f && rec >= 0)
                        for (int i = 0; i < 3; ++i)
                            if (lbm::refl_dir(out_recs[(size_t)rec], base + i) != 0) out_recs[(size_t)rec].w[base + i] /= norm;
                }
            }
    *count = (int64_t)out_cells.size();
    if (!host_cells && !host_records) return LBM_OK;  // size query
    if (!host_cells || !host_records || capacity < *count)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_mesh_reflection_tables: output capacity below the table count");
    std::memcpy(host_cells, out_cells.data(), out_cells.size() * sizeof(int32_t));
    std::memcpy(host_records, out_recs.data(), out_recs.size() * sizeof(lbm::ReflRecord));
    for (int32_t c : out_cells) host_flags[c] |= LBM_REFLECTED;
    return LBM_OK;
}

}  // extern "C"
