// Host-side construction of convex hull shapes (src/shapes/convex-hull.ts create :106-446) in FP64.
//
// The hull itself comes from this file's QuickHull: an initial tetrahedron chosen as the
// reference's builder chooses it (furthest point from the origin, furthest from that, largest
// triangle, largest tetrahedron; src/shapes/utils/convex-hull-builder.ts initialize :65-330),
// then points added furthest first, each replacing the faces it sees with a cone over the
// horizon.  Points within the hull tolerance (1e-3) of the hull are not added, and adjacent
// triangles whose vertices lie within the tolerance of each other's planes are merged into one
// polygon face.  From the finished polygons the shape follows the reference step by step:
//   - face normals and centroids as calculateNormalAndCentroid (convex-hull-builder.ts:646-700):
//     fan normals from the two shortest edges, the centroid as the vertex average;
//   - centre of mass and volume from tetrahedra fanned against the mean face centroid
//     (getCenterOfMassAndVolume :492-563);
//   - the covariance inertia of those tetrahedra about the centre of mass (convex-hull.ts:137-207);
//   - points relative to the centre of mass, planes through the face centroids (:209-260);
//   - for each point the 1-3 neighbouring faces that best define it (:272-329);
//   - the convex radius reduced for thin hulls and sharp vertices (:331-432);
//   - the points shrunk by the convex radius (setConvexHullNoConvexSupport :732-788).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <map>
#include <numeric>
#include <utility>
#include <vector>

namespace cc_hull {

struct V {
    double x, y, z;
};
inline V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V operator*(V a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double len(V a) { return std::sqrt(dot(a, a)); }
inline V normalize(V a) {
    double l = len(a);
    return l > 0 ? a * (1.0 / l) : a;
}

struct Hull {
    std::vector<V> points;          // hull vertices relative to the centre of mass
    std::vector<int> face_first, face_count, vidx;
    std::vector<V> plane_n;         // unit face normals
    std::vector<double> plane_c;    // plane constants: n . x + c = 0
    std::vector<std::array<int, 4>> point_faces;  // count, then up to 3 face indices
    std::vector<V> shrunk;          // points moved inwards by the convex radius
    V com{0, 0, 0};                 // centre of mass in the input frame
    double volume = 0, convex_radius = 0, inner_radius = 0;
    double inertia[9] = {0};        // about the centre of mass, unit density, row-major
    V lo{0, 0, 0}, hi{0, 0, 0};     // bounds of the points (relative to the centre of mass)
};

// ---------------------------------------------------------------------------
// QuickHull
// ---------------------------------------------------------------------------
struct Tri {
    int v[3];
    int adj[3];  // neighbour across edge (v[k], v[k+1])
    V n;
    double d;  // n . x = d on the plane
    bool alive;
    std::vector<int> conflict;
};

inline bool tri_plane(const std::vector<V> &p, Tri &t) {
    V n = cross(p[t.v[1]] - p[t.v[0]], p[t.v[2]] - p[t.v[0]]);
    double l = len(n);
    if (!(l > 0)) return false;
    t.n = n * (1.0 / l);
    t.d = dot(t.n, p[t.v[0]]);
    return true;
}

// Builds the triangulated hull of p; returns false for degenerate (flat or too few) input.
inline bool quickhull(const std::vector<V> &p, double tol, std::vector<Tri> &tris) {
    int n = (int)p.size();
    if (n < 4) return false;
    int i1 = 0;
    double best = -1;
    for (int i = 0; i < n; i++)
        if (dot(p[i], p[i]) > best) best = dot(p[i], p[i]), i1 = i;
    int i2 = -1;
    best = -1;
    for (int i = 0; i < n; i++)
        if (i != i1 && dot(p[i] - p[i1], p[i] - p[i1]) > best) best = dot(p[i] - p[i1], p[i] - p[i1]), i2 = i;
    int i3 = -1;
    best = -1;
    for (int i = 0; i < n; i++) {
        if (i == i1 || i == i2) continue;
        V c = cross(p[i1] - p[i], p[i2] - p[i]);
        if (dot(c, c) > best) best = dot(c, c), i3 = i;
    }
    if (best < 1e-12) return false;
    V pn = normalize(cross(p[i2] - p[i1], p[i3] - p[i1]));
    V cen = (p[i1] + p[i2] + p[i3]) * (1.0 / 3.0);
    int i4 = -1;
    double md = 0;
    for (int i = 0; i < n; i++) {
        if (i == i1 || i == i2 || i == i3) continue;
        double d = dot(p[i] - cen, pn);
        if (std::fabs(d) > std::fabs(md)) md = d, i4 = i;
    }
    if (i4 < 0 || std::fabs(md) <= tol) return false;  // flat: no volume
    if (md < 0) std::swap(i2, i3);  // faces of the tetrahedron face outwards
    tris.clear();
    auto add = [&](int a, int b, int c) {
        Tri t;
        t.v[0] = a;
        t.v[1] = b;
        t.v[2] = c;
        t.adj[0] = t.adj[1] = t.adj[2] = -1;
        t.alive = true;
        tri_plane(p, t);
        tris.push_back(t);
        return (int)tris.size() - 1;
    };
    add(i1, i2, i4);
    add(i2, i3, i4);
    add(i3, i1, i4);
    add(i1, i3, i2);
    // adjacency from directed edges
    auto link_all = [&](const std::vector<int> &ids) {
        std::map<std::pair<int, int>, std::pair<int, int>> edge;
        for (int f : ids)
            for (int k = 0; k < 3; k++) edge[{tris[f].v[k], tris[f].v[(k + 1) % 3]}] = {f, k};
        for (int f : ids)
            for (int k = 0; k < 3; k++) {
                auto it = edge.find({tris[f].v[(k + 1) % 3], tris[f].v[k]});
                if (it != edge.end()) tris[f].adj[k] = it->second.first;
            }
    };
    link_all({0, 1, 2, 3});
    auto assign = [&](int pi, const std::vector<int> &cands) {
        int bf = -1;
        double bd = tol;
        for (int f : cands) {
            if (!tris[f].alive) continue;
            double d = dot(tris[f].n, p[pi]) - tris[f].d;
            if (d > bd) bd = d, bf = f;
        }
        if (bf >= 0) tris[bf].conflict.push_back(pi);
    };
    std::vector<int> all = {0, 1, 2, 3};
    for (int i = 0; i < n; i++)
        if (i != i1 && i != i2 && i != i3 && i != i4) assign(i, all);
    for (int guard = 0; guard < 4 * n + 16; guard++) {
        // the conflict point furthest from its face
        int ef = -1, ep = -1;
        double ed = 0;
        for (int f = 0; f < (int)tris.size(); f++) {
            if (!tris[f].alive) continue;
            for (int pi : tris[f].conflict) {
                double d = dot(tris[f].n, p[pi]) - tris[f].d;
                if (d > ed) ed = d, ef = f, ep = pi;
            }
        }
        if (ef < 0) break;
        // faces visible from ep
        std::vector<int> visible, stack = {ef};
        std::vector<char> seen(tris.size(), 0);
        seen[ef] = 1;
        while (!stack.empty()) {
            int f = stack.back();
            stack.pop_back();
            visible.push_back(f);
            for (int k = 0; k < 3; k++) {
                int g = tris[f].adj[k];
                if (g < 0 || seen[g]) continue;
                if (dot(tris[g].n, p[ep]) - tris[g].d > 0) {
                    seen[g] = 1;
                    stack.push_back(g);
                }
            }
        }
        // horizon edges (a, b) of visible faces next to hidden ones; new faces (a, b, ep)
        std::vector<int> orphans, fresh;
        std::vector<std::pair<int, int>> outer;  // hidden neighbour and its edge index
        for (int f : visible) {
            for (int k = 0; k < 3; k++) {
                int g = tris[f].adj[k];
                if (g >= 0 && seen[g]) continue;
                int a = tris[f].v[k], b = tris[f].v[(k + 1) % 3];
                int nf = add(a, b, ep);
                fresh.push_back(nf);
                tris[nf].adj[0] = g;
                if (g >= 0)
                    for (int m = 0; m < 3; m++)
                        if (tris[g].v[m] == b && tris[g].v[(m + 1) % 3] == a) tris[g].adj[m] = nf;
            }
        }
        for (int f : visible) {
            tris[f].alive = false;
            for (int pi : tris[f].conflict)
                if (pi != ep) orphans.push_back(pi);
            tris[f].conflict.clear();
        }
        // link the new faces to each other around the apex
        std::map<std::pair<int, int>, int> spoke;
        for (int f : fresh) {
            spoke[{tris[f].v[1], tris[f].v[2]}] = f;  // (b, ep)
            spoke[{tris[f].v[2], tris[f].v[0]}] = f;  // (ep, a)
        }
        for (int f : fresh) {
            auto i = spoke.find({tris[f].v[2], tris[f].v[1]});
            if (i != spoke.end()) tris[f].adj[1] = i->second;
            auto j = spoke.find({tris[f].v[0], tris[f].v[2]});
            if (j != spoke.end()) tris[f].adj[2] = j->second;
        }
        for (int pi : orphans) assign(pi, fresh);
    }
    for (const Tri &t : tris)
        if (t.alive && !t.conflict.empty()) return false;
    return true;
}

// fan normal from the two shortest edges and the vertex average (calculateNormalAndCentroid)
inline void face_normal_centroid(const std::vector<V> &p, const std::vector<int> &loop, V &normal, V &centroid) {
    normal = {0, 0, 0};
    V y0 = p[loop[0]], y1 = p[loop[1]];
    centroid = y0 + y1;
    for (size_t k = 2; k < loop.size(); k++) {
        V y2 = p[loop[k]];
        V e0 = y1 - y0, e1 = y2 - y1, e2 = y0 - y2;
        V nrm = dot(e1, e1) < dot(e2, e2) ? cross(e0, e1) : cross(e2, e0);
        normal = normal + nrm;
        centroid = centroid + y2;
        y1 = y2;
    }
    centroid = centroid * (1.0 / (double)loop.size());
}

// plane3.intersect: the point on three planes (n . x + c = 0); false when they do not meet in one
inline bool intersect3(V n1, double c1, V n2, double c2, V n3, double c3, V &out) {
    V n23 = cross(n2, n3);
    double den = dot(n1, n23);
    if (den == 0.0) return false;
    out = (n23 * (-c1) + cross(n3, n1) * (-c2) + cross(n1, n2) * (-c3)) * (1.0 / den);
    return true;
}

// Builds the hull shape of the input points.  Returns 0 on success, 1 for a degenerate input,
// 2 for more than max_points hull vertices.
inline int build(const std::vector<V> &in, double convex_radius, double hull_tolerance, double max_error_radius,
                 int max_points, Hull &out) {
    std::vector<Tri> tris;
    if (!quickhull(in, hull_tolerance, tris)) return 1;
    std::vector<int> alive;
    for (int f = 0; f < (int)tris.size(); f++)
        if (tris[f].alive) alive.push_back(f);
    // merge neighbouring triangles that lie in one plane (within the tolerance)
    std::vector<int> group(tris.size());
    std::iota(group.begin(), group.end(), 0);
    std::function<int(int)> root = [&](int x) { return group[x] == x ? x : group[x] = root(group[x]); };
    for (int f : alive)
        for (int k = 0; k < 3; k++) {
            int g = tris[f].adj[k];
            if (g < 0 || g < f) continue;
            bool flat = true;
            for (int m = 0; m < 3 && flat; m++) {
                flat = std::fabs(dot(tris[f].n, in[tris[g].v[m]]) - tris[f].d) <= hull_tolerance &&
                       std::fabs(dot(tris[g].n, in[tris[f].v[m]]) - tris[g].d) <= hull_tolerance;
            }
            if (flat && dot(tris[f].n, tris[g].n) > 0) group[root(f)] = root(g);
        }
    // boundary loops of the groups, in the order the faces were made
    std::vector<std::vector<int>> loops;
    std::vector<int> group_ids;
    std::map<int, int> loop_of;
    for (int f : alive) {
        int r = root(f);
        if (loop_of.count(r)) continue;
        loop_of[r] = (int)loops.size();
        std::map<int, int> next;  // boundary edge a -> b
        for (int h : alive) {
            if (root(h) != r) continue;
            for (int k = 0; k < 3; k++) {
                int g = tris[h].adj[k];
                if (g >= 0 && root(g) == r) continue;
                next[tris[h].v[k]] = tris[h].v[(k + 1) % 3];
            }
        }
        // begin the loop at the first vertex of the group's first triangle when it is on the boundary
        int start = next.count(tris[f].v[0]) ? tris[f].v[0] : next.begin()->first;
        std::vector<int> loop = {start};
        for (int guard = 0; guard < (int)next.size(); guard++) {
            int b = next[loop.back()];
            if (b == start) break;
            loop.push_back(b);
        }
        loops.push_back(loop);
    }
    // centre of mass and volume (getCenterOfMassAndVolume)
    std::vector<V> fn(loops.size()), fc(loops.size());
    for (size_t i = 0; i < loops.size(); i++) face_normal_centroid(in, loops[i], fn[i], fc[i]);
    V v4{0, 0, 0};
    for (V c : fc) v4 = v4 + c;
    v4 = v4 * (1.0 / (double)loops.size());
    double vol = 0;
    V com{0, 0, 0};
    for (const auto &lp : loops) {
        V v1 = in[lp[0]], v2 = in[lp[1]];
        for (size_t k = 2; k < lp.size(); k++) {
            V v3 = in[lp[k]];
            double t = dot(v1 - v4, cross(v2 - v4, v3 - v4));
            vol += t;
            com = com + (v1 + v2 + v3 + v4) * t;
            v2 = v3;
        }
    }
    if (vol > 1.1920929e-7)
        com = com * (1.0 / (4.0 * vol));
    else
        com = v4;
    out.volume = vol / 6.0;
    out.com = com;
    // covariance inertia of the fan tetrahedra about the centre of mass (unit density)
    double C[9] = {0};
    const double K[9] = {1.0 / 60, 1.0 / 120, 1.0 / 120, 1.0 / 120, 1.0 / 60, 1.0 / 120, 1.0 / 120, 1.0 / 120, 1.0 / 60};
    for (const auto &lp : loops) {
        V a = in[lp[0]] - com, b = in[lp[1]] - com;
        for (size_t k = 2; k < lp.size(); k++) {
            V c = in[lp[k]] - com;
            double det = a.x * (b.y * c.z - b.z * c.y) - a.y * (b.x * c.z - b.z * c.x) + a.z * (b.x * c.y - b.y * c.x);
            double A[9] = {a.x, b.x, c.x, a.y, b.y, c.y, a.z, b.z, c.z};  // columns a, b, c
            double T[9];
            for (int r = 0; r < 3; r++)
                for (int q = 0; q < 3; q++) T[3 * r + q] = A[3 * r] * K[q] + A[3 * r + 1] * K[3 + q] + A[3 * r + 2] * K[6 + q];
            for (int r = 0; r < 3; r++)
                for (int q = 0; q < 3; q++)
                    C[3 * r + q] += det * (T[3 * r] * A[3 * q] + T[3 * r + 1] * A[3 * q + 1] + T[3 * r + 2] * A[3 * q + 2]);
            b = c;
        }
    }
    double tr = C[0] + C[4] + C[8];
    for (int k = 0; k < 9; k++) out.inertia[k] = (k % 4 == 0 ? tr : 0.0) - C[k];
    // points relative to the centre of mass, in first-use order; faces and planes
    std::map<int, int> remap;
    out.points.clear();
    out.face_first.clear();
    out.face_count.clear();
    out.vidx.clear();
    out.plane_n.clear();
    out.plane_c.clear();
    out.lo = {1e300, 1e300, 1e300};
    out.hi = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < loops.size(); i++) {
        out.face_first.push_back((int)out.vidx.size());
        out.face_count.push_back((int)loops[i].size());
        for (int v : loops[i]) {
            auto it = remap.find(v);
            int idx;
            if (it == remap.end()) {
                V q = in[v] - com;
                idx = (int)out.points.size();
                remap[v] = idx;
                out.points.push_back(q);
                out.lo = {std::min(out.lo.x, q.x), std::min(out.lo.y, q.y), std::min(out.lo.z, q.z)};
                out.hi = {std::max(out.hi.x, q.x), std::max(out.hi.y, q.y), std::max(out.hi.z, q.z)};
            } else {
                idx = it->second;
            }
            out.vidx.push_back(idx);
        }
        V nn = normalize(fn[i]);
        out.plane_n.push_back(nn);
        out.plane_c.push_back(-dot(nn, fc[i] - com));
    }
    if ((int)out.points.size() > max_points) return 2;
    // the faces that best define each point (largest tetrahedron of normals, else the widest
    // pair, else one face)
    int np = (int)out.points.size(), nf = (int)loops.size();
    out.point_faces.assign(np, {0, -1, -1, -1});
    for (int pi = 0; pi < np; pi++) {
        std::vector<int> nb;
        for (int f = 0; f < nf; f++)
            for (int k = 0; k < out.face_count[f]; k++)
                if (out.vidx[out.face_first[f] + k] == pi) {
                    nb.push_back(f);
                    break;
                }
        if (nb.size() < 2) return 1;
        double bigv = 0.05, smallest = std::cos(1.0 * M_PI / 180.0);
        int b3[3] = {-1, -1, -1}, b2[2] = {-1, -1};
        for (size_t a = 0; a < nb.size(); a++)
            for (size_t b = a + 1; b < nb.size(); b++) {
                V c = cross(out.plane_n[nb[a]], out.plane_n[nb[b]]);
                double d = dot(out.plane_n[nb[a]], out.plane_n[nb[b]]);
                if (d < smallest) {
                    smallest = d;
                    b2[0] = nb[a];
                    b2[1] = nb[b];
                }
                for (size_t e = b + 1; e < nb.size(); e++) {
                    double v = std::fabs(dot(c, out.plane_n[nb[e]]));
                    if (v > bigv) {
                        bigv = v;
                        b3[0] = nb[a];
                        b3[1] = nb[b];
                        b3[2] = nb[e];
                    }
                }
            }
        if (b3[0] != -1)
            out.point_faces[pi] = {3, b3[0], b3[1], b3[2]};
        else if (b2[0] != -1)
            out.point_faces[pi] = {2, b2[0], b2[1], -1};
        else
            out.point_faces[pi] = {1, nb[0], -1, -1};
    }
    // convex radius: fit twice into the thinnest direction, and keep sharp vertices within the
    // allowed error
    double r = convex_radius;
    if (r > 0) {
        double min_size = 1e300;
        for (int f = 0; f < nf; f++) {
            double md = 0;
            for (const V &q : out.points) md = std::max(md, -(dot(out.plane_n[f], q) + out.plane_c[f]));
            min_size = std::min(min_size, md);
        }
        r = std::min(r, 0.5 * min_size);
    }
    if (r > 0) {
        for (int pi = 0; pi < np; pi++) {
            const auto &pf = out.point_faces[pi];
            if (pf[0] == 1) continue;
            V n1 = out.plane_n[pf[1]], n2 = out.plane_n[pf[2]], n3;
            V mask{1, 1, 1};
            if (pf[0] == 3) {
                n3 = out.plane_n[pf[3]];
            } else {
                n3 = normalize(cross(n1, n2));
                mask = {1, 1, 0};
            }
            // rows n1, n2, n3; shift = N^-1 mask
            double det = dot(n1, cross(n2, n3));
            if (std::fabs(det) < 1e-12) {
                r = 0;
                break;
            }
            V shift = (cross(n2, n3) * mask.x + cross(n3, n1) * mask.y + cross(n1, n2) * mask.z) * (1.0 / det);
            double off = len(shift);
            if (off > 1) r = std::min(r, max_error_radius / (off - 1));
        }
    }
    out.convex_radius = r;
    double inner = 1e300;
    for (int f = 0; f < nf; f++) inner = std::min(inner, -out.plane_c[f]);
    out.inner_radius = std::max(0.0, inner);
    // points shrunk by the convex radius
    out.shrunk.resize(np);
    for (int pi = 0; pi < np; pi++) {
        const auto &pf = out.point_faces[pi];
        V q = out.points[pi];
        if (pf[0] == 1) {
            out.shrunk[pi] = q - out.plane_n[pf[1]] * r;
            continue;
        }
        V n1 = out.plane_n[pf[1]], n2 = out.plane_n[pf[2]];
        double c1 = -dot(n1, q) + r, c2 = -dot(n2, q) + r;  // planes through q, moved inwards by r
        V n3;
        double c3;
        if (pf[0] == 3) {
            n3 = out.plane_n[pf[3]];
            c3 = -dot(n3, q) + r;
        } else {
            n3 = normalize(cross(n1, n2));
            c3 = -dot(n3, q);
        }
        V s;
        if (!intersect3(n1, c1, n2, c2, n3, c3, s)) s = q - n1 * r;
        out.shrunk[pi] = s;
    }
    return 0;
}

// Principal moments and axes of a symmetric 3x3 inertia tensor by cyclic Jacobi rotations;
// axes are the columns of R (a proper rotation), I = R diag(d) R^T.
inline void principal_axes(const double I[9], double d[3], double R[9]) {
    double a[3][3] = {{I[0], I[1], I[2]}, {I[3], I[4], I[5]}, {I[6], I[7], I[8]}};
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = std::fabs(a[0][1]) + std::fabs(a[0][2]) + std::fabs(a[1][2]);
        if (off < 1e-300) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (std::fabs(a[p][q]) < 1e-300) continue;
                double theta = (a[q][q] - a[p][p]) / (2 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < 3; k++) {  // A = J^T A J
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int k = 0; k < 3; k++) d[k] = a[k][k];
    double det = v[0][0] * (v[1][1] * v[2][2] - v[1][2] * v[2][1]) - v[0][1] * (v[1][0] * v[2][2] - v[1][2] * v[2][0]) +
                 v[0][2] * (v[1][0] * v[2][1] - v[1][1] * v[2][0]);
    if (det < 0)
        for (int k = 0; k < 3; k++) v[k][2] = -v[k][2];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) R[3 * r + c] = v[r][c];
}

}  // namespace cc_hull
