// Host-side triangle mesh construction (src/shapes/utils/triangle-mesh-builder.ts and
// triangle-mesh-bvh.ts), FP64 as the reference computes it:
//   * vertices welded on a 1e-8 grid (deduplicateVertices triangle-mesh-builder.ts:238-262);
//   * triangles whose edge cross product is shorter than the degenerate tolerance dropped
//     (:83-108), the rest with their unit normal, all three edges active;
//   * duplicate triangles dropped, whatever their rotation (:137-185);
//   * active edges: an edge shared by exactly two triangles whose normals are within the cosine
//     threshold is inactive in both (computeActiveEdges :285-335); boundary and non-manifold
//     edges stay active;
//   * a BVH of at most maxLeafTris triangles per leaf, split at the middle of the longest extent
//     of the triangle-bounds centres (BvhSplitStrategy.CENTER triangle-mesh-bvh.ts:590-606),
//     triangles partitioned in place (:924-957), nodes written in pre-order, the right child's
//     offset in the parent (:397-418).  The triangle order the partition leaves is the order
//     of the triangle indices (sub-shape ids) every query reports.
#pragma once

#include <cmath>
#include <cstdint>
#include <map>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace cc_mesh {

struct Mesh {
    std::vector<double> positions;  // x y z per welded vertex
    std::vector<int> tris;          // a b c per triangle
    std::vector<double> normals;    // unit normal per triangle
    std::vector<int> active;        // active-edge bits per triangle: AB 1, BC 2, CA 4
    std::vector<int> material;      // material id per triangle (-1: none)
    std::vector<double> nodes;      // 8 per node: min xyz, max xyz, right child or first
                                    // triangle, split axis or -(count + 1) for a leaf
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // bounds of the root node
};

struct BuildSettings {
    double degenerate_tolerance = 1e-6;
    int max_leaf_tris = 8;
    double active_edge_cos = 0.996195;  // cos 5 degrees (triangle-mesh.ts:98-103)
};

namespace detail {

struct TempNode {
    double lo[3], hi[3];
    int left = -1, right = -1;  // indices into the temp node list (-1: leaf)
    int axis = 0, start = -1, count = 0;
};

inline void swap_tri(Mesh &m, std::vector<double> &bd, int a, int b) {
    if (a == b) return;
    for (int k = 0; k < 3; k++) std::swap(m.tris[3 * a + k], m.tris[3 * b + k]);
    for (int k = 0; k < 3; k++) std::swap(m.normals[3 * a + k], m.normals[3 * b + k]);
    std::swap(m.active[a], m.active[b]);
    std::swap(m.material[a], m.material[b]);
    for (int k = 0; k < 6; k++) std::swap(bd[6 * a + k], bd[6 * b + k]);
}

// buildRecursive triangle-mesh-bvh.ts:433-553 with the CENTER split
inline int build_node(Mesh &m, std::vector<double> &bd, std::vector<TempNode> &nodes, int start, int end,
                      int max_leaf) {
    int id = (int)nodes.size();
    nodes.emplace_back();
    TempNode n;
    double cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    int count = end - start;
    if (count > 0) {
        for (int k = 0; k < 3; k++) {
            double c = bd[6 * start + 2 * k], h = bd[6 * start + 2 * k + 1];
            n.lo[k] = c - h;
            n.hi[k] = c + h;
            cmin[k] = cmax[k] = c;
        }
        for (int i = start + 1; i < end; i++)
            for (int k = 0; k < 3; k++) {
                double c = bd[6 * i + 2 * k], h = bd[6 * i + 2 * k + 1];
                if (c - h < n.lo[k]) n.lo[k] = c - h;
                if (c + h > n.hi[k]) n.hi[k] = c + h;
                if (c < cmin[k]) cmin[k] = c;
                if (c > cmax[k]) cmax[k] = c;
            }
    }
    auto leaf = [&]() {
        n.start = start;
        n.count = count;
        nodes[id] = n;
        return id;
    };
    if (count <= max_leaf) return leaf();
    double ext[3] = {cmax[0] - cmin[0], cmax[1] - cmin[1], cmax[2] - cmin[2]};
    const double MIN_SIZE = 1e-5;
    if (ext[0] < MIN_SIZE && ext[1] < MIN_SIZE && ext[2] < MIN_SIZE) return leaf();
    int axis = (ext[0] >= ext[1] && ext[0] >= ext[2]) ? 0 : (ext[1] >= ext[2] ? 1 : 2);
    double pos = (cmin[axis] + cmax[axis]) / 2;
    // partitionTriangles triangle-mesh-bvh.ts:924-957
    int l = start, r = end - 1;
    while (l <= r) {
        if (bd[6 * l + 2 * axis] < pos) {
            l++;
        } else if (bd[6 * r + 2 * axis] >= pos) {
            r--;
        } else {
            swap_tri(m, bd, l, r);
            l++;
            r--;
        }
    }
    int mid = l;
    if (mid == start || mid == end) return leaf();
    nodes[id] = n;
    int left = build_node(m, bd, nodes, start, mid, max_leaf);
    int right = build_node(m, bd, nodes, mid, end, max_leaf);
    nodes[id].left = left;
    nodes[id].right = right;
    nodes[id].axis = axis;
    return id;
}

// populateBuffer triangle-mesh-bvh.ts:397-418: pre-order, offsets in doubles
inline size_t populate(std::vector<double> &buf, const std::vector<TempNode> &nodes, int id, size_t off) {
    const TempNode &n = nodes[id];
    for (int k = 0; k < 3; k++) {
        buf[off + k] = n.lo[k];
        buf[off + 3 + k] = n.hi[k];
    }
    if (n.left < 0) {
        buf[off + 6] = n.start;
        buf[off + 7] = -(n.count + 1);
        return off + 8;
    }
    size_t left_end = populate(buf, nodes, n.left, off + 8);
    buf[off + 6] = (double)left_end;
    buf[off + 7] = n.axis;
    return populate(buf, nodes, n.right, left_end);
}

}  // namespace detail

// buildTriangleMesh triangle-mesh-builder.ts:62-231
inline Mesh build(const double *positions, int nv, const int *indices, int nt, const int *materials,
                  const BuildSettings &s) {
    Mesh m;
    // deduplicateVertices: weld on a 1e-8 grid (Math.round: halves up), first occurrence wins
    std::vector<int> index_map(nv);
    std::map<std::tuple<double, double, double>, int> weld;
    auto q = [](double v) { return std::floor(v * 1e8 + 0.5) + 0.0; };
    for (int i = 0; i < nv; i++) {
        auto key = std::make_tuple(q(positions[3 * i]), q(positions[3 * i + 1]), q(positions[3 * i + 2]));
        auto it = weld.find(key);
        if (it == weld.end()) {
            int id = (int)(m.positions.size() / 3);
            weld.emplace(key, id);
            for (int k = 0; k < 3; k++) m.positions.push_back(positions[3 * i + k]);
            index_map[i] = id;
        } else {
            index_map[i] = it->second;
        }
    }
    // triangles: drop degenerate ones, normal from the edge cross product
    struct Tri {
        int a, b, c, mat;
        double n[3];
    };
    std::vector<Tri> tris;
    for (int t = 0; t < nt; t++) {
        int a = index_map[indices[3 * t]], b = index_map[indices[3 * t + 1]], c = index_map[indices[3 * t + 2]];
        const double *pa = &m.positions[3 * a], *pb = &m.positions[3 * b], *pc = &m.positions[3 * c];
        double e1[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
        double e2[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
        double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        if (len < s.degenerate_tolerance) continue;
        double inv = 1.0 / std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        tris.push_back({a, b, c, materials ? materials[t] : -1, {cr[0] * inv, cr[1] * inv, cr[2] * inv}});
    }
    // duplicates: rotate the lowest index first (winding kept), then (a, b, c, material)
    std::map<std::tuple<int, int, int, int>, int> seen;
    for (const Tri &t : tris) {
        int a = t.a, b = t.b, c = t.c, ca, cb, cc;
        if (a < b) {
            if (a < c) {
                ca = a, cb = b, cc = c;
            } else {
                ca = c, cb = a, cc = b;
            }
        } else {
            if (b < c) {
                ca = b, cb = c, cc = a;
            } else {
                ca = c, cb = a, cc = b;
            }
        }
        if (!seen.emplace(std::make_tuple(ca, cb, cc, t.mat), 1).second) continue;
        m.tris.insert(m.tris.end(), {t.a, t.b, t.c});
        m.normals.insert(m.normals.end(), {t.n[0], t.n[1], t.n[2]});
        m.active.push_back(0b111);
        m.material.push_back(t.mat);
    }
    const int count = (int)m.active.size();
    // computeActiveEdges triangle-mesh-builder.ts:285-335
    if (s.active_edge_cos >= 0.0) {
        struct Refs {
            int count = 0, t0 = 0, t1 = 0;
        };
        std::unordered_map<int64_t, Refs> edges;
        std::vector<int64_t> order;  // edges in first-seen order (phase 2 visits them in that order)
        for (int t = 0; t < count; t++) {
            const int v[3] = {m.tris[3 * t], m.tris[3 * t + 1], m.tris[3 * t + 2]};
            for (int e = 0; e < 3; e++) {
                int ia = v[e], ib = v[(e + 1) % 3], bit = 1 << e;
                int64_t key = (int64_t)std::min(ia, ib) * 67108864LL + std::max(ia, ib);
                auto it = edges.find(key);
                if (it == edges.end()) {
                    Refs r;
                    r.count = 1;
                    r.t0 = (t << 3) | bit;
                    edges.emplace(key, r);
                    order.push_back(key);
                } else if (it->second.count == 1) {
                    it->second.t1 = (t << 3) | bit;
                    it->second.count = 2;
                } else {
                    m.active[t] |= bit;  // third triangle on the edge: non-manifold, active
                    it->second.count++;
                }
            }
        }
        for (int64_t key : order) {
            const Refs &r = edges[key];
            if (r.count != 2) continue;
            int t0 = r.t0 >> 3, b0 = r.t0 & 7, t1 = r.t1 >> 3, b1 = r.t1 & 7;
            double d = m.normals[3 * t0] * m.normals[3 * t1] + m.normals[3 * t0 + 1] * m.normals[3 * t1 + 1] +
                       m.normals[3 * t0 + 2] * m.normals[3 * t1 + 2];
            if (d >= s.active_edge_cos) {
                m.active[t0] &= ~b0;
                m.active[t1] &= ~b1;
            }
        }
    }
    if (count == 0) return m;
    // BVH (triangle-mesh-bvh.ts:368-392): triangle bounds as (centre, half extent) per axis
    std::vector<double> bd(6 * (size_t)count);
    for (int t = 0; t < count; t++) {
        for (int k = 0; k < 3; k++) {
            double a = m.positions[3 * m.tris[3 * t] + k], b = m.positions[3 * m.tris[3 * t + 1] + k],
                   c = m.positions[3 * m.tris[3 * t + 2] + k];
            double mn = a, mx = a;
            if (b < mn) mn = b;
            if (c < mn) mn = c;
            if (b > mx) mx = b;
            if (c > mx) mx = c;
            bd[6 * t + 2 * k] = (mn + mx) * 0.5;
            bd[6 * t + 2 * k + 1] = (mx - mn) * 0.5;
        }
    }
    std::vector<detail::TempNode> nodes;
    nodes.reserve(2 * (size_t)count);
    int root = detail::build_node(m, bd, nodes, 0, count, s.max_leaf_tris);
    m.nodes.assign(8 * nodes.size(), 0.0);
    detail::populate(m.nodes, nodes, root, 0);
    for (int k = 0; k < 3; k++) {
        m.lo[k] = m.nodes[k];
        m.hi[k] = m.nodes[3 + k];
    }
    return m;
}

// subShape.pushIndex sub-shape.ts:60-64 on an empty id: the low ceil(log2(count)) bits hold the
// triangle index, the others stay set
inline uint32_t triangle_sub_shape_id(int tri, int count) {
    uint32_t max_index = (uint32_t)(count - 1);
    int bits = max_index == 0 ? 0 : 32 - __builtin_clz(max_index);
    uint32_t mask = bits >= 32 ? 0xffffffffu : ((1u << bits) - 1u);
    return (0xffffffffu & ~mask) | (uint32_t)tri;
}

}  // namespace cc_mesh
