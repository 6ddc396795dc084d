// Contact constraints, contact cache, islands and the island-partitioned
// sequential-impulse solver with integration and sleeping fused in.
//
// Reference: addContactConstraint (src/constraints/contact-constraints.ts:437-857),
// the contact cache (src/contacts.ts), islands (src/islands.ts), the solver
// loops of updateWorld (src/update.ts:101-233), warm start / velocity /
// position solve (contact-constraints.ts:906-1216, constraint-part/
// axis-constraint-part.ts:500-847), velocityIntegrationUpdate
// (update.ts:896-976) and island sleeping (islands.ts:392-423, body/sleep.ts).
//
// Islands are independent, so each is solved to completion by one owner:
//  * islands with few contacts: one thread runs the reference's sequential
//    Gauss-Seidel order exactly (contacts sorted by (sortKey, A, B));
//  * larger islands: one CTA sorts the contacts the same way, colours them
//    greedily in that order (min rank claims a body first) and sweeps the
//    colours in parallel.
// After the velocity iterations the owner stores impulses into the cache,
// integrates its bodies, runs the position iterations, derives positions and
// decides sleeping for the island - the integration and sleep test are fused
// into the last solver pass.
#include <math_constants.h>

#include "cc_internal.cuh"
#include "cc_swing.cuh"

namespace cc {

static __constant__ DevSettings c_settings;

void upload_settings_solver(const DevSettings &s, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(c_settings, &s, sizeof(DevSettings), 0, cudaMemcpyHostToDevice, st);
}

constexpr int SMALL_ISLAND_MAX_CONS = 64;  // upper bound of the per-thread class (register arrays)
constexpr int SMALL_ISLAND_MAX_BODIES = 64;
constexpr int SMALL_ISLAND_MAX_JOINTS = 16;  // bound of the per-thread class's joint list (register array)
// islands above the per-thread class and within these limits run on one warp
constexpr int WARP_MAX_CONS = 256;
constexpr int WARP_MAX_BODIES = 128;
// The per-warp tier in two instances: islands of at most 32 contacts and 48 bodies (nearly all of
// them) with a small shared-memory footprint, so that more warps fit on an SM, and the rest.
constexpr int WARP_S_CONS = 32, WARP_S_BODIES = 48;
constexpr int WARP_MAX_COLOURS = 64;  // colours past this one are swept by one lane in order

struct CacheTables {
    unsigned long long *keys[2];
    CacheRecord *recs[2];
    int *parity;
};

__device__ __forceinline__ unsigned int hash64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (unsigned int)k;
}

__device__ int cache_find(const unsigned long long *keys, int cap, unsigned long long key) {
    unsigned int mask = (unsigned)cap - 1u;
    unsigned int h = hash64(key) & mask;
    for (int probe = 0; probe < cap; probe++) {
        unsigned long long k = keys[h];
        if (k == key) return (int)h;
        if (k == EMPTY_KEY) return -1;
        h = (h + 1u) & mask;
    }
    return -1;
}
__device__ int cache_insert(unsigned long long *keys, int cap, unsigned long long key) {
    unsigned int mask = (unsigned)cap - 1u;
    unsigned int h = hash64(key) & mask;
    for (int probe = 0; probe < cap; probe++) {
        unsigned long long prev = atomicCAS(&keys[h], EMPTY_KEY, key);
        if (prev == EMPTY_KEY || prev == key) return (int)h;
        h = (h + 1u) & mask;
    }
    return -1;
}

// combineMaterial combine-material.ts:40-57
__device__ float combine(float a, float b, int ma, int mb) {
    const int prio[5] = {0, 1, 3, 4, 2};
    int mode = prio[ma] >= prio[mb] ? ma : mb;
    switch (mode) {
        case 1:
            return a * b;
        case 2:
            return fminf(a, b);
        case 3:
            return fmaxf(a, b);
        case 4:
            return sqrtf(a * b);
        default:
            return (a + b) * 0.5f;
    }
}

// computeContactSortKey contact-constraints.ts:1222-1231
__device__ uint32_t contact_sort_key(int a, int b, uint32_t sa, uint32_t sb) {
    uint32_t h = 0;
    h = h * 31u + (uint32_t)a;
    h = h * 31u + (uint32_t)b;
    h = h * 31u + sa;
    h = h * 31u + sb;
    return h;
}

__device__ __forceinline__ Sym3 load_sym(const float4 *iw, int i) {
    float4 a = iw[2 * i], b = iw[2 * i + 1];
    return Sym3{a.x, a.y, a.z, a.w, b.x, b.y};
}

// inverse effective mass of one axis (calculateInverseEffectiveMass, axis-constraint-part.ts:86-148)
__device__ __forceinline__ float inv_eff_mass(bool dynA, bool dynB, float imA, float imB, const Sym3 &IA,
                                              const Sym3 &IB, float3 rA, float3 rB, float3 ax) {
    float iem = 0.f;
    if (dynA) {
        float3 c = cross3(rA, ax);
        iem += imA + dot3(symmul(IA, c), c);
    }
    if (dynB) {
        float3 c = cross3(rB, ax);
        iem += imB + dot3(symmul(IB, c), c);
    }
    return iem;
}

// ---------------------------------------------------------------------------
// Contact cache key (the contact's (idA, idB, subShapeIdA, subShapeIdB), contacts.ts:481-513):
// (A << 32) | B for convex pairs; with a sub-shape (a mesh triangle, a compound child), bit 63
// set and A, B and the sub-shape indices in 21 bits each.  The indices are the low bits of the
// sub-shape ids (the triangle's, the child's), packed side by side while they fit in 21 bits
// (a mesh of up to 2^21 triangles, or a compound of 2^k children against a mesh of up to
// 2^(21-k)); past that they are folded into 21 bits by a multiplicative hash.
__device__ __forceinline__ int sub_index_bits(const DevWorld &w, int body) {
    const int s = shape_of(w.flags[body]);
    if (s == SHAPE_MESH) return w.meshes[mesh_of(w.shape[body])].sub_bits;
    if (s == SHAPE_COMPOUND) return w.compounds[compound_of(w.shape[body])].sub_bits;
    return 0;
}
__device__ __forceinline__ unsigned long long contact_key(const DevWorld &w, int A, int B, uint32_t subA,
                                                          uint32_t subB) {
    if (subA == 0xffffffffu && subB == 0xffffffffu)
        return ((unsigned long long)(unsigned)A << 32) | (unsigned)B;
    const int ba = subA != 0xffffffffu ? sub_index_bits(w, A) : 0;
    const int bb = subB != 0xffffffffu ? sub_index_bits(w, B) : 0;
    auto low = [](uint32_t sub, int bits) { return bits >= 32 ? sub : (sub & ((1u << bits) - 1u)); };
    const unsigned long long M = (1ull << MESH_KEY_BITS) - 1ull;
    unsigned long long idx;
    if (ba + bb <= MESH_KEY_BITS)
        idx = ((unsigned long long)low(subA, ba) << bb) | low(subB, bb);
    else
        idx = ((unsigned long long)(subA * 0x9E3779B1u ^ subB * 0x85EBCA77u)) >> (32 - MESH_KEY_BITS);
    return (1ull << 63) | (((unsigned long long)A & M) << 42) | (((unsigned long long)B & M) << 21) | (idx & M);
}

// contact setup: one manifold per thread
// ---------------------------------------------------------------------------
__global__ void k_contact_setup(DevWorld w, CacheTables ct, float dt) {
    int par = *ct.parity;
    const unsigned long long *pkeys = ct.keys[par ^ 1];
    const CacheRecord *precs = ct.recs[par ^ 1];
    unsigned long long *ckeys = ct.keys[par];
    CacheRecord *crecs = ct.recs[par];
    int nm = min(w.ctr->num_manifolds, w.max_manifolds);
    for (int mi = blockIdx.x * blockDim.x + threadIdx.x; mi < nm; mi += gridDim.x * blockDim.x) {
        Manifold m = w.manifolds[mi];
        float3 base = m.base;
        int A = m.a, B = m.b;
        uint32_t subA = m.sub_a, subB = m.sub_b;
        float3 nrm = m.normal;
        float3 ra[4], rb[4];
        for (int k = 0; k < 4; k++) {
            ra[k] = m.ra[k];
            rb[k] = m.rb[k];
        }
        if (A > B) {  // ids grow with the body index: order by id (contact-constraints.ts:448-453)
            int t = A;
            A = B;
            B = t;
            uint32_t ts = subA;
            subA = subB;
            subB = ts;
            nrm = -nrm;
            for (int k = 0; k < 4; k++) {
                float3 tt = ra[k];
                ra[k] = rb[k];
                rb[k] = tt;
            }
        }
        unsigned long long key = contact_key(w, A, B, subA, subB);
        int prev = cache_find(pkeys, w.cache_cap, key);
        int slot = cache_insert(ckeys, w.cache_cap, key);
        if (slot < 0) {
            atomicOr(&w.ctr->overflow, OVF_CACHE);
            continue;
        }
        // onContactPersisted / onContactAdded (contact-constraints.ts:494-499), sensors included
        w.contact_event[mi] = prev >= 0 ? 2 : 1;
        uint32_t fa = w.flags[A], fb = w.flags[B];
        int ma = motion_of(fa), mb = motion_of(fb);
        float4 qa = w.quat[A], qb = w.quat[B];
        float3 comA = xyz(w.com[A]) - base, comB = xyz(w.com[B]) - base;
        Mat3 RA = quat_to_mat(qa), RB = quat_to_mat(qb);
        float4 ia = w.inv_inertia[A], ib = w.inv_inertia[B];
        float4 mta = w.material[A], mtb = w.material[B];
        float friction = combine(mta.x, mtb.x, (fa >> F_FCOMB_SHIFT) & 7, (fb >> F_FCOMB_SHIFT) & 7);
        float restitution = combine(mta.y, mtb.y, (fa >> F_RCOMB_SHIFT) & 7, (fb >> F_RCOMB_SHIFT) & 7);
        bool sensor = ((fa | fb) & F_SENSOR) != 0;
        CacheRecord rec;
        rec.key = key;
        rec.n = m.n;
        rec.pad = 0;
        bool creates = !sensor && ((ma == DYNAMIC && ia.w != 0.f) || (mb == DYNAMIC && ib.w != 0.f));
        if (!creates) {
            for (int k = 0; k < m.n; k++) {
                rec.p1[k] = mtmul(RA, ra[k] - comA);
                rec.p2[k] = mtmul(RB, rb[k] - comB);
                rec.ln[k] = rec.lt1[k] = rec.lt2[k] = 0.f;
            }
            crecs[slot] = rec;
            continue;
        }
        int ci = mi;  // one constraint slot per manifold
        ContactConstraint c;
        c.a = A;
        c.b = B;
        c.n = m.n;
        c.island = -1;
        c.normal = nrm;
        c.friction = friction;
        if (fabsf(nrm.x) > fabsf(nrm.y)) {
            float tl = sqrtf(nrm.x * nrm.x + nrm.z * nrm.z);
            c.t1 = f3(nrm.z / tl, 0.f, -nrm.x / tl);
        } else {
            float tl = sqrtf(nrm.y * nrm.y + nrm.z * nrm.z);
            c.t1 = f3(0.f, nrm.z / tl, -nrm.y / tl);
        }
        c.t2 = cross3(nrm, c.t1);
        c.invMassA = ia.w;
        c.invMassB = ib.w;
        c.sort_key = contact_sort_key(A, B, subA, subB);
        c.cache_slot = slot;
        c.pad0 = prev;  // record of the previous step's table this contact was matched with (-1: none)
        c.pad1 = 0;
        bool dynA = ma == DYNAMIC, dynB = mb == DYNAMIC;
        Sym3 IA{0, 0, 0, 0, 0, 0}, IB{0, 0, 0, 0, 0, 0};
        if (dynA) IA = world_inv_inertia(qa, w.inertia_rot[A], xyz(ia), dof_of(fa));
        if (dynB) IB = world_inv_inertia(qb, w.inertia_rot[B], xyz(ib), dof_of(fb));
        float4 va = w.linvel[A], wa = w.angvel[A], vb = w.linvel[B], wb = w.angvel[B];
        float3 g = f3(c_settings.gravity[0], c_settings.gravity[1], c_settings.gravity[2]);
        const CacheRecord *pr = prev >= 0 ? &precs[prev] : nullptr;
        int pn = pr ? pr->n : 0;
        for (int k = 0; k < m.n; k++) {
            ContactPoint &p = c.p[k];
            float3 pa = ra[k], pb = rb[k];
            p.localA = mtmul(RA, pa - comA);
            p.localB = mtmul(RB, pb - comB);
            p.lam_n = p.lam_t1 = p.lam_t2 = 0.f;
            int matched = -1;
            for (int j = 0; j < pn; j++) {
                float3 d1 = p.localA - pr->p1[j], d2 = p.localB - pr->p2[j];
                float th = c_settings.preserve_lambda_dsq;
                if (lensq3(d1) < th && lensq3(d2) < th) {
                    p.lam_n = pr->ln[j];
                    p.lam_t1 = pr->lt1[j];
                    p.lam_t2 = pr->lt2[j];
                    matched = j;
                    break;
                }
            }
            float3 mid = (pa + pb) * 0.5f;
            p.rA = mid - comA;
            p.rB = mid - comB;
            // calculateNormalVelocityBias contact-constraints.ts:288-423
            bool aM = ma != STATIC, bM = mb != STATIC;
            float3 v1 = xyz(va) + cross3(xyz(wa), p.rA);
            float3 v2 = xyz(vb) + cross3(xyz(wb), p.rB);
            float3 rv = aM && bM ? v2 - v1 : (aM ? -v1 : (bM ? v2 : f3(0.f, 0.f, 0.f)));
            float nv = dot3(rv, nrm);
            float pen = dot3(pa - pb, nrm);
            float spec = fmaxf(0.f, -pen / dt);
            float bias = spec;
            if (restitution > 0.f && nv < -c_settings.min_vel_restitution && nv < -spec) {
                float3 rel = f3(0.f, 0.f, 0.f);
                if (aM && bM)
                    rel = g * (mtb.z - mta.z);
                else if (aM)
                    rel = g * (-mta.z);
                else if (bM)
                    rel = g * mtb.z;
                if (dynA) rel = rel + xyz(w.force[A]) * (-ia.w);
                if (dynB) rel = rel + xyz(w.force[B]) * ib.w;
                float fdv = fminf(0.f, dot3(rel, nrm) * dt);
                bias = restitution * (nv - fdv);
            }
            p.bias_n = bias;
            float iem = inv_eff_mass(dynA, dynB, c.invMassA, c.invMassB, IA, IB, p.rA, p.rB, nrm);
            if (iem == 0.f) {
                p.eff_n = 0.f;
                p.lam_n = 0.f;
            } else {
                p.eff_n = 1.f / iem;
            }
            if (friction > 0.f) {
                float i1 = inv_eff_mass(dynA, dynB, c.invMassA, c.invMassB, IA, IB, p.rA, p.rB, c.t1);
                float i2 = inv_eff_mass(dynA, dynB, c.invMassA, c.invMassB, IA, IB, p.rA, p.rB, c.t2);
                if (i1 == 0.f) {
                    p.eff_t1 = 0.f;
                    p.lam_t1 = 0.f;
                } else {
                    p.eff_t1 = 1.f / i1;
                }
                if (i2 == 0.f) {
                    p.eff_t2 = 0.f;
                    p.lam_t2 = 0.f;
                } else {
                    p.eff_t2 = 1.f / i2;
                }
            } else {
                p.eff_t1 = p.eff_t2 = 0.f;
                p.lam_t1 = p.lam_t2 = 0.f;
            }
            p.pad = __int_as_float(matched);  // cached point that warm-started this one (-1: none)
            rec.p1[k] = p.localA;
            rec.p2[k] = p.localB;
            rec.ln[k] = p.lam_n;
            rec.lt1[k] = p.lam_t1;
            rec.lt2[k] = p.lam_t2;
        }
        crecs[slot] = rec;
        w.cons[ci] = c;
        w.cons_of_manifold[mi] = ci;
        atomicAdd(&w.ctr->num_points, m.n);
        if (ma == DYNAMIC && sleeping_of(fa)) w.wake[A] = 1;
        if (mb == DYNAMIC && sleeping_of(fb)) w.wake[B] = 1;
    }
}

// sleep test points (getSleepTestPoints sleep.ts:22-74)
__device__ void sleep_points(const DevWorld &w, int i, uint32_t f, float4 sp, float4 q, float3 com, float3 out[3]) {
    int sh = shape_of(f);
    float3 e = sh == SHAPE_BOX ? f3(sp.x, sp.y, sp.z)
                               : (sh == SHAPE_CAPSULE ? f3(sp.x, sp.y + sp.x, sp.x) : f3(sp.x, sp.x, sp.x));
    if (sh == SHAPE_CYLINDER) e = f3(sp.y, sp.x, sp.y);
    if (sh == SHAPE_HULL) {  // half extents of the hull's bounds
        const DevHull &h = w.hulls[hull_of(sp)];
        e = f3(0.5f * (h.hi.x - h.lo.x), 0.5f * (h.hi.y - h.lo.y), 0.5f * (h.hi.z - h.lo.z));
    }
    if (f & F_DECORATED) {  // half extents of the decorated shape's bounds
        const DevFrame &d = w.frames[i];
        e = f3((float)(0.5 * (d.hi[0] - d.lo[0])), (float)(0.5 * (d.hi[1] - d.lo[1])), (float)(0.5 * (d.hi[2] - d.lo[2])));
    }
    out[0] = com;
    int lowest = (e.x <= e.y && e.x <= e.z) ? 0 : (e.y <= e.z ? 1 : 2);
    float3 X = f3(1.f, 0.f, 0.f), Y = f3(0.f, 1.f, 0.f), Z = f3(0.f, 0.f, 1.f);
    if (lowest == 0) {
        out[1] = com + qrot(q, Y) * e.y;
        out[2] = com + qrot(q, Z) * e.z;
    } else if (lowest == 1) {
        out[1] = com + qrot(q, X) * e.x;
        out[2] = com + qrot(q, Z) * e.z;
    } else {
        out[1] = com + qrot(q, X) * e.x;
        out[2] = com + qrot(q, Y) * e.y;
    }
}
__device__ void reset_sleep(DevWorld &w, int i) {
    float3 p[3];
    sleep_points(w, i, w.flags[i], w.shape[i], w.quat[i], xyz(w.com[i]), p);
    for (int k = 0; k < 3; k++) w.sleep_sph[3 * i + k] = make_float4(p[k].x, p[k].y, p[k].z, 0.f);
    w.sleep_timer[i] = 0.f;
}

// wake bodies touched by a new contact constraint (update.ts:84-91, sleep.ts:186-203)
__global__ void k_apply_wake(DevWorld w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        if (!w.wake[i]) continue;
        w.wake[i] = 0;
        w.flags[i] &= ~F_SLEEPING;
        reset_sleep(w, i);
    }
}

// ---------------------------------------------------------------------------
// islands: union-find over contact constraints between active bodies
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool active_body(uint32_t f) { return motion_of(f) != STATIC && !sleeping_of(f); }

// Union-find root with path splitting.  Parent links written by other CTAs
// must be seen while linking, so loads bypass L1 (__ldcg) and stores go to L2
// (__stcg); a plain load could keep returning a stale L1 line, making a CAS
// retry loop spin on a root that was already hooked elsewhere.
__device__ int uf_find(int *parent, int i) {
    while (true) {
        int p = __ldcg(&parent[i]);
        if (p == i) return i;
        int gp = __ldcg(&parent[p]);
        if (gp != p) __stcg(&parent[i], gp);  // path splitting
        i = p;
    }
}

__global__ void k_uf_init(DevWorld w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        w.uf_parent[i] = i;
        w.island_body_count[i] = 0;
        w.island_cons_count[i] = 0;
        w.island_fill_b[i] = 0;
        w.island_fill_c[i] = 0;
        w.island_iters[3 * i] = w.island_iters[3 * i + 1] = w.island_iters[3 * i + 2] = 0;
        if (w.island_joint_count) {
            w.island_joint_count[i] = 0;
            w.island_fill_j[i] = 0;
        }
        if (w.ccd_flag) w.ccd_flag[i] = 0;
    }
}

// A union-find link that gave up leaves islands that may share bodies; the solve tiers then
// skip the step rather than let two islands' solvers touch one body (the host reports
// CC_ERR_CAPACITY for the step).
__device__ __forceinline__ bool islands_failed(const DevWorld &w) {
    return (*(volatile int *)&w.ctr->overflow & OVF_ISLAND) != 0;
}

// union of the sets of two bodies (bounded retry; gives up with an overflow flag)
__device__ void uf_union(DevWorld &w, int a, int b) {
    for (int guard = 0; guard < c_settings.link_attempts; guard++) {
        int ra = uf_find(w.uf_parent, a), rb = uf_find(w.uf_parent, b);
        if (ra == rb) return;
        int hi = max(ra, rb), lo = min(ra, rb);
        if (atomicCAS(&w.uf_parent[hi], hi, lo) == hi) return;
    }
    atomicOr(&w.ctr->overflow, OVF_ISLAND);  // bounded retry gave up: report it
}

// contacts between active bodies (islands.ts:103-140) and enabled joints between
// active bodies (linkUserConstraints islands.ts:209-224) join their bodies' islands
__global__ void k_uf_link(DevWorld w) {
    int nm = min(w.ctr->num_manifolds, w.max_manifolds);
    for (int ci = blockIdx.x * blockDim.x + threadIdx.x; ci < nm; ci += gridDim.x * blockDim.x) {
        if (w.cons_of_manifold[ci] < 0) continue;
        int a = w.cons[ci].a, b = w.cons[ci].b;
        if (!active_body(w.flags[a]) || !active_body(w.flags[b])) continue;
        uf_union(w, a, b);
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < joint_total(w); k += gridDim.x * blockDim.x) {
        const DevJointHead &h = joint_head(w, joint_id_at(w, k));
        if (!(h.flags & JF_ENABLED)) continue;
        if (!active_body(w.flags[h.a]) || !active_body(w.flags[h.b])) continue;
        uf_union(w, h.a, h.b);
    }
}

__global__ void k_uf_roots(DevWorld w, int *root_flag) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        bool act = active_body(w.flags[i]);
        int r = act ? uf_find(w.uf_parent, i) : -1;
        w.uf_parent[i] = r;
        root_flag[i] = (act && r == i) ? 1 : 0;
    }
}

// a body's or joint's iteration overrides joining its island's (islands.ts:350-375)
__device__ __forceinline__ void add_iteration_overrides(DevWorld &w, int isl, uint32_t ovr) {
    int v = (int)(ovr & 0xffu), p = (int)((ovr >> 8) & 0xffu);
    int *s = w.island_iters + 3 * (size_t)isl;
    if (v > 0) atomicMax(&s[0], v);
    if (p > 0) atomicMax(&s[1], p);
    int f = (v == 0 ? 1 : 0) | (p == 0 ? 2 : 0);
    if (f) atomicOr(&s[2], f);
}

__global__ void k_island_count(DevWorld w, const int *island_id_of_root) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        int r = w.uf_parent[i];
        int isl = r >= 0 ? island_id_of_root[r] : -1;
        w.island_of_body[i] = isl;
        if (isl >= 0) {
            atomicAdd(&w.island_body_count[isl], 1);
            if (motion_of(w.flags[i]) == DYNAMIC) add_iteration_overrides(w, isl, w.iter_ovr[i]);
        }
    }
    int nm = min(w.ctr->num_manifolds, w.max_manifolds);
    for (int ci = blockIdx.x * blockDim.x + threadIdx.x; ci < nm; ci += gridDim.x * blockDim.x) {
        if (w.cons_of_manifold[ci] < 0) continue;
        int a = w.cons[ci].a, b = w.cons[ci].b;
        int owner = active_body(w.flags[a]) ? a : b;
        int r = w.uf_parent[owner];
        int isl = r >= 0 ? island_id_of_root[r] : -1;
        w.cons[ci].island = isl;
        if (isl >= 0) atomicAdd(&w.island_cons_count[isl], 1);
    }
    // a joint belongs to the island of its lower active body (islands.ts:163-178, 318-332)
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < joint_total(w); k += gridDim.x * blockDim.x) {
        DevJointHead &h = joint_head(w, joint_id_at(w, k));
        int isl = -1;
        if (h.flags & JF_ENABLED) {
            bool aa = active_body(w.flags[h.a]), ab = active_body(w.flags[h.b]);
            if (aa || ab) {
                int r = w.uf_parent[aa ? h.a : h.b];
                isl = r >= 0 ? island_id_of_root[r] : -1;
            }
        }
        h.island = isl;
        if (isl >= 0) {
            atomicAdd(&w.island_joint_count[isl], 1);
            add_iteration_overrides(w, isl, (uint32_t)h.iter_ovr);
        }
    }
}

__global__ void k_island_scatter(DevWorld w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        int isl = w.island_of_body[i];
        if (isl < 0) continue;
        int k = atomicAdd(&w.island_fill_b[isl], 1);
        w.island_bodies[w.island_body_off[isl] + k] = i;
    }
    int nm = min(w.ctr->num_manifolds, w.max_manifolds);
    for (int ci = blockIdx.x * blockDim.x + threadIdx.x; ci < nm; ci += gridDim.x * blockDim.x) {
        if (w.cons_of_manifold[ci] < 0) continue;
        int isl = w.cons[ci].island;
        if (isl < 0) continue;
        int k = atomicAdd(&w.island_fill_c[isl], 1);
        w.island_cons[w.island_cons_off[isl] + k] = ci;
    }
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < joint_total(w); k += gridDim.x * blockDim.x) {
        int id = joint_id_at(w, k);
        int isl = joint_head(w, id).island;
        if (isl < 0) continue;
        int f = atomicAdd(&w.island_fill_j[isl], 1);
        w.island_joints[w.island_joint_off[isl] + f] = id;
    }
}

// split islands into the per-thread and per-CTA classes
// the per-warp tier's size class of an island of nc contacts: 9-16 -> 0, 17-32 -> 1, ... 129-256 -> 4
__device__ __forceinline__ int mid_size_class(int nc) { return 31 - __clz(max(nc - 1, 1)) - 3; }

// Entry k of a bucketed island list, the buckets taken from the last (largest islands) down;
// -1 past the end.
__device__ __forceinline__ int bucketed_island(const int *list, size_t cap, const int *counts, int nbuckets, int k) {
    for (int b = nbuckets - 1; b >= 0; b--) {
        const int c = counts[b];
        if (k < c) return list[(size_t)b * cap + k];
        k -= c;
    }
    return -1;
}

// Island classes of k_island_classify: a per-thread or per-warp size bucket, or one of these.
enum : int { CL_NONE = -1, CL_MID0 = 100, CL_GIANT = 1000, CL_SMALL_JOINT, CL_LARGE_JOINT, CL_LARGE };

__global__ void k_island_classify(DevWorld w, int *small_list, int *large_list) {
    const int ni = w.ctr->num_islands;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // the lanes of a warp stay together through the loop: the list slots are taken with one
    // atomic per class present in the warp
    for (int base = blockIdx.x * blockDim.x; base < ni; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        int cls = CL_NONE, tot = 0;
        if (i < ni) {
            const int nc = w.island_cons_count[i], nb = w.island_body_count[i];
            const int nj = joint_total(w) > 0 ? w.island_joint_count[i] : 0;
            tot = nc + nj;
            if (nc + nj > w.giant_min) {  // a pile: the whole grid solves it
                cls = CL_GIANT;
            } else if (nj > 0) {
                // islands with joints: one thread in the reference's exact order when small (a lone
                // ragdoll), else the per-CTA solve
                cls = (nj <= c_settings.small_island_max_joints && nc <= SMALL_ISLAND_MAX_CONS &&
                       nb <= SMALL_ISLAND_MAX_BODIES)
                          ? CL_SMALL_JOINT
                          : CL_LARGE_JOINT;
            } else if (nc <= c_settings.small_island_max_cons && nb <= SMALL_ISLAND_MAX_BODIES) {
                cls = min(nc, SMALL_BUCKETS - 1);
            } else if (nc <= WARP_MAX_CONS && nb <= WARP_MAX_BODIES) {
                // classes 0 and 1 (at most 32 contacts) go to the small instance when their bodies fit
                int b = min(max(mid_size_class(nc), 0), MID_BUCKETS - 1);
                if (b < 2 && nb > WARP_S_BODIES) b = 2;
                cls = CL_MID0 + b;
            } else {
                cls = CL_LARGE;
            }
        }
        const int mx = __reduce_max_sync(FULL, tot);
        if (lane == 0 && mx > 0) atomicMax(&w.ctr->max_island_constraints, mx);
        const unsigned same = __match_any_sync(FULL, cls);
        const int leader = __ffs(same) - 1, cnt = __popc(same);
        int *ctr = nullptr, *list = nullptr, *total = nullptr;
        if (cls == CL_GIANT) {
            ctr = &w.ctr->num_giant_islands;
            list = w.giant_list;
        } else if (cls == CL_SMALL_JOINT) {
            ctr = &w.ctr->num_small_joint_islands;
            list = w.small_joint_list;
        } else if (cls == CL_LARGE_JOINT) {
            ctr = &w.ctr->num_large_joint_islands;
            list = w.large_joint_list;
        } else if (cls == CL_LARGE) {
            ctr = &w.ctr->num_large_islands;
            list = large_list;
        } else if (cls >= CL_MID0) {
            ctr = &w.ctr->mid_bucket[cls - CL_MID0];
            list = w.mid_list + (size_t)(cls - CL_MID0) * w.cap;
            total = &w.ctr->num_mid_islands;
        } else if (cls >= 0) {
            ctr = &w.ctr->small_bucket[cls];
            list = small_list + (size_t)cls * w.cap;
            total = &w.ctr->num_small_islands;
        }
        int slot = 0;
        if (ctr && lane == leader) {
            slot = atomicAdd(ctr, cnt);
            if (total) atomicAdd(total, cnt);
        }
        slot = __shfl_sync(same, slot, leader);
        if (ctr) list[slot + __popc(same & ((1u << lane) - 1u))] = i;
    }
}

// ---------------------------------------------------------------------------
// solver primitives (FP32), body velocities in global memory
// ---------------------------------------------------------------------------
struct BodyRef {
    float3 v, w;
    float im;
    Sym3 I;
    int motion;
    int dof;
};
__device__ __forceinline__ BodyRef load_body(const DevWorld &w, int i) {
    BodyRef b;
    float4 v = w.linvel[i], av = w.angvel[i];
    uint32_t f = w.flags[i];
    b.v = xyz(v);
    b.w = xyz(av);
    b.im = w.inv_inertia[i].w;
    b.motion = motion_of(f);
    b.dof = dof_of(f);
    if (b.motion == DYNAMIC)
        b.I = load_sym(w.inv_inertia_world, i);
    else
        b.I = Sym3{0, 0, 0, 0, 0, 0};
    return b;
}
__device__ __forceinline__ void store_body_vel(DevWorld &w, int i, const BodyRef &b) {
    if (b.motion != DYNAMIC) return;
    w.linvel[i] = make_float4(b.v.x, b.v.y, b.v.z, 0.f);
    w.angvel[i] = make_float4(b.w.x, b.w.y, b.w.z, 0.f);
}
__device__ __forceinline__ void mask_lin(BodyRef &b) {
    if (!(b.dof & 1)) b.v.x = 0.f;
    if (!(b.dof & 2)) b.v.y = 0.f;
    if (!(b.dof & 4)) b.v.z = 0.f;
}
// getTotalLambda axis-constraint-part.ts:578-625 (softness 0, bias b)
__device__ __forceinline__ float total_lambda(const BodyRef &A, const BodyRef &B, float3 ax, float3 rA, float3 rB,
                                              float eff, float lam, float bias) {
    bool mA = A.motion != STATIC, mB = B.motion != STATIC;
    float jv = 0.f;
    if (mA && mB)
        jv = dot3(ax, A.v - B.v);
    else if (mA)
        jv = dot3(ax, A.v);
    else if (mB)
        jv = -dot3(ax, B.v);
    if (mA) jv += dot3(cross3(rA, ax), A.w);
    if (mB) jv -= dot3(cross3(rB, ax), B.w);
    return lam + eff * (jv - bias);
}
// applyLambda axis-constraint-part.ts:640-707
__device__ __forceinline__ void apply_impulse(BodyRef &A, BodyRef &B, float imA, float imB, float3 ax, float3 rA,
                                              float3 rB, float dl) {
    if (dl == 0.f) return;
    if (A.motion == DYNAMIC) {
        A.v = A.v - ax * (dl * imA);
        mask_lin(A);
        A.w = A.w - symmul(A.I, cross3(rA, ax)) * dl;
    }
    if (B.motion == DYNAMIC) {
        B.v = B.v + ax * (dl * imB);
        mask_lin(B);
        B.w = B.w + symmul(B.I, cross3(rB, ax)) * dl;
    }
}

// warm start of one constraint (contact-constraints.ts:906-955)
__device__ void warm_start_con(ContactConstraint &c, BodyRef &A, BodyRef &B, float ratio) {
    for (int k = 0; k < c.n; k++) {
        ContactPoint &p = c.p[k];
        if (p.eff_t1 != 0.f || p.eff_t2 != 0.f) {
            p.lam_t1 *= ratio;
            apply_impulse(A, B, c.invMassA, c.invMassB, c.t1, p.rA, p.rB, p.lam_t1);
            p.lam_t2 *= ratio;
            apply_impulse(A, B, c.invMassA, c.invMassB, c.t2, p.rA, p.rB, p.lam_t2);
        }
        p.lam_n *= ratio;
        apply_impulse(A, B, c.invMassA, c.invMassB, c.normal, p.rA, p.rB, p.lam_n);
    }
}

// one PGS pass over one contact (contact-constraints.ts:963-1053)
__device__ void solve_velocity_con(ContactConstraint &c, BodyRef &A, BodyRef &B) {
    if (A.motion != DYNAMIC && B.motion != DYNAMIC) return;
    for (int k = 0; k < c.n; k++) {
        ContactPoint &p = c.p[k];
        if (p.eff_t1 != 0.f || p.eff_t2 != 0.f) {
            float l1 = total_lambda(A, B, c.t1, p.rA, p.rB, p.eff_t1, p.lam_t1, 0.f);
            float l2 = total_lambda(A, B, c.t2, p.rA, p.rB, p.eff_t2, p.lam_t2, 0.f);
            float mf = c.friction * p.lam_n;
            float fm = l1 * l1 + l2 * l2;
            if (fm > mf * mf) {
                float s = mf / sqrtf(fm);
                l1 *= s;
                l2 *= s;
            }
            float d1 = l1 - p.lam_t1;
            p.lam_t1 = l1;
            apply_impulse(A, B, c.invMassA, c.invMassB, c.t1, p.rA, p.rB, d1);
            float d2 = l2 - p.lam_t2;
            p.lam_t2 = l2;
            apply_impulse(A, B, c.invMassA, c.invMassB, c.t2, p.rA, p.rB, d2);
        }
    }
    for (int k = 0; k < c.n; k++) {
        ContactPoint &p = c.p[k];
        float tl = total_lambda(A, B, c.normal, p.rA, p.rB, p.eff_n, p.lam_n, p.bias_n);
        tl = fmaxf(0.f, tl);
        float dl = tl - p.lam_n;
        p.lam_n = tl;
        apply_impulse(A, B, c.invMassA, c.invMassB, c.normal, p.rA, p.rB, dl);
    }
}

// rotation step (rigid-body-step.ts:55-97)
__device__ __forceinline__ float4 rotation_step(float4 q, float3 a) {
    float l = sqrtf(lensq3(a));
    if (l > 1.0e-6f) {
        float3 axis = a * (1.f / l);
        float s, co;
        sincosf(l * 0.5f, &s, &co);
        float4 r = make_float4(axis.x * s, axis.y * s, axis.z * s, co);
        q = qnormalize(qmul(r, q));
    }
    return q;
}

struct PoseRef {
    float3 com;
    float4 q;
};

// position solve of one contact (contact-constraints.ts:1098-1216); returns true if an impulse was applied
__device__ bool solve_position_con(DevWorld &w, const ContactConstraint &c, PoseRef &PA, PoseRef &PB, int ma, int mb,
                                   uint32_t fa, uint32_t fb) {
    if (ma != DYNAMIC && mb != DYNAMIC) return false;
    bool any = false;
    // rotations and inverse inertias are taken once per contact, as the reference does
    const Mat3 RA = quat_to_mat(PA.q), RB = quat_to_mat(PB.q);
    Sym3 IA{0, 0, 0, 0, 0, 0}, IB{0, 0, 0, 0, 0, 0};
    if (ma == DYNAMIC) IA = world_inv_inertia(PA.q, w.inertia_rot[c.a], xyz(w.inv_inertia[c.a]), dof_of(fa));
    if (mb == DYNAMIC) IB = world_inv_inertia(PB.q, w.inertia_rot[c.b], xyz(w.inv_inertia[c.b]), dof_of(fb));
    for (int k = 0; k < c.n; k++) {
        const ContactPoint &p = c.p[k];
        float3 pa = PA.com + mmul(RA, p.localA);
        float3 pb = PB.com + mmul(RB, p.localB);
        float sep = dot3(pb - pa, c.normal) + c_settings.slop;
        sep = fmaxf(sep, -c_settings.max_pen);
        if (sep >= 0.f) continue;
        float3 mid = (pa + pb) * 0.5f;
        float3 rA = mid - PA.com, rB = mid - PB.com;
        float iem = inv_eff_mass(ma == DYNAMIC, mb == DYNAMIC, c.invMassA, c.invMassB, IA, IB, rA, rB, c.normal);
        if (iem == 0.f) continue;
        float eff = 1.f / iem;
        float lambda = -eff * c_settings.baumgarte * sep;
        if (ma == DYNAMIC) {
            PA.com = PA.com - c.normal * (lambda * c.invMassA);
            int d = dof_of(fa);
            if (!(d & 1)) PA.com.x = 0.f;
            if (!(d & 2)) PA.com.y = 0.f;
            if (!(d & 4)) PA.com.z = 0.f;
            PA.q = rotation_step(PA.q, -(symmul(IA, cross3(rA, c.normal)) * lambda));
        }
        if (mb == DYNAMIC) {
            PB.com = PB.com + c.normal * (lambda * c.invMassB);
            int d = dof_of(fb);
            if (!(d & 1)) PB.com.x = 0.f;
            if (!(d & 2)) PB.com.y = 0.f;
            if (!(d & 4)) PB.com.z = 0.f;
            PB.q = rotation_step(PB.q, symmul(IB, cross3(rB, c.normal)) * lambda);
        }
        any = true;
    }
    return any;
}

// velocity integration of one body (update.ts:896-976).  With ccd set, a LINEAR_CAST dynamic
// non-sensor body whose step is longer than the cast threshold rotates about its position and
// leaves its translation to the continuous-collision pass (update.ts:930-968).
__device__ void integrate_body(DevWorld &w, int i, float dt, bool ccd) {
    uint32_t f = w.flags[i];
    int m = motion_of(f);
    if (m == STATIC || sleeping_of(f)) return;
    float3 v = xyz(w.linvel[i]), av = xyz(w.angvel[i]);
    if (m == DYNAMIC) {
        float4 d = w.damping[i];
        float ls = lensq3(v);
        if (ls > d.z * d.z) v = normalize3(v) * d.z;
        float as = lensq3(av);
        if (as > d.w * d.w) av = normalize3(av) * d.w;
        w.linvel[i] = make_float4(v.x, v.y, v.z, 0.f);
        w.angvel[i] = make_float4(av.x, av.y, av.z, 0.f);
    }
    float4 q = rotation_step(w.quat[i], av * dt);
    w.quat[i] = q;
    if (ccd && (f & F_LINEAR_CAST) && m == DYNAMIC && !(f & F_SENSOR)) {
        float thr = c_settings.ccd_threshold * shape_inner_radius(w, i, f, w.shape[i]);
        if (lensq3(v * dt) > thr * thr) {
            // setQuaternion rigid-body.ts:737-752: the centre of mass follows the rotation
            float3 c = xyz(w.pos[i]) + qrot(q, shape_com(w, i, f, w.shape[i]));
            w.com[i] = make_float4(c.x, c.y, c.z, 0.f);
            w.ccd_flag[i] = 1;
            return;
        }
    }
    float3 com = xyz(w.com[i]) + v * dt;
    w.com[i] = make_float4(com.x, com.y, com.z, 0.f);
}

// positions from the centre of mass, force clear (update.ts:322-330, 235-238)
__device__ void finish_body(DevWorld &w, int i) {
    uint32_t f = w.flags[i];
    if (motion_of(f) == STATIC || sleeping_of(f)) return;
    // updatePositionFromCenterOfMass rigid-body.ts:545-553: position = com - rotation x shape com
    float3 com = xyz(w.com[i]) - qrot(w.quat[i], shape_com(w, i, f, w.shape[i]));
    w.pos[i] = make_float4(com.x, com.y, com.z, 0.f);
    w.force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.torque[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// updateSleepState sleep.ts:88-117
__device__ bool sleep_update(DevWorld &w, int i, float dt) {
    uint32_t f = w.flags[i];
    if (!(f & F_ALLOW_SLEEP) || (f & F_SENSOR)) return false;
    float3 p[3];
    sleep_points(w, i, f, w.shape[i], w.quat[i], xyz(w.com[i]), p);
    float maxMove = c_settings.sleep_threshold * c_settings.time_before_sleep;
    for (int k = 0; k < 3; k++) {
        float4 s = w.sleep_sph[3 * i + k];
        float d = sqrtf(lensq3(xyz(s) - p[k]));
        s.w = fmaxf(s.w, d);
        w.sleep_sph[3 * i + k] = s;
        if (s.w > maxMove) {
            reset_sleep(w, i);
            return false;
        }
    }
    float t = w.sleep_timer[i] + dt;
    w.sleep_timer[i] = t;
    return t >= c_settings.time_before_sleep;
}
__device__ void sleep_body(DevWorld &w, int i) {
    w.flags[i] |= F_SLEEPING;
    w.linvel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.angvel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// world inverse inertia of the island's dynamic bodies at the start of the solve
__device__ void prepare_body(DevWorld &w, int i) {
    uint32_t f = w.flags[i];
    if (motion_of(f) != DYNAMIC) return;
    float4 ii = w.inv_inertia[i];
    Sym3 s = world_inv_inertia(w.quat[i], w.inertia_rot[i], xyz(ii), dof_of(f));
    w.inv_inertia_world[2 * i] = make_float4(s.xx, s.xy, s.xz, s.yy);
    w.inv_inertia_world[2 * i + 1] = make_float4(s.yz, s.zz, 0.f, 0.f);
}

__device__ __forceinline__ bool con_less(const ContactConstraint &x, const ContactConstraint &y) {
    if (x.sort_key != y.sort_key) return x.sort_key < y.sort_key;
    if (x.a != y.a) return x.a < y.a;
    return x.b < y.b;
}

__device__ void store_impulses(DevWorld &w, CacheRecord *crecs, const ContactConstraint &c) {
    CacheRecord *r = crecs + c.cache_slot;
    for (int k = 0; k < c.n; k++) {
        r->ln[k] = c.p[k].lam_n;
        r->lt1[k] = c.p[k].lam_t1;
        r->lt2[k] = c.p[k].lam_t2;
    }
}

#include "cc_joints.cuh"

// wakeBodiesInUserConstraints (update.ts:853-888): an enabled joint with an awake body
// wakes its sleeping dynamic body.  The reference walks the joints in order, so a wake can
// run down a chain within one step; the scan finds whether any joint has work, and only
// then one thread walks them in order (joints of different worlds never share a body).
__device__ __forceinline__ bool joint_wakes(const DevWorld &w, const DevJointHead &h) {
    if (!(h.flags & JF_ENABLED)) return false;
    uint32_t fa = w.flags[h.a], fb = w.flags[h.b];
    bool act = !sleeping_of(fa) || !sleeping_of(fb);
    bool dyn = motion_of(fa) == DYNAMIC || motion_of(fb) == DYNAMIC;
    return act && dyn && ((sleeping_of(fa) && motion_of(fa) == DYNAMIC) || (sleeping_of(fb) && motion_of(fb) == DYNAMIC));
}
__global__ void k_joint_wake_scan(DevWorld w) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < joint_total(w); k += gridDim.x * blockDim.x)
        if (joint_wakes(w, joint_head(w, joint_id_at(w, k)))) *w.joint_wake = 1;
}
__global__ void k_joint_wake_serial(DevWorld w) {
    if (!*w.joint_wake) return;
    *w.joint_wake = 0;
    for (int k = 0; k < joint_total(w); k++) {
        const DevJointHead &h = joint_head(w, joint_id_at(w, k));
        if (!joint_wakes(w, h)) continue;
        int ids[2] = {h.a, h.b};
        for (int e = 0; e < 2; e++) {
            int i = ids[e];
            uint32_t f = w.flags[i];
            if (!(sleeping_of(f) && motion_of(f) == DYNAMIC)) continue;
            w.flags[i] = f & ~F_SLEEPING;
            reset_sleep(w, i);
        }
    }
}
// setupVelocityConstraints (constraints.ts:276-287) for every enabled joint with an awake
// body (updateSleeping constraints.ts:264-274)
__global__ void k_joint_setup(DevWorld w, float dt) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < joint_total(w); k += gridDim.x * blockDim.x) {
        int id = joint_id_at(w, k);
        if (joint_active(w, joint_head(w, id))) joint_setup(w, id, dt);
    }
}

// ---------------------------------------------------------------------------
// small islands: one thread runs the island in the reference's exact order
// ---------------------------------------------------------------------------
// JOINTS: the islands with joints (their own list); the contact-only instance carries no joint code
template <bool JOINTS>
__global__ void __launch_bounds__(128) k_solve_small(DevWorld w, CacheTables ct, const int *small_list, float dt,
                                                      float ratio, int phase) {
    if (islands_failed(w)) return;
    int ns = JOINTS ? w.ctr->num_small_joint_islands : w.ctr->num_small_islands;
    CacheRecord *crecs = ct.recs[*ct.parity];
    // Islands without joints come by size, most contacts first, in chunks of 32: a warp's lanes
    // solve islands of one size.  Chunk c goes to block c mod gridDim.x, so the chunks of the
    // largest islands are spread over the blocks (and the SMs) rather than packed into the first.
    const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
    for (int r = 0;; r++) {
        const int s = JOINTS ? (r * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x
                             : ((r * wpb + (threadIdx.x >> 5)) * gridDim.x + blockIdx.x) * 32 + lane;
        if (s >= ns) break;
        int isl = JOINTS ? small_list[s] : bucketed_island(small_list, w.cap, w.ctr->small_bucket, SMALL_BUCKETS, s);
        int vel_iters, pos_iters;  // the island's iteration counts (islands.ts:344-386)
        island_iterations(w, isl, c_settings.vel_iters, c_settings.pos_iters, vel_iters, pos_iters);
        int nb = w.island_body_count[isl], nc = w.island_cons_count[isl];
        int nj = JOINTS ? w.island_joint_count[isl] : 0;
        const int *bl = w.island_bodies + w.island_body_off[isl];
        const int *cl = w.island_cons + w.island_cons_off[isl];
        int order[SMALL_ISLAND_MAX_CONS];
        for (int k = 0; k < nc; k++) order[k] = cl[k];
        // sortContactIndices: insertion sort by (sortKey, idA, idB)
        for (int k = 1; k < nc; k++) {
            int x = order[k];
            int j = k - 1;
            while (j >= 0 && con_less(w.cons[x], w.cons[order[j]])) {
                order[j + 1] = order[j];
                j--;
            }
            order[j + 1] = x;
        }
        // joints: warm started type by type in creation order (constraints.ts:290-303), solved
        // by (priority, index, type) (sortConstraintIds constraints.ts:248-261)
        int jord[SMALL_ISLAND_MAX_JOINTS];
        if (nj > 0) {
            const int *jl = w.island_joints + w.island_joint_off[isl];
            for (int k = 0; k < nj; k++) {
                int x = jl[k], j = k - 1;
                while (j >= 0 && jord[j] > x) {
                    jord[j + 1] = jord[j];
                    j--;
                }
                jord[j + 1] = x;
            }
        }
        const bool vel = phase != SOLVE_POSITION;
        if (vel) {
            for (int k = 0; k < nb; k++) prepare_body(w, bl[k]);
            if ((nc > 0 || nj > 0) && c_settings.warm_starting) {
                for (int k = 0; k < nc; k++) {
                    ContactConstraint &c = w.cons[order[k]];
                    BodyRef A = load_body(w, c.a), B = load_body(w, c.b);
                    warm_start_con(c, A, B, ratio);
                    store_body_vel(w, c.a, A);
                    store_body_vel(w, c.b, B);
                }
                for (int k = 0; k < nj; k++) joint_warm(w, jord[k], ratio);
            }
        }
        for (int k = 1; k < nj; k++) {  // now into solve order
            int x = jord[k], j = k - 1;
            while (j >= 0 && joint_before(w, x, jord[j])) {
                jord[j + 1] = jord[j];
                j--;
            }
            jord[j + 1] = x;
        }
        if (vel) {
            if (nc > 0 || nj > 0) {
                for (int it = 0; it < vel_iters; it++) {
                    for (int k = 0; k < nc; k++) {
                        ContactConstraint &c = w.cons[order[k]];
                        BodyRef A = load_body(w, c.a), B = load_body(w, c.b);
                        solve_velocity_con(c, A, B);
                        store_body_vel(w, c.a, A);
                        store_body_vel(w, c.b, B);
                    }
                    for (int k = 0; k < nj; k++) joint_solve_velocity(w, jord[k], dt);
                }
                for (int k = 0; k < nc; k++) store_impulses(w, crecs, w.cons[order[k]]);
            }
            for (int k = 0; k < nb; k++) integrate_body(w, bl[k], dt, phase == SOLVE_VELOCITY);
            if (phase == SOLVE_VELOCITY) continue;
        }
        if (nc > 0 || nj > 0) {
            for (int it = 0; it < pos_iters; it++) {
                bool any = false;
                for (int k = 0; k < nc; k++) {
                    const ContactConstraint &c = w.cons[order[k]];
                    uint32_t fa = w.flags[c.a], fb = w.flags[c.b];
                    PoseRef PA{xyz(w.com[c.a]), w.quat[c.a]}, PB{xyz(w.com[c.b]), w.quat[c.b]};
                    bool applied = solve_position_con(w, c, PA, PB, motion_of(fa), motion_of(fb), fa, fb);
                    if (applied) {
                        if (motion_of(fa) == DYNAMIC) {
                            w.com[c.a] = make_float4(PA.com.x, PA.com.y, PA.com.z, 0.f);
                            w.quat[c.a] = PA.q;
                        }
                        if (motion_of(fb) == DYNAMIC) {
                            w.com[c.b] = make_float4(PB.com.x, PB.com.y, PB.com.z, 0.f);
                            w.quat[c.b] = PB.q;
                        }
                        any = true;
                    }
                }
                for (int k = 0; k < nj; k++) any = joint_solve_position(w, jord[k], dt) || any;
                if (!any) break;
            }
        }
        for (int k = 0; k < nb; k++) finish_body(w, bl[k]);
        if (c_settings.allow_sleeping) {
            bool all = true;
            for (int k = 0; k < nb; k++) {
                int i = bl[k];
                if (motion_of(w.flags[i]) != DYNAMIC) continue;
                bool cs = sleep_update(w, i, dt);
                all = all && cs;
            }
            if (all)
                for (int k = 0; k < nb; k++)
                    if (motion_of(w.flags[bl[k]]) == DYNAMIC) sleep_body(w, bl[k]);
        }
    }
}

// ---------------------------------------------------------------------------
// large islands: one CTA per island, contacts sorted by the reference key,
// greedily coloured in that order and swept colour by colour
// ---------------------------------------------------------------------------
constexpr int LARGE_BLOCK = 256;
constexpr int JOINT_COLOURS = 64;  // joint colours of the per-CTA solve; the rest go to one thread

template <bool JOINTS>
__global__ void __launch_bounds__(LARGE_BLOCK) k_solve_large(DevWorld w, CacheTables ct, const int *large_list,
                                                              int *scratch_order, int *scratch_colour,
                                                              int *scratch_claim, float dt, float ratio,
                                                              int phase) {
    if (islands_failed(w)) return;
    __shared__ int s_any;
    __shared__ int s_ncol;
    __shared__ int s_colour_start[257];
    __shared__ int s_jstart[JOINT_COLOURS + 2];
    int nl = JOINTS ? w.ctr->num_large_joint_islands : w.ctr->num_large_islands;
    CacheRecord *crecs = ct.recs[*ct.parity];
    for (int li = blockIdx.x; li < nl; li += gridDim.x) {
        int isl = large_list[li];
        int vel_iters, pos_iters;
        island_iterations(w, isl, c_settings.vel_iters, c_settings.pos_iters, vel_iters, pos_iters);
        int nb = w.island_body_count[isl], nc = w.island_cons_count[isl];
        const int *bl = w.island_bodies + w.island_body_off[isl];
        const int *cl = w.island_cons + w.island_cons_off[isl];
        int *order = scratch_order + w.island_cons_off[isl];
        int *colour = scratch_colour + w.island_cons_off[isl];
        // rank of each contact in (sortKey, A, B) order (ties cannot occur: keys include both bodies)
        for (int k = threadIdx.x; k < nc; k += blockDim.x) {
            const ContactConstraint &c = w.cons[cl[k]];
            int rank = 0;
            for (int j = 0; j < nc; j++) {
                const ContactConstraint &o = w.cons[cl[j]];
                if (con_less(o, c) || (!con_less(c, o) && j < k)) rank++;
            }
            order[rank] = cl[k];
        }
        const bool vel = phase != SOLVE_POSITION;
        if (vel)
            for (int k = threadIdx.x; k < nb; k += blockDim.x) prepare_body(w, bl[k]);
        // the island's joints in index order (warm start) and in (priority, index) order
        // (sortConstraintIds constraints.ts:248-261)
        int nj = JOINTS ? w.island_joint_count[isl] : 0;
        const int *jl = w.island_joints + (nj > 0 ? w.island_joint_off[isl] : 0);
        int *j_idx = const_cast<int *>(jl) + w.max_joints;
        int *j_pri = j_idx + w.max_joints;
        for (int k = threadIdx.x; k < nj; k += blockDim.x) {
            int jk = jl[k];
            int r1 = 0, r2 = 0;
            for (int m = 0; m < nj; m++) {
                int jm = jl[m];
                r1 += jm < jk;  // ids order by type, then creation index
                r2 += joint_before(w, jm, jk);
            }
            j_idx[r1] = jk;
            j_pri[r2] = jk;
        }
        __syncthreads();
        // greedy colouring in rank order: per round, the lowest rank claims each dynamic body
        for (int k = threadIdx.x; k < nc; k += blockDim.x) colour[k] = -1;
        if (threadIdx.x == 0) s_ncol = 0;
        __syncthreads();
        int round = 0;
        while (true) {
            for (int k = threadIdx.x; k < nb; k += blockDim.x) scratch_claim[bl[k]] = 0x7fffffff;
            __syncthreads();
            int left = 0;
            for (int k = threadIdx.x; k < nc; k += blockDim.x) {
                if (colour[k] >= 0) continue;
                left = 1;
                const ContactConstraint &c = w.cons[order[k]];
                if (motion_of(w.flags[c.a]) == DYNAMIC) atomicMin(&scratch_claim[c.a], k);
                if (motion_of(w.flags[c.b]) == DYNAMIC) atomicMin(&scratch_claim[c.b], k);
            }
            if (!__syncthreads_or(left)) break;
            for (int k = threadIdx.x; k < nc; k += blockDim.x) {
                if (colour[k] >= 0) continue;
                const ContactConstraint &c = w.cons[order[k]];
                bool oka = motion_of(w.flags[c.a]) != DYNAMIC || scratch_claim[c.a] == k;
                bool okb = motion_of(w.flags[c.b]) != DYNAMIC || scratch_claim[c.b] == k;
                if (oka && okb) colour[k] = round;
            }
            __syncthreads();
            round++;
            if (round >= 256) {
                // put the rest in the last colour, solved serially by one thread
                for (int k = threadIdx.x; k < nc; k += blockDim.x)
                    if (colour[k] < 0) colour[k] = 256;
                __syncthreads();
                break;
            }
        }
        int ncol = round;
        // counting sort of ranks by colour (stable: keeps rank order inside a colour)
        if (threadIdx.x == 0) {
            for (int c = 0; c <= 256; c++) s_colour_start[c] = 0;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < nc; k += blockDim.x) atomicAdd(&s_colour_start[min(colour[k], 256)], 1);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int c = 0; c <= 256; c++) {
                int t = s_colour_start[c];
                s_colour_start[c] = acc;
                acc += t;
            }
            s_ncol = ncol;
        }
        __syncthreads();
        // place contacts: sequential per colour by one thread keeps rank order
        int *sorted = scratch_claim + w.cap;  // second half of the claim scratch
        int *sorted_i = sorted + w.island_cons_off[isl];
        if (threadIdx.x == 0) {
            int fill[257];
            for (int c = 0; c <= 256; c++) fill[c] = s_colour_start[c];
            for (int k = 0; k < nc; k++) {
                int c = min(colour[k], 256);
                sorted_i[fill[c]++] = order[k];
            }
        }
        __syncthreads();
        // joints: greedy colouring in solve order like the contacts, JOINT_COLOURS colours at most
        // (the rest is solved by one thread in order); warm starting stays serial in index order
        int *j_col = j_pri + w.max_joints;
        int *j_grp = j_col + w.max_joints;
        if (nj > 0) {
            for (int k = threadIdx.x; k < nj; k += blockDim.x) j_col[k] = -1;
            int jround = 0;
            while (true) {
                for (int k = threadIdx.x; k < nb; k += blockDim.x) scratch_claim[bl[k]] = 0x7fffffff;
                __syncthreads();
                int left = 0;
                for (int k = threadIdx.x; k < nj; k += blockDim.x) {
                    if (j_col[k] >= 0) continue;
                    left = 1;
                    const DevJointHead &h = joint_head(w, j_pri[k]);
                    if (motion_of(w.flags[h.a]) == DYNAMIC) atomicMin(&scratch_claim[h.a], k);
                    if (motion_of(w.flags[h.b]) == DYNAMIC) atomicMin(&scratch_claim[h.b], k);
                }
                if (!__syncthreads_or(left)) break;
                for (int k = threadIdx.x; k < nj; k += blockDim.x) {
                    if (j_col[k] >= 0) continue;
                    const DevJointHead &h = joint_head(w, j_pri[k]);
                    bool oka = motion_of(w.flags[h.a]) != DYNAMIC || scratch_claim[h.a] == k;
                    bool okb = motion_of(w.flags[h.b]) != DYNAMIC || scratch_claim[h.b] == k;
                    if (oka && okb) j_col[k] = jround;
                }
                __syncthreads();
                if (++jround >= JOINT_COLOURS) {
                    for (int k = threadIdx.x; k < nj; k += blockDim.x)
                        if (j_col[k] < 0) j_col[k] = JOINT_COLOURS;
                    __syncthreads();
                    break;
                }
            }
            if (threadIdx.x == 0) {  // counting sort by colour, rank order inside a colour
                for (int c = 0; c <= JOINT_COLOURS + 1; c++) s_jstart[c] = 0;
                for (int k = 0; k < nj; k++) s_jstart[j_col[k] + 1]++;
                for (int c = 0; c <= JOINT_COLOURS; c++) s_jstart[c + 1] += s_jstart[c];
                int fill[JOINT_COLOURS + 1];
                for (int c = 0; c <= JOINT_COLOURS; c++) fill[c] = s_jstart[c];
                for (int k = 0; k < nj; k++) j_grp[fill[j_col[k]]++] = j_pri[k];
            }
            __syncthreads();
        }
        // joint colours in turn: parallel inside a colour, the last (overflow) colour by one thread
        auto joint_sweep = [&](int mode) -> bool {
            bool any = false;
            for (int c = 0; c <= JOINT_COLOURS; c++) {
                int s0 = s_jstart[c], s1 = s_jstart[c + 1];
                if (s1 <= s0) continue;
                int kbeg = c < JOINT_COLOURS ? s0 + (int)threadIdx.x : (threadIdx.x == 0 ? s0 : s1);
                int kstep = c < JOINT_COLOURS ? (int)blockDim.x : 1;
                for (int k = kbeg; k < s1; k += kstep) {
                    if (mode == 0)
                        joint_solve_velocity(w, j_grp[k], dt);
                    else
                        any = joint_solve_position(w, j_grp[k], dt) || any;
                }
                __syncthreads();
            }
            return any;
        };
        int colour_end_last = nc;
        // warm start (per colour)
        auto sweep = [&](int mode) {
            for (int c = 0; c <= 256; c++) {
                int s0 = s_colour_start[c];
                int s1 = (c < 256) ? s_colour_start[c + 1] : colour_end_last;
                if (s1 <= s0) {
                    if (c >= s_ncol) break;
                    continue;
                }
                if (c < 256) {
                    for (int k = s0 + threadIdx.x; k < s1; k += blockDim.x) {
                        ContactConstraint &con = w.cons[sorted_i[k]];
                        BodyRef A = load_body(w, con.a), B = load_body(w, con.b);
                        if (mode == 0)
                            warm_start_con(con, A, B, ratio);
                        else
                            solve_velocity_con(con, A, B);
                        store_body_vel(w, con.a, A);
                        store_body_vel(w, con.b, B);
                    }
                } else if (threadIdx.x == 0) {
                    for (int k = s0; k < s1; k++) {
                        ContactConstraint &con = w.cons[sorted_i[k]];
                        BodyRef A = load_body(w, con.a), B = load_body(w, con.b);
                        if (mode == 0)
                            warm_start_con(con, A, B, ratio);
                        else
                            solve_velocity_con(con, A, B);
                        store_body_vel(w, con.a, A);
                        store_body_vel(w, con.b, B);
                    }
                }
                __syncthreads();
            }
        };
        // contacts, then joints (update.ts:116-165)
        if (vel) {
            if (c_settings.warm_starting) {
                sweep(0);
                if (nj > 0) {
                    __syncthreads();
                    if (threadIdx.x == 0)
                        for (int k = 0; k < nj; k++) joint_warm(w, j_idx[k], ratio);
                    __syncthreads();
                }
            }
            for (int it = 0; it < vel_iters; it++) {
                sweep(1);
                if (nj > 0) {
                    __syncthreads();
                    joint_sweep(0);
                }
            }
            for (int k = threadIdx.x; k < nc; k += blockDim.x) store_impulses(w, crecs, w.cons[cl[k]]);
            for (int k = threadIdx.x; k < nb; k += blockDim.x) integrate_body(w, bl[k], dt, phase == SOLVE_VELOCITY);
            __syncthreads();
            if (phase == SOLVE_VELOCITY) continue;
        }
        for (int it = 0; it < pos_iters; it++) {
            if (threadIdx.x == 0) s_any = 0;
            __syncthreads();
            for (int c = 0; c <= 256; c++) {
                int s0 = s_colour_start[c];
                int s1 = (c < 256) ? s_colour_start[c + 1] : colour_end_last;
                if (s1 <= s0) {
                    if (c >= s_ncol) break;
                    continue;
                }
                int kbeg = (c < 256) ? s0 + (int)threadIdx.x : (threadIdx.x == 0 ? s0 : s1);
                int kstep = (c < 256) ? (int)blockDim.x : 1;
                for (int k = kbeg; k < s1; k += kstep) {
                    const ContactConstraint &con = w.cons[sorted_i[k]];
                    uint32_t fa = w.flags[con.a], fb = w.flags[con.b];
                    PoseRef PA{xyz(w.com[con.a]), w.quat[con.a]}, PB{xyz(w.com[con.b]), w.quat[con.b]};
                    if (solve_position_con(w, con, PA, PB, motion_of(fa), motion_of(fb), fa, fb)) {
                        if (motion_of(fa) == DYNAMIC) {
                            w.com[con.a] = make_float4(PA.com.x, PA.com.y, PA.com.z, 0.f);
                            w.quat[con.a] = PA.q;
                        }
                        if (motion_of(fb) == DYNAMIC) {
                            w.com[con.b] = make_float4(PB.com.x, PB.com.y, PB.com.z, 0.f);
                            w.quat[con.b] = PB.q;
                        }
                        s_any = 1;
                    }
                }
                __syncthreads();
            }
            if (nj > 0) {
                __syncthreads();
                if (joint_sweep(1)) s_any = 1;
                __syncthreads();
            }
            if (!s_any) break;
            __syncthreads();
        }
        for (int k = threadIdx.x; k < nb; k += blockDim.x) finish_body(w, bl[k]);
        __syncthreads();
        if (c_settings.allow_sleeping) {
            int mine = 1;
            for (int k = threadIdx.x; k < nb; k += blockDim.x) {
                int i = bl[k];
                if (motion_of(w.flags[i]) != DYNAMIC) continue;
                if (!sleep_update(w, i, dt)) mine = 0;
            }
            int all = __syncthreads_and(mine);
            if (all)
                for (int k = threadIdx.x; k < nb; k += blockDim.x)
                    if (motion_of(w.flags[bl[k]]) == DYNAMIC) sleep_body(w, bl[k]);
        }
        __syncthreads();
    }
}


// ---------------------------------------------------------------------------
// mid-size islands: one warp per island.  The island's contacts are sorted by
// the reference key (bitonic sort in shared memory), greedily coloured in that
// order, and swept colour by colour with the island's body velocities held in
// shared memory; a __syncwarp separates the colours.
// ---------------------------------------------------------------------------
constexpr int WARP_BLOCK = 128;
constexpr int WARPS_PER_BLOCK = WARP_BLOCK / 32;

// one warp's island in shared memory, for islands of at most MC contacts and MB bodies
template <int MC, int MB>
struct WarpIslandT {
    uint32_t key[MC];  // sort key, then colour
    int ia[MC];        // body A id, then local index of A (-1: not in the island)
    int ib[MC];
    int idx[MC];       // constraint index in rank order
    int sorted[MC];    // ranks grouped by colour, rank order inside a colour
    int cstart[WARP_MAX_COLOURS + 2];
    float4 v[MB];    // linear velocity | inverse mass
    float4 av[MB];   // angular velocity | flags (bit pattern)
    float4 I0[MB];   // world inverse inertia xx xy xz yy
    float2 I1[MB];   // yz zz
    int body[MB];
    int claim[MB];
};
using WarpIsland = WarpIslandT<WARP_MAX_CONS, WARP_MAX_BODIES>;
using WarpIslandS = WarpIslandT<WARP_S_CONS, WARP_S_BODIES>;

template <class WI>
__device__ __forceinline__ bool rank_less(const WI &s, int x, int y) {
    if (s.key[x] != s.key[y]) return s.key[x] < s.key[y];
    if (s.ia[x] != s.ia[y]) return s.ia[x] < s.ia[y];
    return s.ib[x] < s.ib[y];
}

template <class WI>
__device__ __forceinline__ BodyRef warp_body(const DevWorld &w, const WI &s, int local, int global) {
    if (local < 0) return load_body(w, global);
    BodyRef b;
    float4 v = s.v[local], av = s.av[local];
    uint32_t f = __float_as_uint(av.w);
    b.v = xyz(v);
    b.w = xyz(av);
    b.im = v.w;
    b.motion = motion_of(f);
    b.dof = dof_of(f);
    float4 i0 = s.I0[local];
    float2 i1 = s.I1[local];
    b.I = Sym3{i0.x, i0.y, i0.z, i0.w, i1.x, i1.y};
    return b;
}
template <class WI>
__device__ __forceinline__ void warp_store(WI &s, int local, const BodyRef &b) {
    if (local < 0 || b.motion != DYNAMIC) return;
    s.v[local] = make_float4(b.v.x, b.v.y, b.v.z, s.v[local].w);
    s.av[local] = make_float4(b.w.x, b.w.y, b.w.z, s.av[local].w);
}

// WI: the shared-memory island (its capacity); the islands of size classes [b0, b1) of the
// per-warp list, taken from *cursor after the first round
template <class WI>
__global__ void __launch_bounds__(WARP_BLOCK) k_solve_warp(DevWorld w, CacheTables ct, float dt, float ratio,
                                                            int phase, int b0, int b1, int *cursor) {
    if (islands_failed(w)) return;
    extern __shared__ __align__(16) unsigned char warp_smem_raw[];  // WARPS_PER_BLOCK islands
    const int lane = threadIdx.x & 31;
    WI &S = reinterpret_cast<WI *>(warp_smem_raw)[threadIdx.x >> 5];
    const unsigned FULL = 0xffffffffu;
    int nmid = 0;
    for (int b = b0; b < b1; b++) nmid += w.ctr->mid_bucket[b];
    CacheRecord *crecs = ct.recs[*ct.parity];
    // The first island of warp k of every block is island k x gridDim.x + blockIdx.x of the list
    // (largest first), so the largest islands start together on different SMs; the rest come
    // from the cursor, after the first round's.
    const int nwarps = gridDim.x * WARPS_PER_BLOCK;
    bool first = true;
    while (true) {
        int li = 0;
        if (first)
            li = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
        else if (lane == 0)
            li = nwarps + atomicAdd(cursor, 1);
        li = __shfl_sync(FULL, li, 0);
        first = false;
        if (li >= nmid) break;
        // the largest islands are taken first, so the last ones to finish are small
        const int isl = bucketed_island(w.mid_list + (size_t)b0 * w.cap, w.cap, w.ctr->mid_bucket + b0, b1 - b0, li);
        int vel_iters, pos_iters;
        island_iterations(w, isl, c_settings.vel_iters, c_settings.pos_iters, vel_iters, pos_iters);
        const int nb = w.island_body_count[isl], nc = w.island_cons_count[isl];
        const int *bl = w.island_bodies + w.island_body_off[isl];
        const int *cl = w.island_cons + w.island_cons_off[isl];
        // bodies: velocities, inverse mass, flags and world inverse inertia into shared memory
        for (int k = lane; k < nb; k += 32) {
            int i = bl[k];
            uint32_t f = w.flags[i];
            float4 ii = w.inv_inertia[i];
            float4 v = w.linvel[i], av = w.angvel[i];
            Sym3 I{0, 0, 0, 0, 0, 0};
            if (motion_of(f) == DYNAMIC) I = world_inv_inertia(w.quat[i], w.inertia_rot[i], xyz(ii), dof_of(f));
            S.v[k] = make_float4(v.x, v.y, v.z, ii.w);
            S.av[k] = make_float4(av.x, av.y, av.z, __uint_as_float(f));
            S.I0[k] = make_float4(I.xx, I.xy, I.xz, I.yy);
            S.I1[k] = make_float2(I.yz, I.zz);
            S.body[k] = i;
            w.body_local[i] = k;
        }
        // contacts: keys for the rank sort, padded to a power of two
        int P = 32;
        while (P < nc) P <<= 1;
        for (int k = lane; k < P; k += 32) {
            if (k < nc) {
                int ci = cl[k];
                const ContactConstraint &c = w.cons[ci];
                S.key[k] = c.sort_key;
                S.ia[k] = c.a;
                S.ib[k] = c.b;
                S.idx[k] = ci;
            } else {
                S.key[k] = 0xffffffffu;
                S.ia[k] = 0x7fffffff;
                S.ib[k] = 0x7fffffff;
                S.idx[k] = -1;
            }
        }
        __syncwarp();
        // sortContactIndices (contact-constraints.ts:1240-1264): bitonic sort by (sortKey, idA, idB)
        for (int kk = 2; kk <= P; kk <<= 1) {
            for (int j = kk >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < P; i += 32) {
                    int l = i ^ j;
                    if (l > i) {
                        bool up = (i & kk) == 0;
                        if (rank_less(S, l, i) == up) {
                            uint32_t tk = S.key[i];
                            S.key[i] = S.key[l];
                            S.key[l] = tk;
                            int t = S.ia[i];
                            S.ia[i] = S.ia[l];
                            S.ia[l] = t;
                            t = S.ib[i];
                            S.ib[i] = S.ib[l];
                            S.ib[l] = t;
                            t = S.idx[i];
                            S.idx[i] = S.idx[l];
                            S.idx[l] = t;
                        }
                    }
                }
                __syncwarp();
            }
        }
        // local body indices (-1 when the body is not one of this island's bodies)
        for (int k = lane; k < nc; k += 32) {
            int a = S.ia[k], b = S.ib[k];
            int la = w.body_local[a], lb = w.body_local[b];
            S.ia[k] = (la >= 0 && la < nb && S.body[la] == a) ? la : -1;
            S.ib[k] = (lb >= 0 && lb < nb && S.body[lb] == b) ? lb : -1;
            S.key[k] = 0xffffffffu;  // colour: unassigned
        }
        __syncwarp();
        // greedy colouring in rank order: per round, the lowest unassigned rank on each dynamic body claims it
        int ncol = 0;
        bool tail = false;
        while (true) {
            for (int k = lane; k < nb; k += 32) S.claim[k] = 0x7fffffff;
            __syncwarp();
            bool left = false;
            for (int k = lane; k < nc; k += 32) {
                if (S.key[k] != 0xffffffffu) continue;
                left = true;
                int la = S.ia[k], lb = S.ib[k];
                if (la >= 0 && motion_of(__float_as_uint(S.av[la].w)) == DYNAMIC) atomicMin(&S.claim[la], k);
                if (lb >= 0 && motion_of(__float_as_uint(S.av[lb].w)) == DYNAMIC) atomicMin(&S.claim[lb], k);
            }
            __syncwarp();
            if (!__any_sync(FULL, left)) break;
            if (ncol == WARP_MAX_COLOURS) {
                for (int k = lane; k < nc; k += 32)
                    if (S.key[k] == 0xffffffffu) S.key[k] = WARP_MAX_COLOURS;
                tail = true;
                __syncwarp();
                break;
            }
            for (int k = lane; k < nc; k += 32) {
                if (S.key[k] != 0xffffffffu) continue;
                int la = S.ia[k], lb = S.ib[k];
                bool oka = la < 0 || motion_of(__float_as_uint(S.av[la].w)) != DYNAMIC || S.claim[la] == k;
                bool okb = lb < 0 || motion_of(__float_as_uint(S.av[lb].w)) != DYNAMIC || S.claim[lb] == k;
                if (oka && okb) S.key[k] = (uint32_t)ncol;
            }
            __syncwarp();
            ncol++;
        }
        const int nsweep = ncol + (tail ? 1 : 0);
        // group ranks by colour, keeping rank order inside each colour
        {
            int pos = 0;
            for (int c = 0; c < nsweep; c++) {
                uint32_t col = (c < ncol) ? (uint32_t)c : (uint32_t)WARP_MAX_COLOURS;
                if (lane == 0) S.cstart[c] = pos;
                for (int base = 0; base < nc; base += 32) {
                    int k = base + lane;
                    bool pred = k < nc && S.key[k] == col;
                    unsigned m = __ballot_sync(FULL, pred);
                    if (pred) S.sorted[pos + __popc(m & ((1u << lane) - 1u))] = k;
                    pos += __popc(m);
                }
            }
            if (lane == 0) S.cstart[nsweep] = pos;
        }
        __syncwarp();
        // warm start and velocity iterations, colour by colour
        const bool vel = phase != SOLVE_POSITION;
        for (int pass = (c_settings.warm_starting ? -1 : 0); vel && pass < vel_iters; pass++) {
            for (int c = 0; c < nsweep; c++) {
                int s0 = S.cstart[c], s1 = S.cstart[c + 1];
                bool serial = tail && c == ncol;
                int e0 = serial ? (lane == 0 ? s0 : s1) : s0 + lane;
                int es = serial ? 1 : 32;
                for (int e = e0; e < s1; e += es) {
                    int k = S.sorted[e];
                    ContactConstraint &con = w.cons[S.idx[k]];
                    int la = S.ia[k], lb = S.ib[k];
                    BodyRef A = warp_body(w, S, la, con.a), B = warp_body(w, S, lb, con.b);
                    if (pass < 0)
                        warm_start_con(con, A, B, ratio);
                    else
                        solve_velocity_con(con, A, B);
                    warp_store(S, la, A);
                    warp_store(S, lb, B);
                }
                __syncwarp();
            }
        }
        if (vel) {
            for (int k = lane; k < nc; k += 32) store_impulses(w, crecs, w.cons[S.idx[k]]);
            // velocities back to global memory, then integration (update.ts:896-976)
            for (int k = lane; k < nb; k += 32) {
                int i = S.body[k];
                if (motion_of(__float_as_uint(S.av[k].w)) == DYNAMIC) {
                    float4 v = S.v[k], av = S.av[k];
                    w.linvel[i] = make_float4(v.x, v.y, v.z, 0.f);
                    w.angvel[i] = make_float4(av.x, av.y, av.z, 0.f);
                }
                integrate_body(w, i, dt, phase == SOLVE_VELOCITY);
            }
            __syncwarp();
            if (phase == SOLVE_VELOCITY) continue;
        }
        // position iterations (contact-constraints.ts:1098-1216), early exit as update.ts:218-221
        for (int it = 0; it < pos_iters; it++) {
            bool any = false;
            for (int c = 0; c < nsweep; c++) {
                int s0 = S.cstart[c], s1 = S.cstart[c + 1];
                bool serial = tail && c == ncol;
                int e0 = serial ? (lane == 0 ? s0 : s1) : s0 + lane;
                int es = serial ? 1 : 32;
                for (int e = e0; e < s1; e += es) {
                    const ContactConstraint &con = w.cons[S.idx[S.sorted[e]]];
                    uint32_t fa = w.flags[con.a], fb = w.flags[con.b];
                    PoseRef PA{xyz(w.com[con.a]), w.quat[con.a]}, PB{xyz(w.com[con.b]), w.quat[con.b]};
                    if (solve_position_con(w, con, PA, PB, motion_of(fa), motion_of(fb), fa, fb)) {
                        if (motion_of(fa) == DYNAMIC) {
                            w.com[con.a] = make_float4(PA.com.x, PA.com.y, PA.com.z, 0.f);
                            w.quat[con.a] = PA.q;
                        }
                        if (motion_of(fb) == DYNAMIC) {
                            w.com[con.b] = make_float4(PB.com.x, PB.com.y, PB.com.z, 0.f);
                            w.quat[con.b] = PB.q;
                        }
                        any = true;
                    }
                }
                __syncwarp();
            }
            if (!__any_sync(FULL, any)) break;
        }
        for (int k = lane; k < nb; k += 32) finish_body(w, S.body[k]);
        __syncwarp();
        if (c_settings.allow_sleeping) {
            bool mine = true;
            for (int k = lane; k < nb; k += 32) {
                int i = S.body[k];
                if (motion_of(w.flags[i]) != DYNAMIC) continue;
                if (!sleep_update(w, i, dt)) mine = false;
            }
            if (__all_sync(FULL, mine))
                for (int k = lane; k < nb; k += 32)
                    if (motion_of(w.flags[S.body[k]]) == DYNAMIC) sleep_body(w, S.body[k]);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// giant islands: an island with more than giant_min constraints (a pile of
// thousands of bodies) is solved by the whole grid.  One cooperative launch,
// co-resident blocks meeting at a bounded grid barrier, walks the giant
// islands one after another:
//   colouring  - greedy, in the reference's solve order, without sorting: per
//                round every uncoloured constraint claims its dynamic bodies
//                with a 64-bit atomicMin of its order key, and the ones that
//                hold all their claims take the round's colour.  Contacts and
//                joints are coloured side by side with their own claims;
//   sweeps     - warm start, velocity and position iterations visit the
//                contact colours, then the joint colours; inside a colour the
//                constraints share no dynamic body, so their order does not
//                change the result.
// ---------------------------------------------------------------------------
constexpr int GIANT_BLOCK = 256;

// Grid barrier over the co-resident blocks of the cooperative launch.  The wait is bounded:
// a block that gives up raises bar_error and OVF_TIMEOUT, and every block then leaves.
__device__ bool grid_barrier(DevCounters *ctr, unsigned nblocks) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &ctr->bar_gen;
        volatile int *err = &ctr->bar_error;
        unsigned g = *gen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&ctr->bar_count, 1u) == nblocks - 1) {
            atomicExch(&ctr->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctr->bar_gen, 1u);
        } else {
            unsigned spins = 0;
            while (*gen == g) {
                if (*err || ++spins > c_settings.wait_polls) {
                    atomicExch(&ctr->bar_error, 1);
                    atomicOr(&ctr->overflow, OVF_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok && !*err;
    }
    __syncthreads();
    return s_ok != 0;
}

// order keys: contacts by (sortKey, idA, idB) with A < B; for a claim on body X the other body
// breaks ties, which orders the contacts sharing X as the full key does
__device__ __forceinline__ unsigned long long contact_claim_key(const ContactConstraint &c, int x) {
    return ((unsigned long long)c.sort_key << 32) | (unsigned)(x == c.a ? c.b : c.a);
}
__device__ __forceinline__ unsigned long long joint_claim_key(const DevWorld &w, int id) {
    const DevJointHead &h = joint_head(w, id);
    return ((unsigned long long)((unsigned)h.priority ^ 0x80000000u) << 32) | ((unsigned long long)h.index << 3) |
           (unsigned)joint_type_of(id);
}

__global__ void __launch_bounds__(GIANT_BLOCK) k_solve_giant(DevWorld w, CacheTables ct, float dt, float ratio,
                                                              int phase) {
    DevCounters *ctr = w.ctr;
    const int ng = ctr->num_giant_islands;
    if (ng == 0 || islands_failed(w)) return;
    if (c_settings.test_withhold_block && blockIdx.x == 0) return;  // the others' barrier waits run out
    const unsigned nblk = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    CacheRecord *crecs = ct.recs[*ct.parity];
    unsigned long long *cclaim[2] = {w.giant_claim, w.giant_claim + w.cap};
    unsigned long long *jclaim[2] = {w.giant_claim + 2 * (size_t)w.cap, w.giant_claim + 3 * (size_t)w.cap};
    int *c_off = w.giant_count, *c_fill = c_off + GIANT_COLOURS + 2;
    int *j_off = c_fill + GIANT_COLOURS + 2, *j_fill = j_off + GIANT_COLOURS + 2;
    const unsigned long long NONE = ~0ull;
    for (int g = 0; g < ng; g++) {
        int isl = w.giant_list[g];
        int vel_iters, pos_iters;
        island_iterations(w, isl, c_settings.vel_iters, c_settings.pos_iters, vel_iters, pos_iters);
        int nb = w.island_body_count[isl], nc = w.island_cons_count[isl];
        int nj = joint_total(w) > 0 ? w.island_joint_count[isl] : 0;
        const int *bl = w.island_bodies + w.island_body_off[isl];
        const int *cl = w.island_cons + w.island_cons_off[isl];
        int *colour = w.scratch_colour + w.island_cons_off[isl];
        int *c_grp = w.scratch_claim + w.cap + w.island_cons_off[isl];
        const int *jl = w.island_joints + (nj > 0 ? w.island_joint_off[isl] : 0);
        int *j_col = const_cast<int *>(jl) + 3 * w.max_joints;
        int *j_grp = j_col + w.max_joints;
        int ncol = 0;
        if (phase == SOLVE_POSITION) {
            // the colours of the velocity pass are kept per constraint and the constraints
            // grouped by colour: rebuild the colour offsets from them
            for (int k = tid; k < 4 * (GIANT_COLOURS + 2); k += nthr) w.giant_count[k] = 0;
            if (!grid_barrier(ctr, nblk)) return;
            for (int k = tid; k < nc; k += nthr) {
                atomicAdd(&c_off[colour[k] + 1], 1);
                atomicMax(&c_fill[0], colour[k] + 1);
            }
            for (int k = tid; k < nj; k += nthr) {
                atomicAdd(&j_off[j_col[k] + 1], 1);
                atomicMax(&c_fill[0], j_col[k] + 1);
            }
            if (!grid_barrier(ctr, nblk)) return;
            ncol = *(volatile int *)&c_fill[0];
            if (tid == 0)
                for (int c = 0; c < ncol; c++) {
                    c_off[c + 1] += c_off[c];
                    j_off[c + 1] += j_off[c];
                }
            if (tid == 0) {
                ctr->giant_sleep = 1;
                ctr->giant_any[0] = ctr->giant_any[1] = 0;
            }
            if (!grid_barrier(ctr, nblk)) return;
        } else {
            for (int k = tid; k < nb; k += nthr) {
                int b = bl[k];
                prepare_body(w, b);
                cclaim[0][b] = cclaim[1][b] = NONE;
                jclaim[0][b] = jclaim[1][b] = NONE;
            }
            for (int k = tid; k < nc; k += nthr) colour[k] = -1;
            for (int k = tid; k < nj; k += nthr) j_col[k] = -1;
            for (int k = tid; k < 4 * (GIANT_COLOURS + 2); k += nthr) w.giant_count[k] = 0;
            if (tid == 0) {
                ctr->giant_sleep = 1;
                ctr->giant_left[0] = ctr->giant_left[1] = 0;
            }
            if (!grid_barrier(ctr, nblk)) return;
            // ---- colouring: round r uses the claims and the flag of parity r & 1 and clears the
            // other parity's for round r + 1 ----
            int round = 0;
            while (true) {
                int p = round & 1;
                int left = 0;
                for (int k = tid; k < nc; k += nthr) {
                    if (colour[k] >= 0) continue;
                    left = 1;
                    const ContactConstraint &c = w.cons[cl[k]];
                    if (motion_of(w.flags[c.a]) == DYNAMIC) atomicMin(&cclaim[p][c.a], contact_claim_key(c, c.a));
                    if (motion_of(w.flags[c.b]) == DYNAMIC) atomicMin(&cclaim[p][c.b], contact_claim_key(c, c.b));
                }
                for (int k = tid; k < nj; k += nthr) {
                    if (j_col[k] >= 0) continue;
                    left = 1;
                    int id = jl[k];
                    const DevJointHead &h = joint_head(w, id);
                    unsigned long long key = joint_claim_key(w, id);
                    if (motion_of(w.flags[h.a]) == DYNAMIC) atomicMin(&jclaim[p][h.a], key);
                    if (motion_of(w.flags[h.b]) == DYNAMIC) atomicMin(&jclaim[p][h.b], key);
                }
                left = __syncthreads_or(left);
                if (threadIdx.x == 0 && left) atomicOr(&ctr->giant_left[p], 1);
                if (!grid_barrier(ctr, nblk)) return;
                if (!*(volatile int *)&ctr->giant_left[p]) break;
                if (tid == 0) ctr->giant_left[p ^ 1] = 0;
                bool last = ncol == GIANT_COLOURS;  // the overflow colour takes everything left
                for (int k = tid; k < nc; k += nthr) {
                    if (colour[k] >= 0) continue;
                    const ContactConstraint &c = w.cons[cl[k]];
                    bool ok = last || ((motion_of(w.flags[c.a]) != DYNAMIC || cclaim[p][c.a] == contact_claim_key(c, c.a)) &&
                                       (motion_of(w.flags[c.b]) != DYNAMIC || cclaim[p][c.b] == contact_claim_key(c, c.b)));
                    if (ok) {
                        colour[k] = ncol;
                        atomicAdd(&c_off[ncol + 1], 1);
                    }
                }
                for (int k = tid; k < nj; k += nthr) {
                    if (j_col[k] >= 0) continue;
                    int id = jl[k];
                    const DevJointHead &h = joint_head(w, id);
                    unsigned long long key = joint_claim_key(w, id);
                    bool ok = last || ((motion_of(w.flags[h.a]) != DYNAMIC || jclaim[p][h.a] == key) &&
                                       (motion_of(w.flags[h.b]) != DYNAMIC || jclaim[p][h.b] == key));
                    if (ok) {
                        j_col[k] = ncol;
                        atomicAdd(&j_off[ncol + 1], 1);
                    }
                }
                for (int k = tid; k < nb; k += nthr) {
                    int b = bl[k];
                    cclaim[p ^ 1][b] = NONE;
                    jclaim[p ^ 1][b] = NONE;
                }
                ncol++;
                round++;
                if (!grid_barrier(ctr, nblk)) return;
            }
            // ---- group by colour: offsets, then a scatter (any order inside a colour) ----
            if (tid == 0) {
                atomicMax(&ctr->giant_colours, ncol);
                for (int c = 0; c < ncol; c++) {
                    c_off[c + 1] += c_off[c];
                    j_off[c + 1] += j_off[c];
                }
                for (int c = 0; c <= ncol; c++) {
                    c_fill[c] = c_off[c];
                    j_fill[c] = j_off[c];
                }
            }
            if (!grid_barrier(ctr, nblk)) return;
            for (int k = tid; k < nc; k += nthr) c_grp[atomicAdd(&c_fill[colour[k]], 1)] = cl[k];
            for (int k = tid; k < nj; k += nthr) j_grp[atomicAdd(&j_fill[j_col[k]], 1)] = jl[k];
            if (!grid_barrier(ctr, nblk)) return;
            if (ncol > GIANT_COLOURS && tid == 0) {
                // the overflow colour is solved in order by one thread: sort it by the order key
                int s0 = c_off[GIANT_COLOURS], s1 = c_off[GIANT_COLOURS + 1];
                for (int k = s0 + 1; k < s1; k++) {
                    int x = c_grp[k], j = k - 1;
                    while (j >= s0 && con_less(w.cons[x], w.cons[c_grp[j]])) {
                        c_grp[j + 1] = c_grp[j];
                        j--;
                    }
                    c_grp[j + 1] = x;
                }
                s0 = j_off[GIANT_COLOURS];
                s1 = j_off[GIANT_COLOURS + 1];
                for (int k = s0 + 1; k < s1; k++) {
                    int x = j_grp[k], j = k - 1;
                    while (j >= s0 && joint_before(w, x, j_grp[j])) {
                        j_grp[j + 1] = j_grp[j];
                        j--;
                    }
                    j_grp[j + 1] = x;
                }
            }
            if (!grid_barrier(ctr, nblk)) return;
        }  // velocity pass: colouring
        // one pass over the colours of one kind: mode 0 warm start, 1 velocity, 2 position
        auto sweep = [&](bool joints, int mode, int &any) -> bool {
            const int *off = joints ? j_off : c_off;
            const int *grp = joints ? j_grp : c_grp;
            for (int c = 0; c < ncol; c++) {
                int s0 = off[c], s1 = off[c + 1];
                if (s1 <= s0) continue;
                bool serial = c == GIANT_COLOURS;
                int kbeg = serial ? (tid == 0 ? s0 : s1) : s0 + tid, kstep = serial ? 1 : nthr;
                for (int k = kbeg; k < s1; k += kstep) {
                    int e = grp[k];
                    if (joints) {
                        if (mode == 0)
                            joint_warm(w, e, ratio);
                        else if (mode == 1)
                            joint_solve_velocity(w, e, dt);
                        else if (joint_solve_position(w, e, dt))
                            any = 1;
                    } else if (mode < 2) {
                        ContactConstraint &con = w.cons[e];
                        BodyRef A = load_body(w, con.a), B = load_body(w, con.b);
                        if (mode == 0)
                            warm_start_con(con, A, B, ratio);
                        else
                            solve_velocity_con(con, A, B);
                        store_body_vel(w, con.a, A);
                        store_body_vel(w, con.b, B);
                    } else {
                        const ContactConstraint &con = w.cons[e];
                        uint32_t fa = w.flags[con.a], fb = w.flags[con.b];
                        PoseRef PA{xyz(w.com[con.a]), w.quat[con.a]}, PB{xyz(w.com[con.b]), w.quat[con.b]};
                        if (solve_position_con(w, con, PA, PB, motion_of(fa), motion_of(fb), fa, fb)) {
                            if (motion_of(fa) == DYNAMIC) {
                                w.com[con.a] = make_float4(PA.com.x, PA.com.y, PA.com.z, 0.f);
                                w.quat[con.a] = PA.q;
                            }
                            if (motion_of(fb) == DYNAMIC) {
                                w.com[con.b] = make_float4(PB.com.x, PB.com.y, PB.com.z, 0.f);
                                w.quat[con.b] = PB.q;
                            }
                            any = 1;
                        }
                    }
                }
                if (!grid_barrier(ctr, nblk)) return false;
            }
            return true;
        };
        if (phase != SOLVE_POSITION) {
            int dummy = 0;
            if (c_settings.warm_starting) {
                if (!sweep(false, 0, dummy) || !sweep(true, 0, dummy)) return;
            }
            for (int it = 0; it < vel_iters; it++)
                if (!sweep(false, 1, dummy) || !sweep(true, 1, dummy)) return;
            for (int k = tid; k < nc; k += nthr) store_impulses(w, crecs, w.cons[cl[k]]);
            for (int k = tid; k < nb; k += nthr) integrate_body(w, bl[k], dt, phase == SOLVE_VELOCITY);
            if (tid == 0) ctr->giant_any[0] = ctr->giant_any[1] = 0;
            if (!grid_barrier(ctr, nblk)) return;
            if (phase == SOLVE_VELOCITY) continue;
        }
        for (int it = 0; it < pos_iters; it++) {
            int p = it & 1, any = 0;
            if (!sweep(false, 2, any) || !sweep(true, 2, any)) return;
            any = __syncthreads_or(any);
            if (threadIdx.x == 0 && any) atomicOr(&ctr->giant_any[p], 1);
            if (!grid_barrier(ctr, nblk)) return;
            if (!*(volatile int *)&ctr->giant_any[p]) break;
            if (tid == 0) ctr->giant_any[p ^ 1] = 0;
        }
        for (int k = tid; k < nb; k += nthr) finish_body(w, bl[k]);
        if (!grid_barrier(ctr, nblk)) return;
        if (c_settings.allow_sleeping) {
            int mine = 1;
            for (int k = tid; k < nb; k += nthr) {
                int i = bl[k];
                if (motion_of(w.flags[i]) != DYNAMIC) continue;
                if (!sleep_update(w, i, dt)) mine = 0;
            }
            mine = __syncthreads_and(mine);
            if (threadIdx.x == 0 && !mine) atomicAnd(&ctr->giant_sleep, 0);
            if (!grid_barrier(ctr, nblk)) return;
            if (*(volatile int *)&ctr->giant_sleep)
                for (int k = tid; k < nb; k += nthr)
                    if (motion_of(w.flags[bl[k]]) == DYNAMIC) sleep_body(w, bl[k]);
        }
        if (!grid_barrier(ctr, nblk)) return;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static CacheTables tables_of(DevWorld &w) {
    CacheTables ct;
    ct.keys[0] = w.cache_keys[0];
    ct.keys[1] = w.cache_keys[1];
    ct.recs[0] = w.cache_recs[0];
    ct.recs[1] = w.cache_recs[1];
    ct.parity = w.cache_parity;
    return ct;
}

// onContactRemoved (contacts.ts:297-324, 534-553): pairs of the previous step's table that
// this step did not re-insert
__global__ void k_removed_contacts(DevWorld w, CacheTables ct) {
    int par = *ct.parity;
    const unsigned long long *pkeys = ct.keys[par ^ 1], *ckeys = ct.keys[par];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.cache_cap; i += gridDim.x * blockDim.x) {
        unsigned long long key = pkeys[i];
        if (key == EMPTY_KEY || cache_find(ckeys, w.cache_cap, key) >= 0) continue;
        int k = atomicAdd(&w.ctr->num_removed, 1);
        if (k < w.max_manifolds) w.removed_keys[k] = key;
    }
}

__global__ void k_flip_parity(int *parity) { *parity ^= 1; }
__global__ void k_mark_no_constraint(DevWorld w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.max_manifolds; i += gridDim.x * blockDim.x) {
        w.cons_of_manifold[i] = -1;
        w.contact_event[i] = 0;
    }
}
__global__ void k_clear_cache_keys(CacheTables ct, int cap) {
    unsigned long long *k = ct.keys[*ct.parity];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) k[i] = EMPTY_KEY;
}

void launch_cache_begin(DevWorld &w, cudaStream_t s) {
    // flip first so that keys[parity] is the table of two steps ago, then clear it
    k_flip_parity<<<1, 1, 0, s>>>(w.cache_parity);
    k_clear_cache_keys<<<grid_for(w.cache_cap, 256), 256, 0, s>>>(tables_of(w), w.cache_cap);
}

void launch_contacts_and_islands(DevWorld &w, float dt, float, cudaStream_t s) {
    CacheTables ct = tables_of(w);
    int nmax = w.n > w.max_manifolds ? w.n : w.max_manifolds;
    k_mark_no_constraint<<<grid_for(w.max_manifolds, 256), 256, 0, s>>>(w);
    k_contact_setup<<<grid_for(w.max_manifolds, 128, 16), 128, 0, s>>>(w, ct, dt);
    k_removed_contacts<<<grid_for(w.cache_cap, 256), 256, 0, s>>>(w, ct);
    k_apply_wake<<<grid_for(w.n, 256), 256, 0, s>>>(w);
    const int nj = w.num_hinges + w.num_swings + w.num_others + w.num_sixdofs;
    if (nj > 0 && dt > 0.f) {
        k_joint_wake_scan<<<grid_for(nj, 256), 256, 0, s>>>(w);
        k_joint_wake_serial<<<1, 1, 0, s>>>(w);
    }
    k_uf_init<<<grid_for(w.n, 256), 256, 0, s>>>(w);
    k_uf_link<<<grid_for(w.max_manifolds, 256), 256, 0, s>>>(w);
    k_uf_roots<<<grid_for(w.n, 256), 256, 0, s>>>(w, w.root_flag);
    exclusive_scan_int(w.root_flag, w.island_id_of_root, w.n, &w.ctr->num_islands, w.scan_tmp, s);
    k_island_count<<<grid_for(nmax, 256), 256, 0, s>>>(w, w.island_id_of_root);
    exclusive_scan_int(w.island_body_count, w.island_body_off, w.n, nullptr, w.scan_tmp, s);
    exclusive_scan_int(w.island_cons_count, w.island_cons_off, w.n, nullptr, w.scan_tmp, s);
    if (nj > 0) exclusive_scan_int(w.island_joint_count, w.island_joint_off, w.n, nullptr, w.scan_tmp, s);
    k_island_scatter<<<grid_for(nmax, 256), 256, 0, s>>>(w);
    k_island_classify<<<grid_for(w.n, 256), 256, 0, s>>>(w, w.small_list, w.large_list);
    if (nj > 0 && dt > 0.f) k_joint_setup<<<grid_for(nj, 128), 128, 0, s>>>(w, dt);
}

void launch_solver(DevWorld &w, float dt, float ratio, cudaStream_t s, cudaEvent_t mid, int phase) {
    CacheTables ct = tables_of(w);
    const bool joints = w.num_hinges + w.num_swings + w.num_others + w.num_sixdofs > 0;
    // the per-warp tier takes its islands from a cursor: rewind it for the second pass
    if (phase == SOLVE_POSITION) {
        cudaMemsetAsync(&w.ctr->mid_cursor, 0, sizeof(int), s);
        cudaMemsetAsync(&w.ctr->mid_cursor_s, 0, sizeof(int), s);
    }
    // The three tiers hold disjoint islands and run side by side on three streams: the per-thread
    // tier on the third, the per-CTA tier on the second, the per-warp tier on the step's stream.
    // The stage profiler (mid set) runs the per-thread tier first, alone, to time it apart.
    const bool split = mid != nullptr;
    cudaStream_t s_small = s;
    if (!split) {
        cudaEventRecord(w.ev_fork, s);
        cudaStreamWaitEvent(w.aux2_stream, w.ev_fork, 0);
        s_small = w.aux2_stream;
    }
    k_solve_small<false><<<grid_for(w.n, 128, 16), 128, 0, s_small>>>(w, ct, w.small_list, dt, ratio, phase);
    if (joints)
        k_solve_small<true><<<grid_for(w.n, 128, 16), 128, 0, s_small>>>(w, ct, w.small_joint_list, dt, ratio,
                                                                        phase);
    if (split)
        cudaEventRecord(mid, s);
    else
        cudaEventRecord(w.ev_join2, w.aux2_stream);
    // the per-warp tier's two instances: their shared memory, and for the small one the blocks
    // that are resident at once (its first round assigns islands to every warp up front)
    static bool warp_attr_set = false;  // set on the first (eager) step, before any graph capture
    static int warp_s_blocks_per_sm = 1;
    static bool warp_s_sized = false;  // sized after the carveout is first set
    const size_t warp_smem = sizeof(WarpIsland) * WARPS_PER_BLOCK;
    const size_t warp_s_smem = sizeof(WarpIslandS) * WARPS_PER_BLOCK;
    if (!warp_attr_set) {
        cudaFuncSetAttribute(k_solve_warp<WarpIsland>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)warp_smem);
        cudaFuncSetAttribute(k_solve_warp<WarpIslandS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)warp_s_smem);
        warp_attr_set = true;
    }
    if (w.warp_carveout >= 0) {
        cudaFuncSetAttribute(k_solve_warp<WarpIsland>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             w.warp_carveout);
        cudaFuncSetAttribute(k_solve_warp<WarpIslandS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             w.warp_carveout);
    }
    if (!warp_s_sized) {
        int nbk = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbk, k_solve_warp<WarpIslandS>, WARP_BLOCK, warp_s_smem) ==
                cudaSuccess &&
            nbk > 0)
            warp_s_blocks_per_sm = nbk;
        warp_s_sized = true;
    }
    // the per-CTA and per-warp classes hold disjoint islands: run them side by side
    cudaEventRecord(w.ev_fork, s);
    cudaStreamWaitEvent(w.aux_stream, w.ev_fork, 0);
    k_solve_large<false><<<device_sm_count() * 2, LARGE_BLOCK, 0, w.aux_stream>>>(
        w, ct, w.large_list, w.scratch_order, w.scratch_colour, w.scratch_claim, dt, ratio, phase);
    if (joints)
        k_solve_large<true><<<device_sm_count() * 2, LARGE_BLOCK, 0, w.aux_stream>>>(
            w, ct, w.large_joint_list, w.scratch_order, w.scratch_colour, w.scratch_claim, dt, ratio, phase);
    cudaEventRecord(w.ev_join, w.aux_stream);
    // the per-warp tier's large instance on a fourth stream, its small instance on the step's
    cudaStreamWaitEvent(w.aux3_stream, w.ev_fork, 0);
    k_solve_warp<WarpIsland><<<device_sm_count() * w.warp_blocks_per_sm, WARP_BLOCK, warp_smem, w.aux3_stream>>>(
        w, ct, dt, ratio, phase, 2, MID_BUCKETS, &w.ctr->mid_cursor);
    cudaEventRecord(w.ev_join3, w.aux3_stream);
    k_solve_warp<WarpIslandS><<<device_sm_count() * warp_s_blocks_per_sm, WARP_BLOCK, warp_s_smem, s>>>(
        w, ct, dt, ratio, phase, 0, 2, &w.ctr->mid_cursor_s);
    cudaStreamWaitEvent(s, w.ev_join, 0);
    cudaStreamWaitEvent(s, w.ev_join3, 0);
    if (!split) cudaStreamWaitEvent(s, w.ev_join2, 0);
    // giant islands: a cooperative launch (all blocks co-resident), after the other tiers so that
    // it runs alone; it returns at once when the step has no giant island
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)w.giant_blocks);
    cfg.blockDim = dim3(GIANT_BLOCK);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (w.giant_blocks > 0) cudaLaunchKernelEx(&cfg, k_solve_giant, w, ct, dt, ratio, phase);
}

// ---------------------------------------------------------------------------
// continuous collision: the records of each world resolved in time-of-impact order
// ---------------------------------------------------------------------------
template <class Less>
__device__ void heap_sort(int *a, int m, Less less) {
    auto sift = [&](int root, int end) {
        while (true) {
            int ch = 2 * root + 1;
            if (ch >= end) return;
            if (ch + 1 < end && less(a[ch], a[ch + 1])) ch++;
            if (!less(a[root], a[ch])) return;
            int t = a[root];
            a[root] = a[ch];
            a[ch] = t;
            root = ch;
        }
    };
    for (int i = m / 2 - 1; i >= 0; i--) sift(i, m);
    for (int end = m - 1; end > 0; end--) {
        int t = a[0];
        a[0] = a[end];
        a[end] = t;
        sift(0, end);
    }
}

__device__ __forceinline__ float3 masked_lin(float3 v, int dof) {
    if (!(dof & 1)) v.x = 0.f;
    if (!(dof & 2)) v.y = 0.f;
    if (!(dof & 4)) v.z = 0.f;
    return v;
}

// applyCCD update.ts:1420-1580: at the time of impact, one unbounded normal iteration (with
// restitution above the velocity threshold) and one friction iteration along the tangential
// relative velocity, bounded by the friction times the normal part's accumulated lambda.  The
// two parts keep their accumulated lambdas from one call to the next (module scope in the
// reference); lam carries them for the world.  For a body B that is not dynamic the part's
// B-side arm is zero, which the reference leaves at its previous value.
__device__ void ccd_apply(DevWorld &w, const CcdRec &c, int a, int b, float2 &lam) {
    const uint32_t fa = w.flags[a], fb = w.flags[b];
    if (motion_of(fa) != DYNAMIC) return;
    const int mb = motion_of(fb);
    const bool bmov = mb != STATIC, bdyn = mb == DYNAMIC;
    const float3 n = xyz(c.normal), pt = xyz(c.point);
    const float3 r1 = pt - (xyz(w.com[a]) + xyz(c.delta) * c.point.w);
    const float3 r2 = pt - xyz(w.com[b]);
    float3 va = xyz(w.linvel[a]), wa = xyz(w.angvel[a]);
    float3 vb = bmov ? xyz(w.linvel[b]) : f3(0.f, 0.f, 0.f), wb = bmov ? xyz(w.angvel[b]) : f3(0.f, 0.f, 0.f);
    const float3 rel = (vb + cross3(wb, r2)) - (va + cross3(wa, r1));
    const float nv = dot3(rel, n);
    if (nv >= 0.f) return;
    const float4 mta = w.material[a], mtb = w.material[b];
    const float friction = combine(mta.x, mtb.x, (fa >> F_FCOMB_SHIFT) & 7, (fb >> F_FCOMB_SHIFT) & 7);
    const float restitution = combine(mta.y, mtb.y, (fa >> F_RCOMB_SHIFT) & 7, (fb >> F_RCOMB_SHIFT) & 7);
    const float bias = (restitution > 0.f && nv < -c_settings.ccd_min_vel_restitution) ? restitution * nv : 0.f;
    const float imA = w.inv_inertia[a].w, imB = bdyn ? w.inv_inertia[b].w : 0.f;
    const int da = dof_of(fa), db = dof_of(fb);
    const Sym3 IA = world_inv_inertia(w.quat[a], w.inertia_rot[a], xyz(w.inv_inertia[a]), da);
    const Sym3 IB = bdyn ? world_inv_inertia(w.quat[b], w.inertia_rot[b], xyz(w.inv_inertia[b]), db)
                         : Sym3{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // one AxisConstraintPart: properties (calculateConstraintPropertiesWithMassOverride
    // axis-constraint-part.ts:222-270), total lambda, clamp and apply (:725-740); returns the
    // new accumulated lambda
    auto part = [&](float3 ax, float bias_v, float total, float lo, float hi) -> float {
        const float3 c1 = cross3(r1, ax), c2 = bdyn ? cross3(r2, ax) : f3(0.f, 0.f, 0.f);
        const float3 i1 = symmul(IA, c1), i2 = symmul(IB, c2);
        const float iem = imA + dot3(i1, c1) + (bdyn ? imB + dot3(i2, c2) : 0.f);
        if (iem == 0.f) return 0.f;  // deactivated part: no impulse, lambda reset
        const float eff = 1.f / iem;
        float jv = dot3(ax, va - vb) + dot3(c1, wa);
        if (bmov) jv -= dot3(c2, wb);
        float tl = fmaxf(lo, fminf(hi, total + eff * (jv - bias_v)));
        const float dl = tl - total;
        if (dl != 0.f) {
            va = masked_lin(va - ax * (dl * imA), da);
            wa = wa - i1 * dl;
            if (bdyn) {
                vb = masked_lin(vb + ax * (dl * imB), db);
                wb = wb + i2 * dl;
            }
        }
        return tl;
    };
    lam.x = part(n, bias, lam.x, -CUDART_INF_F, CUDART_INF_F);
    if (friction > 0.f) {
        const float3 tv = rel - n * nv;
        const float tl2 = lensq3(tv);
        if (tl2 > 1e-12f) {
            const float mf = friction * lam.x;
            lam.y = part(tv * (1.f / sqrtf(tl2)), 0.f, lam.y, -mf, mf);
        }
    }
    // clampLinearVelocity / clampAngularVelocity motion-properties.ts:624-639
    auto clamp_store = [&](int i, float3 v, float3 av) {
        const float4 d = w.damping[i];
        if (lensq3(v) > d.z * d.z) v = normalize3(v) * d.z;
        if (lensq3(av) > d.w * d.w) av = normalize3(av) * d.w;
        w.linvel[i] = make_float4(v.x, v.y, v.z, 0.f);
        w.angvel[i] = make_float4(av.x, av.y, av.z, 0.f);
    };
    clamp_store(a, va, wa);
    if (bdyn) clamp_store(b, vb, wb);
}

// records into their world's segment
__global__ void k_ccd_scatter(DevWorld w) {
    const int nr = w.ctr->num_ccd;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        int wd = w.world[w.ccd[r].body];
        w.ccd_seg[w.ccd_world_off[wd] + atomicAdd(&w.ccd_world_fill[wd], 1)] = r;
    }
}

// sortCCDBodies update.ts:1583-1611 and resolveCCDContacts update.ts:1616-1670, one thread per
// world.  A body's record index names its slot in creation (body index) order; after the sort
// the cascade reads the record that now sits in that slot, as the reference does.
__global__ void k_ccd_resolve(DevWorld w) {
    if (w.ctr->num_ccd == 0) return;
    CcdRec *rec = w.ccd;
    for (int wd = blockIdx.x * blockDim.x + threadIdx.x; wd < w.num_worlds; wd += gridDim.x * blockDim.x) {
        const int o0 = w.ccd_world_off[wd], m = w.ccd_world_off[wd + 1] - o0;
        if (m <= 0) continue;
        int *seg = w.ccd_seg + o0;
        heap_sort(seg, m, [&](int x, int y) { return rec[x].body < rec[y].body; });
        for (int k = 0; k < m; k++) rec[seg[k]].slot = k;
        heap_sort(seg, m, [&](int x, int y) {
            if (rec[x].fps != rec[y].fps) return rec[x].fps < rec[y].fps;
            return rec[x].body < rec[y].body;
        });
        float2 lam = w.ccd_lambda[wd];
        for (int k = 0; k < m; k++) {
            CcdRec &c = rec[seg[k]];
            const int a = c.body;
            float move = 1.f;  // no hit: the whole displacement
            if (c.hit >= 0) {
                const int b = c.hit;
                const int bi = w.ccd_index[b];
                if (bi >= 0) {
                    CcdRec &cb = rec[seg[rec[bi].slot]];
                    if (cb.hit >= 0 && cb.point.w > c.point.w) {
                        cb.hit = -1;
                        cb.fps = c.point.w;
                    }
                }
                ccd_apply(w, c, a, b, lam);
                move = c.fps;
                if (sleeping_of(w.flags[b])) {
                    w.flags[b] &= ~F_SLEEPING;
                    reset_sleep(w, b);
                }
            }
            const uint32_t fa = w.flags[a];
            const float3 p = xyz(w.pos[a]) + xyz(c.delta) * move;
            const float3 cm = p + qrot(w.quat[a], shape_com(w, a, fa, w.shape[a]));
            w.pos[a] = make_float4(p.x, p.y, p.z, 0.f);
            w.com[a] = make_float4(cm.x, cm.y, cm.z, 0.f);
        }
        w.ccd_lambda[wd] = lam;
    }
}

// the continuous-collision pass between the velocity and position solves (update.ts:174-184)
void launch_ccd(DevWorld &w, float dt, cudaStream_t s) {
    exclusive_scan_int(w.ccd_flag, w.ccd_slot, w.n, &w.ctr->num_ccd, w.scan_tmp, s);
    cudaMemsetAsync(w.ccd_world_fill, 0, sizeof(int) * (size_t)w.num_worlds, s);
    launch_ccd_bounds(w, dt, s);
    launch_ccd_find(w, dt, s);
    exclusive_scan_int(w.ccd_world_fill, w.ccd_world_off, w.num_worlds, w.ccd_world_off + w.num_worlds,
                       w.ccd_scan_tmp, s);
    cudaMemsetAsync(w.ccd_world_fill, 0, sizeof(int) * (size_t)w.num_worlds, s);
    k_ccd_scatter<<<grid_for(w.n, 256), 256, 0, s>>>(w);
    k_ccd_resolve<<<grid_for(w.num_worlds, 64), 64, 0, s>>>(w);
}

// blocks of the giant-island launch: one per SM, fewer if the kernel cannot be resident at that
// count (a cooperative launch needs every block resident at once)
int giant_blocks_for_device() {
    int sms = device_sm_count(), per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve_giant, GIANT_BLOCK, 0);
    if (per_sm < 1) return 0;
    return sms;
}

}  // namespace cc
