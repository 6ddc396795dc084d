// Adjoint of a rollout: vector-Jacobian product of the velocity solve and the integration of
// every step over that step's fixed contact set.
//
// What is differentiated, per step and per awake dynamic body:
//   v1 = mask(ldf (v + a dt)),  w1 = mask(adf w)          force integration (update.ts:245-319)
//   warm start and PGS over the step's contact rows       contact-constraints.ts:906-1053
//   x += v2 dt                                            velocity integration (update.ts:896-976)
// The contact rows (normals, tangents, moment arms, effective masses, biases, world inverse
// inertias) and the position-solve corrections are constants of the step; the maximum-velocity
// clamps are taken as inactive.  The warm start of a step reads the previous step's final
// impulses through the contact cache match (contacts.ts:481-513, contact-constraints.ts:651-686),
// so impulse adjoints flow back across steps.  Friction coefficients enter through the friction
// disc radius mu * lambda_n (contact-constraints.ts:1001-1010) and the combine mode
// (combine-material.ts:40-57).  The loss is the sum over worlds of |centroid_w - target_w|^2 of
// the world's dynamic bodies after the last step.
//
// Inside an island one thread replays the solve in the reference's sequential order
// (sortContactIndices, contact-constraints.ts:1240-1264) keeping the pre-projection value u of
// every row update, then runs the exact reverse sweep; a row update
//   u = lambda + eff (J v - bias),  lambda' = P(u),  v' = v + M^-1 G^T (lambda' - lambda)
// (G = -J) reverses as
//   d_bar = G M^-1 v_bar',  u_bar = P'(u)^T (lambda'_bar + d_bar),
//   lambda_bar = u_bar - d_bar,  v_bar = v_bar' + eff u_bar J^T.
#include "cc_internal.cuh"

namespace cc {

static __constant__ DevSettings c_settings;

void upload_settings_adjoint(const DevSettings &s, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(c_settings, &s, sizeof(DevSettings), 0, cudaMemcpyHostToDevice, st);
}

constexpr int ROWS_PER_CON = 12;  // 4 points x (t1, t2, n)

// Impulse adjoints handed from a step to the step before it are keyed by the body pair
// (idA << 32 | idB, the contact cache key), in an open-addressing table of the adjoint's own:
// cache slot numbers depend on the order of concurrent inserts, so a segment recomputed from
// a checkpoint may place a pair elsewhere than the original forward did.
__device__ __forceinline__ unsigned int adj_hash(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (unsigned int)k;
}
__device__ int adj_find(const unsigned long long *keys, int cap, unsigned long long key) {
    unsigned int mask = (unsigned)cap - 1u, h = adj_hash(key) & mask;
    for (int probe = 0; probe < cap; probe++) {
        unsigned long long k = keys[h];
        if (k == key) return (int)h;
        if (k == EMPTY_KEY) return -1;
        h = (h + 1u) & mask;
    }
    return -1;
}
__device__ int adj_insert(unsigned long long *keys, int cap, unsigned long long key) {
    unsigned int mask = (unsigned)cap - 1u, h = adj_hash(key) & mask;
    for (int probe = 0; probe < cap; probe++) {
        unsigned long long prev = atomicCAS(&keys[h], EMPTY_KEY, key);
        if (prev == EMPTY_KEY || prev == key) return (int)h;
        h = (h + 1u) & mask;
    }
    return -1;
}
__device__ __forceinline__ unsigned long long pair_key(const ContactConstraint &c) {
    return ((unsigned long long)(unsigned)c.a << 32) | (unsigned)c.b;
}

// ---------------------------------------------------------------------------
// tape of one step, taken between the contact setup and the solver
// ---------------------------------------------------------------------------
__global__ void k_tape_record(DevWorld w, TapeStep t) {
    int nm = min(w.ctr->num_manifolds, w.max_manifolds);
    int ni = w.ctr->num_islands;
    int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (tid == 0) {
        t.counts[0] = nm;
        t.counts[1] = ni;
    }
    for (int i = tid; i < nm; i += stride) {
        int ci = w.cons_of_manifold[i];
        t.valid[i] = ci;
        if (ci >= 0) t.cons[ci] = w.cons[ci];
        t.isl_cons[i] = w.island_cons[i];
    }
    for (int i = tid; i < w.n; i += stride) {
        t.v[i] = w.linvel[i];
        t.w[i] = w.angvel[i];
        t.q[i] = w.quat[i];
        t.flags[i] = w.flags[i];
    }
    for (int i = tid; i < ni; i += stride) {
        t.isl_off[i] = w.island_cons_off[i];
        t.isl_cnt[i] = w.island_cons_count[i];
    }
}

void launch_tape_record(DevWorld &w, TapeStep &t, cudaStream_t s) {
    int nmax = w.max_manifolds > w.n ? w.max_manifolds : w.n;
    k_tape_record<<<grid_for(nmax, 256), 256, 0, s>>>(w, t);
}

// The tape of a finished step in the layout of cc_tape_body / cc_tape_contact
// (cc_world_step_taped): the rows as the velocity solve found them, and the final impulses
// that the solve stored into this step's cache record (storeAppliedImpulses,
// contact-constraints.ts:1061-1076).  A manifold without a constraint gets body_a = -1.
__global__ void k_tape_export(DevWorld w, TapeStep t, cc_tape_body *bodies, cc_tape_contact *cons) {
    const int nm = t.counts[0];
    const CacheRecord *recs = w.cache_recs[*w.cache_parity];
    int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (int i = tid; i < w.n; i += stride) {
        uint32_t f = t.flags[i];
        cc_tape_body b;
        float4 v = t.v[i], a = t.w[i];
        b.linear_velocity[0] = v.x;
        b.linear_velocity[1] = v.y;
        b.linear_velocity[2] = v.z;
        b.angular_velocity[0] = a.x;
        b.angular_velocity[1] = a.y;
        b.angular_velocity[2] = a.z;
        const bool dyn = motion_of(f) == DYNAMIC && !sleeping_of(f);
        Sym3 I{0, 0, 0, 0, 0, 0};
        if (dyn) I = world_inv_inertia(t.q[i], w.inertia_rot[i], xyz(w.inv_inertia[i]), dof_of(f));
        b.inv_inertia[0] = I.xx;
        b.inv_inertia[1] = I.xy;
        b.inv_inertia[2] = I.xz;
        b.inv_inertia[3] = I.yy;
        b.inv_inertia[4] = I.yz;
        b.inv_inertia[5] = I.zz;
        b.inv_mass = w.inv_inertia[i].w;
        b.flags = (dyn ? (uint32_t)CC_TAPE_DYNAMIC : 0u) | (motion_of(f) != STATIC ? (uint32_t)CC_TAPE_MOVING : 0u) |
                  ((uint32_t)dof_of(f) << 8);
        bodies[i] = b;
    }
    for (int i = tid; i < nm; i += stride) {
        cc_tape_contact o;
        int ci = t.valid[i];
        if (ci < 0) {
            o.body_a = o.body_b = -1;
            o.num_points = 0;
            cons[i] = o;
            continue;
        }
        const ContactConstraint &c = t.cons[ci];
        const CacheRecord &r = recs[c.cache_slot];
        o.body_a = c.a;
        o.body_b = c.b;
        o.num_points = c.n;
        o.island = c.island;
        o.has_prev = c.pad0 >= 0 ? 1 : 0;
        o.sort_key = c.sort_key;
        const float3 ax[3] = {c.normal, c.t1, c.t2};
        float *dst[3] = {o.normal, o.tangent1, o.tangent2};
        for (int k = 0; k < 3; k++) {
            dst[k][0] = ax[k].x;
            dst[k][1] = ax[k].y;
            dst[k][2] = ax[k].z;
        }
        o.friction = c.friction;
        o.inv_mass_a = c.invMassA;
        o.inv_mass_b = c.invMassB;
        for (int q = 0; q < 4; q++) {
            cc_tape_point &op = o.points[q];
            const ContactPoint &p = c.p[q < c.n ? q : 0];
            op.r_a[0] = p.rA.x;
            op.r_a[1] = p.rA.y;
            op.r_a[2] = p.rA.z;
            op.r_b[0] = p.rB.x;
            op.r_b[1] = p.rB.y;
            op.r_b[2] = p.rB.z;
            op.eff_normal = p.eff_n;
            op.eff_tangent1 = p.eff_t1;
            op.eff_tangent2 = p.eff_t2;
            op.bias_normal = p.bias_n;
            op.lambda_normal = p.lam_n;
            op.lambda_tangent1 = p.lam_t1;
            op.lambda_tangent2 = p.lam_t2;
            const int k = q < c.n ? q : 0;
            op.final_normal = r.ln[k];
            op.final_tangent1 = r.lt1[k];
            op.final_tangent2 = r.lt2[k];
            op.prev_point = q < c.n ? __float_as_int(p.pad) : -1;
        }
        cons[i] = o;
    }
}

void launch_tape_export(DevWorld &w, TapeStep &t, cc_tape_body *bodies, cc_tape_contact *cons, cudaStream_t s) {
    int nmax = w.max_manifolds > w.n ? w.max_manifolds : w.n;
    k_tape_export<<<grid_for(nmax, 256), 256, 0, s>>>(w, t, bodies, cons);
}

// ---------------------------------------------------------------------------
// checkpoints: body state plus the cache table the next step reads (the current parity)
// ---------------------------------------------------------------------------
__global__ void k_ckpt_cache(unsigned long long *keys0, unsigned long long *keys1, CacheRecord *recs0,
                             CacheRecord *recs1, int *parity, unsigned long long *ckeys, CacheRecord *crecs,
                             int *cparity, int cap, int save) {
    int p = save ? *parity : *cparity;
    unsigned long long *k = p ? keys1 : keys0;
    CacheRecord *r = p ? recs1 : recs0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        if (save) {
            unsigned long long key = k[i];
            ckeys[i] = key;
            if (key != EMPTY_KEY) crecs[i] = r[i];
        } else {
            unsigned long long key = ckeys[i];
            k[i] = key;
            if (key != EMPTY_KEY) r[i] = crecs[i];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (save)
            *cparity = p;
        else
            *parity = p;
    }
}

static void copy_body_state(const DevWorld &w, const Checkpoint &c, bool save, cudaStream_t s) {
    size_t n = (size_t)w.n;
    auto cp = [&](void *ck, void *live, size_t bytes) {
        cudaMemcpyAsync(save ? ck : live, save ? live : ck, bytes, cudaMemcpyDeviceToDevice, s);
    };
    cp(c.pos, w.pos, n * sizeof(float4));
    cp(c.quat, w.quat, n * sizeof(float4));
    cp(c.com, w.com, n * sizeof(float4));
    cp(c.linvel, w.linvel, n * sizeof(float4));
    cp(c.angvel, w.angvel, n * sizeof(float4));
    cp(c.force, w.force, n * sizeof(float4));
    cp(c.torque, w.torque, n * sizeof(float4));
    cp(c.sleep_sph, w.sleep_sph, 3 * n * sizeof(float4));
    cp(c.sleep_timer, w.sleep_timer, n * sizeof(float));
    cp(c.flags, w.flags, n * sizeof(uint32_t));
}

void checkpoint_save(const DevWorld &w, Checkpoint &c, cudaStream_t s) {
    copy_body_state(w, c, true, s);
    k_ckpt_cache<<<grid_for(w.cache_cap, 256), 256, 0, s>>>(w.cache_keys[0], w.cache_keys[1], w.cache_recs[0],
                                                            w.cache_recs[1], w.cache_parity, c.keys, c.recs,
                                                            c.parity, w.cache_cap, 1);
}
void checkpoint_restore(DevWorld &w, const Checkpoint &c, cudaStream_t s) {
    copy_body_state(w, c, false, s);
    k_ckpt_cache<<<grid_for(w.cache_cap, 256), 256, 0, s>>>(w.cache_keys[0], w.cache_keys[1], w.cache_recs[0],
                                                            w.cache_recs[1], w.cache_parity, c.keys, c.recs,
                                                            c.parity, w.cache_cap, 0);
}

// ---------------------------------------------------------------------------
// loss and its gradient with respect to the final positions
// ---------------------------------------------------------------------------
// Per-world sums of the dynamic bodies' positions in 40.24 fixed point: integer additions
// commute, so the sums (and the loss and its gradient) do not depend on the order in which
// threads add them.  sums: 4 per world (x, y, z, count).
constexpr float WS_SCALE = 16777216.f;  // 2^24: 6e-8 m resolution, +-5e11 m of summed range
__global__ void k_world_sums(DevWorld w, unsigned long long *sums) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        if (motion_of(w.flags[i]) != DYNAMIC) continue;
        float4 p = w.pos[i];
        unsigned long long *s = sums + 4 * (size_t)w.world[i];
        atomicAdd(&s[0], (unsigned long long)__float2ll_rn(p.x * WS_SCALE));
        atomicAdd(&s[1], (unsigned long long)__float2ll_rn(p.y * WS_SCALE));
        atomicAdd(&s[2], (unsigned long long)__float2ll_rn(p.z * WS_SCALE));
        atomicAdd(&s[3], 1ull);
    }
}
__device__ __forceinline__ float4 world_centroid(const unsigned long long *sums, int k) {
    const unsigned long long *s = sums + 4 * (size_t)k;
    float c = (float)(long long)s[3];
    if (!(c > 0.f)) return make_float4(0.f, 0.f, 0.f, 0.f);
    double inv = 1.0 / ((double)WS_SCALE * (double)c);
    return make_float4((float)((double)(long long)s[0] * inv), (float)((double)(long long)s[1] * inv),
                       (float)((double)(long long)s[2] * inv), c);
}
__global__ void k_loss(int nw, const unsigned long long *sums, const float *targets, float *loss) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nw; k += gridDim.x * blockDim.x) {
        float4 c = world_centroid(sums, k);
        float l = 0.f;
        if (c.w > 0.f) {
            float3 d = f3(c.x - targets[3 * k], c.y - targets[3 * k + 1], c.z - targets[3 * k + 2]);
            l = dot3(d, d);
        }
        loss[k] = l;
    }
}
__global__ void k_xbar(DevWorld w, const unsigned long long *sums, const float *targets, float4 *xbar) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        if (motion_of(w.flags[i]) == DYNAMIC) {
            int k = w.world[i];
            float4 c = world_centroid(sums, k);
            if (c.w > 0.f) {
                float sc = 2.f / c.w;
                g = make_float4((c.x - targets[3 * k]) * sc, (c.y - targets[3 * k + 1]) * sc,
                                (c.z - targets[3 * k + 2]) * sc, 0.f);
            }
        }
        xbar[i] = g;
    }
}

void launch_rollout_loss(const DevWorld &w, const float *targets, unsigned long long *sums, float *loss,
                         AdjBuffers &a, cudaStream_t s) {
    cudaMemsetAsync(sums, 0, sizeof(unsigned long long) * 4 * (size_t)w.num_worlds, s);
    k_world_sums<<<grid_for(w.n, 256), 256, 0, s>>>(w, sums);
    k_loss<<<grid_for(w.num_worlds, 256), 256, 0, s>>>(w.num_worlds, sums, targets, loss);
    k_xbar<<<grid_for(w.n, 256), 256, 0, s>>>(w, sums, targets, a.xbar);
    cudaMemsetAsync(a.vbar, 0, sizeof(float4) * (size_t)w.n, s);
    cudaMemsetAsync(a.wbar, 0, sizeof(float4) * (size_t)w.n, s);
    cudaMemsetAsync(a.mu_body, 0, sizeof(unsigned long long) * (size_t)w.n, s);
    cudaMemsetAsync(a.mu_con, 0, sizeof(float) * (size_t)w.max_manifolds, s);
}

// ---------------------------------------------------------------------------
// reverse of one step
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool awake_dynamic(uint32_t f) { return motion_of(f) == DYNAMIC && !sleeping_of(f); }

// v_bar after the solve gets dt x_bar (x += v dt); replay velocities and world inverse
// inertias of the step come from its tape
__global__ void k_adj_begin(DevWorld w, TapeStep t, AdjBuffers a, float dt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        uint32_t f = t.flags[i];
        a.vwork[i] = t.v[i];
        a.wwork[i] = t.w[i];
        if (awake_dynamic(f)) {
            float4 xb = a.xbar[i], vb = a.vbar[i];
            a.vbar[i] = make_float4(vb.x + dt * xb.x, vb.y + dt * xb.y, vb.z + dt * xb.z, 0.f);
            Sym3 I = world_inv_inertia(t.q[i], w.inertia_rot[i], xyz(w.inv_inertia[i]), dof_of(f));
            a.iw[2 * i] = make_float4(I.xx, I.xy, I.xz, I.yy);
            a.iw[2 * i + 1] = make_float4(I.yz, I.zz, 0.f, 0.f);
        } else {
            a.vbar[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.wbar[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.iw[2 * i] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.iw[2 * i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

struct AdjBody {
    int idx;
    bool movable;  // not static: its velocity enters J v
    bool dynamic;  // receives impulses and carries adjoints
    int dof;
    Sym3 I;
};
__device__ __forceinline__ AdjBody adj_body(const TapeStep &t, const AdjBuffers &a, int i) {
    AdjBody b;
    uint32_t f = t.flags[i];
    b.idx = i;
    b.movable = motion_of(f) != STATIC;
    b.dynamic = awake_dynamic(f);
    b.dof = dof_of(f);
    float4 p = a.iw[2 * i], q = a.iw[2 * i + 1];
    b.I = Sym3{p.x, p.y, p.z, p.w, q.x, q.y};
    return b;
}
__device__ __forceinline__ float3 mask_lin3(float3 v, int dof) {
    return f3((dof & 1) ? v.x : 0.f, (dof & 2) ? v.y : 0.f, (dof & 4) ? v.z : 0.f);
}

// one row of a contact point: axis and the two moment-arm crosses
struct Row {
    float3 ax, cA, cB;
};
__device__ __forceinline__ Row make_row(float3 ax, const ContactPoint &p) {
    return Row{ax, cross3(p.rA, ax), cross3(p.rB, ax)};
}

// J v (getTotalLambda axis-constraint-part.ts:578-625)
__device__ __forceinline__ float row_jv(const AdjBody &A, const AdjBody &B, const AdjBuffers &a, const Row &r) {
    float jv = 0.f;
    if (A.movable) jv += dot3(r.ax, xyz(a.vwork[A.idx])) + dot3(r.cA, xyz(a.wwork[A.idx]));
    if (B.movable) jv -= dot3(r.ax, xyz(a.vwork[B.idx])) + dot3(r.cB, xyz(a.wwork[B.idx]));
    return jv;
}
// v += M^-1 G^T d (applyLambda axis-constraint-part.ts:640-707)
__device__ __forceinline__ void row_apply(const AdjBody &A, const AdjBody &B, AdjBuffers &a, float imA, float imB,
                                          const Row &r, float d) {
    if (d == 0.f) return;
    if (A.dynamic) {
        float3 v = mask_lin3(xyz(a.vwork[A.idx]) - r.ax * (d * imA), A.dof);
        float3 w = xyz(a.wwork[A.idx]) - symmul(A.I, r.cA) * d;
        a.vwork[A.idx] = make_float4(v.x, v.y, v.z, 0.f);
        a.wwork[A.idx] = make_float4(w.x, w.y, w.z, 0.f);
    }
    if (B.dynamic) {
        float3 v = mask_lin3(xyz(a.vwork[B.idx]) + r.ax * (d * imB), B.dof);
        float3 w = xyz(a.wwork[B.idx]) + symmul(B.I, r.cB) * d;
        a.vwork[B.idx] = make_float4(v.x, v.y, v.z, 0.f);
        a.wwork[B.idx] = make_float4(w.x, w.y, w.z, 0.f);
    }
}
// adjoint of an applied impulse: G M^-1 v_bar
__device__ __forceinline__ float row_apply_bar(const AdjBody &A, const AdjBody &B, const AdjBuffers &a, float imA,
                                               float imB, const Row &r) {
    float g = 0.f;
    if (A.dynamic)
        g -= imA * dot3(mask_lin3(r.ax, A.dof), xyz(a.vbar[A.idx])) + dot3(symmul(A.I, r.cA), xyz(a.wbar[A.idx]));
    if (B.dynamic)
        g += imB * dot3(mask_lin3(r.ax, B.dof), xyz(a.vbar[B.idx])) + dot3(symmul(B.I, r.cB), xyz(a.wbar[B.idx]));
    return g;
}
// adjoint through J v: v_bar += s J^T (dynamic bodies only; the others' velocities are constants)
__device__ __forceinline__ void row_jv_bar(const AdjBody &A, const AdjBody &B, AdjBuffers &a, const Row &r,
                                           float s) {
    if (s == 0.f) return;
    if (A.dynamic) {
        float4 v = a.vbar[A.idx], w = a.wbar[A.idx];
        a.vbar[A.idx] = make_float4(v.x + r.ax.x * s, v.y + r.ax.y * s, v.z + r.ax.z * s, 0.f);
        a.wbar[A.idx] = make_float4(w.x + r.cA.x * s, w.y + r.cA.y * s, w.z + r.cA.z * s, 0.f);
    }
    if (B.dynamic) {
        float4 v = a.vbar[B.idx], w = a.wbar[B.idx];
        a.vbar[B.idx] = make_float4(v.x - r.ax.x * s, v.y - r.ax.y * s, v.z - r.ax.z * s, 0.f);
        a.wbar[B.idx] = make_float4(w.x - r.cB.x * s, w.y - r.cB.y * s, w.z - r.cB.z * s, 0.f);
    }
}

// friction disc projection (contact-constraints.ts:1001-1010)
__device__ __forceinline__ void friction_project(float u1, float u2, float mf, float &l1, float &l2) {
    l1 = u1;
    l2 = u2;
    float fm = u1 * u1 + u2 * u2;
    if (fm > mf * mf) {
        float s = mf / sqrtf(fm);
        l1 *= s;
        l2 *= s;
    }
}

__device__ __forceinline__ bool friction_active(const ContactPoint &p) { return p.eff_t1 != 0.f || p.eff_t2 != 0.f; }

// impulses of point q after velocity iteration `it` (it = -1: at the start of the iterations)
struct Lam3 {
    float t1, t2, n;
};
__device__ Lam3 lam_after(const ContactConstraint &c, int q, int it, const float *u_tape, size_t stride_it,
                          size_t row0, float ratio) {
    const ContactPoint &p = c.p[q];
    float s = c_settings.warm_starting ? ratio : 1.f;
    Lam3 start{p.lam_t1 * s, p.lam_t2 * s, p.lam_n * s};
    if (it < 0) return start;
    const float *u = u_tape + (size_t)it * stride_it + row0 + 3 * q;
    Lam3 r;
    r.n = fmaxf(0.f, u[2]);
    if (friction_active(p)) {
        // the disc radius of iteration `it` used lambda_n after iteration it - 1
        float lnb = it > 0 ? fmaxf(0.f, (u_tape + (size_t)(it - 1) * stride_it + row0 + 3 * q)[2]) : start.n;
        friction_project(u[0], u[1], c.friction * lnb, r.t1, r.t2);
    } else {
        r.t1 = r.t2 = 0.f;
    }
    return r;
}

// d combine(a, b) / da and / db for the friction combine modes (combine-material.ts:40-57)
__device__ void combine_grad_friction(float a, float b, int ma, int mb, float &da, float &db) {
    const int prio[5] = {0, 1, 3, 4, 2};
    int mode = prio[ma] >= prio[mb] ? ma : mb;
    switch (mode) {
        case 1:  // multiply
            da = b;
            db = a;
            break;
        case 2:  // min
            da = a <= b ? 1.f : 0.f;
            db = a <= b ? 0.f : 1.f;
            break;
        case 3:  // max
            da = a >= b ? 1.f : 0.f;
            db = a >= b ? 0.f : 1.f;
            break;
        case 4: {  // geometric mean
            float m = sqrtf(a * b);
            da = m > 0.f ? 0.5f * b / m : 0.f;
            db = m > 0.f ? 0.5f * a / m : 0.f;
            break;
        }
        default:  // average
            da = db = 0.5f;
    }
}

__device__ __forceinline__ bool con_before(const ContactConstraint &x, const ContactConstraint &y) {
    if (x.sort_key != y.sort_key) return x.sort_key < y.sort_key;
    if (x.a != y.a) return x.a < y.a;
    return x.b < y.b;
}

// One island per thread: replay (warm start, velocity iterations) in the reference's order, then
// the reverse.  lam_bar of a constraint starts as the adjoint of its final impulses, which the
// next step's reverse left at the constraint's cache slot.
__global__ void k_adj_islands(DevWorld w, TapeStep t, AdjBuffers a, float ratio, AdjHandoff in, AdjHandoff out) {
    const int ni = t.counts[1];
    const int iters = c_settings.vel_iters;
    const size_t stride_it = (size_t)t.counts[0] * ROWS_PER_CON;
    const bool warm = c_settings.warm_starting != 0;
    for (int isl = blockIdx.x * blockDim.x + threadIdx.x; isl < ni; isl += gridDim.x * blockDim.x) {
        int off = t.isl_off[isl], nc = t.isl_cnt[isl];
        if (nc == 0) continue;
        int *ord = t.isl_cons + off;
        for (int k = 1; k < nc; k++) {
            int x = ord[k];
            int j = k - 1;
            while (j >= 0 && con_before(t.cons[x], t.cons[ord[j]])) {
                ord[j + 1] = ord[j];
                j--;
            }
            ord[j + 1] = x;
        }
        // ---- replay: warm start (contact-constraints.ts:906-955)
        if (warm) {
            for (int k = 0; k < nc; k++) {
                const ContactConstraint &c = t.cons[ord[k]];
                AdjBody A = adj_body(t, a, c.a), B = adj_body(t, a, c.b);
                for (int q = 0; q < c.n; q++) {
                    const ContactPoint &p = c.p[q];
                    if (friction_active(p)) {
                        row_apply(A, B, a, c.invMassA, c.invMassB, make_row(c.t1, p), p.lam_t1 * ratio);
                        row_apply(A, B, a, c.invMassA, c.invMassB, make_row(c.t2, p), p.lam_t2 * ratio);
                    }
                    row_apply(A, B, a, c.invMassA, c.invMassB, make_row(c.normal, p), p.lam_n * ratio);
                }
            }
        }
        // ---- replay: velocity iterations (contact-constraints.ts:963-1053), keeping u
        for (int it = 0; it < iters; it++) {
            for (int k = 0; k < nc; k++) {
                int ci = ord[k];
                const ContactConstraint &c = t.cons[ci];
                AdjBody A = adj_body(t, a, c.a), B = adj_body(t, a, c.b);
                if (!A.dynamic && !B.dynamic) continue;
                size_t row0 = (size_t)ci * ROWS_PER_CON;
                float *u = a.u_tape + (size_t)it * stride_it + row0;
                for (int q = 0; q < c.n; q++) {
                    const ContactPoint &p = c.p[q];
                    if (!friction_active(p)) continue;
                    Lam3 before = lam_after(c, q, it - 1, a.u_tape, stride_it, row0, ratio);
                    Row r1 = make_row(c.t1, p), r2 = make_row(c.t2, p);
                    float u1 = before.t1 + p.eff_t1 * row_jv(A, B, a, r1);
                    float u2 = before.t2 + p.eff_t2 * row_jv(A, B, a, r2);
                    u[3 * q] = u1;
                    u[3 * q + 1] = u2;
                    float l1, l2;
                    friction_project(u1, u2, c.friction * before.n, l1, l2);
                    row_apply(A, B, a, c.invMassA, c.invMassB, r1, l1 - before.t1);
                    row_apply(A, B, a, c.invMassA, c.invMassB, r2, l2 - before.t2);
                }
                for (int q = 0; q < c.n; q++) {
                    const ContactPoint &p = c.p[q];
                    Lam3 before = lam_after(c, q, it - 1, a.u_tape, stride_it, row0, ratio);
                    Row rn = make_row(c.normal, p);
                    float un = before.n + p.eff_n * (row_jv(A, B, a, rn) - p.bias_n);
                    u[3 * q + 2] = un;
                    row_apply(A, B, a, c.invMassA, c.invMassB, rn, fmaxf(0.f, un) - before.n);
                }
            }
        }
        // ---- reverse, starting from the adjoints of the final impulses
        for (int k = 0; k < nc; k++) {
            int ci = ord[k];
            const ContactConstraint &c = t.cons[ci];
            float *lb = a.lam_bar + (size_t)ci * ROWS_PER_CON;
            int h = adj_find(in.keys, w.cache_cap, pair_key(c));
            const float *sb = in.vals + (size_t)(h < 0 ? 0 : h) * ROWS_PER_CON;
            for (int r = 0; r < ROWS_PER_CON; r++) lb[r] = h < 0 ? 0.f : sb[r];
        }
        for (int it = iters - 1; it >= 0; it--) {
            for (int k = nc - 1; k >= 0; k--) {
                int ci = ord[k];
                const ContactConstraint &c = t.cons[ci];
                AdjBody A = adj_body(t, a, c.a), B = adj_body(t, a, c.b);
                if (!A.dynamic && !B.dynamic) continue;
                size_t row0 = (size_t)ci * ROWS_PER_CON;
                const float *u = a.u_tape + (size_t)it * stride_it + row0;
                float *lb = a.lam_bar + row0;
                for (int q = c.n - 1; q >= 0; q--) {  // normal rows, last point first
                    const ContactPoint &p = c.p[q];
                    Row rn = make_row(c.normal, p);
                    float db = row_apply_bar(A, B, a, c.invMassA, c.invMassB, rn);
                    float ub = u[3 * q + 2] > 0.f ? lb[3 * q + 2] + db : 0.f;
                    lb[3 * q + 2] = ub - db;
                    row_jv_bar(A, B, a, rn, p.eff_n * ub);
                }
                for (int q = c.n - 1; q >= 0; q--) {  // friction rows, last point first
                    const ContactPoint &p = c.p[q];
                    if (!friction_active(p)) continue;
                    Lam3 before = lam_after(c, q, it - 1, a.u_tape, stride_it, row0, ratio);
                    Row r1 = make_row(c.t1, p), r2 = make_row(c.t2, p);
                    float u1 = u[3 * q], u2 = u[3 * q + 1];
                    float mf = c.friction * before.n;
                    float d2b = row_apply_bar(A, B, a, c.invMassA, c.invMassB, r2);
                    float d1b = row_apply_bar(A, B, a, c.invMassA, c.invMassB, r1);
                    float g1 = lb[3 * q] + d1b, g2 = lb[3 * q + 1] + d2b;  // adjoints of the projected values
                    float ub1 = g1, ub2 = g2, mfb = 0.f;
                    float fm = u1 * u1 + u2 * u2;
                    if (fm > mf * mf) {
                        float len = sqrtf(fm);
                        float h1 = u1 / len, h2 = u2 / len;
                        float hg = h1 * g1 + h2 * g2;
                        float sc = mf / len;
                        ub1 = sc * (g1 - h1 * hg);
                        ub2 = sc * (g2 - h2 * hg);
                        mfb = hg;
                    }
                    lb[3 * q] = ub1 - d1b;
                    lb[3 * q + 1] = ub2 - d2b;
                    row_jv_bar(A, B, a, r1, p.eff_t1 * ub1);
                    row_jv_bar(A, B, a, r2, p.eff_t2 * ub2);
                    // the disc radius used lambda_n before this iteration's normal update, whose adjoint
                    // is lb[3q+2] at this point of the reverse sweep
                    lb[3 * q + 2] += mfb * c.friction;
                    a.mu_con[ci] += mfb * before.n;
                }
            }
        }
        // ---- reverse of the warm start: start impulses, then back to the previous step's cache slots
        for (int k = nc - 1; k >= 0; k--) {
            int ci = ord[k];
            const ContactConstraint &c = t.cons[ci];
            AdjBody A = adj_body(t, a, c.a), B = adj_body(t, a, c.b);
            const float *lb = a.lam_bar + (size_t)ci * ROWS_PER_CON;
            int prev = c.pad0;
            int slot = -1;  // the pair's entry in the hand-off table (the previous step had this pair)
            if (warm && prev >= 0 && ratio != 0.f) {
                slot = adj_insert(out.keys, w.cache_cap, pair_key(c));
                if (slot < 0) continue;
            }
            for (int q = 0; q < c.n; q++) {
                const ContactPoint &p = c.p[q];
                int j = __float_as_int(p.pad);
                if (slot < 0 || j < 0) continue;
                float g[3];
                g[2] = lb[3 * q + 2] + row_apply_bar(A, B, a, c.invMassA, c.invMassB, make_row(c.normal, p));
                g[0] = g[1] = 0.f;
                if (friction_active(p)) {
                    g[0] = lb[3 * q] + row_apply_bar(A, B, a, c.invMassA, c.invMassB, make_row(c.t1, p));
                    g[1] = lb[3 * q + 1] + row_apply_bar(A, B, a, c.invMassA, c.invMassB, make_row(c.t2, p));
                }
                // rows whose effective mass is zero were reset in the setup: no adjoint flows back
                float *o = out.vals + (size_t)slot * ROWS_PER_CON + 3 * j;
                if (p.eff_t1 != 0.f) o[0] += ratio * g[0];
                if (p.eff_t2 != 0.f) o[1] += ratio * g[1];
                if (p.eff_n != 0.f) o[2] += ratio * g[2];
            }
        }
    }
}

// friction adjoint of each constraint to its two bodies through the combine mode
__global__ void k_adj_mu(DevWorld w, TapeStep t, AdjBuffers a) {
    int nm = t.counts[0];
    for (int ci = blockIdx.x * blockDim.x + threadIdx.x; ci < nm; ci += gridDim.x * blockDim.x) {
        if (t.valid[ci] < 0) continue;
        float g = a.mu_con[ci];
        if (g == 0.f) continue;
        a.mu_con[ci] = 0.f;
        const ContactConstraint &c = t.cons[ci];
        uint32_t fa = w.flags[c.a], fb = w.flags[c.b];
        float da, db;
        combine_grad_friction(w.material[c.a].x, w.material[c.b].x, (fa >> F_FCOMB_SHIFT) & 7,
                              (fb >> F_FCOMB_SHIFT) & 7, da, db);
        // integer sums: the same result whatever order the constraints of a body arrive in
        atomicAdd(&a.mu_body[c.a], (unsigned long long)__double2ll_rn((double)(g * da) * ADJ_MU_SCALE));
        atomicAdd(&a.mu_body[c.b], (unsigned long long)__double2ll_rn((double)(g * db) * ADJ_MU_SCALE));
    }
}

// reverse of the force integration: v_bar <- ldf mask(v_bar), w_bar <- adf mask(w_bar)
__global__ void k_adj_force(DevWorld w, TapeStep t, AdjBuffers a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        uint32_t f = t.flags[i];
        if (!awake_dynamic(f)) {
            a.vbar[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            a.wbar[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        int dof = dof_of(f);
        float4 d = w.damping[i];
        float dt = a.dt;
        float ldf = fmaxf(0.f, 1.f - d.x * dt), adf = fmaxf(0.f, 1.f - d.y * dt);
        float3 v = mask_lin3(xyz(a.vbar[i]), dof) * ldf;
        float3 av = xyz(a.wbar[i]);
        av = f3((dof & 8) ? av.x : 0.f, (dof & 16) ? av.y : 0.f, (dof & 32) ? av.z : 0.f) * adf;
        a.vbar[i] = make_float4(v.x, v.y, v.z, 0.f);
        a.wbar[i] = make_float4(av.x, av.y, av.z, 0.f);
    }
}

void launch_adjoint_step(DevWorld &w, TapeStep &t, AdjBuffers &a, float dt, float ratio, const AdjHandoff &in,
                         const AdjHandoff &out, cudaStream_t s) {
    a.dt = dt;
    k_adj_begin<<<grid_for(w.n, 256), 256, 0, s>>>(w, t, a, dt);
    cudaMemsetAsync(out.keys, 0xff, sizeof(unsigned long long) * (size_t)w.cache_cap, s);
    cudaMemsetAsync(out.vals, 0, sizeof(float) * ROWS_PER_CON * (size_t)w.cache_cap, s);
    k_adj_islands<<<grid_for(w.n, 64), 64, 0, s>>>(w, t, a, ratio, in, out);
    k_adj_mu<<<grid_for(w.max_manifolds, 256), 256, 0, s>>>(w, t, a);
    k_adj_force<<<grid_for(w.n, 256), 256, 0, s>>>(w, t, a);
}

}  // namespace cc
