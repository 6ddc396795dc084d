// C ABI of the GB300 world step: world creation, body upload (mass
// properties, sleep spheres), state exchange, and the per-step launch
// sequence captured once into a CUDA graph and replayed every step.
//
// Reference: createWorldSettings (src/world-settings.ts:224-264),
// createWorld (src/world.ts:46-58), rigidBody.create (src/body/rigid-body.ts:
// 390-434), updateWorld (src/update.ts:45-239).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "cc_internal.cuh"
#include "cc_swing.cuh"
#include "cc_hull.h"
#include "cc_mesh.h"

using namespace cc;

struct cc_world {
    cc_world_settings settings;
    DevSettings dev_settings;
    DevWorld w;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    float graph_dt = -1.f, graph_ratio = -1.f;
    double prev_dt = 0.0;
    int steps_done = 0;
    int last_status = CC_OK;
    bool any_iter_override = false;  // a body or joint overrides the iteration counts
    DevCounters last_ctr{};
    std::vector<uint64_t> ids;
    std::vector<DevHinge> hinges;  // host copy of each joint as created (bodies, flags, limits, motors)
    std::vector<DevSwing> swings;
    std::vector<DevJoint> others;  // point, distance, fixed, cone, slider joints by (type, index)
    std::vector<DevSixDof> sixdofs;
    std::vector<cc_hull::Hull> hulls;  // convex hull shapes as built
    std::vector<cc_mesh::Mesh> meshes;  // triangle meshes as built
    // compound shapes as registered: the children and the FP64 mass properties of compound.ts
    struct Compound {
        std::vector<cc_compound_child> children;
        double mass = 0, inertia[9] = {}, com[3] = {}, lo[3] = {}, hi[3] = {}, inner = 0;
        int sub_bits = 0;
    };
    std::vector<Compound> compounds;
    bool hulls_dirty = false, meshes_dirty = false, compounds_dirty = false;  // added since the last upload
    DevRay *q_rays = nullptr;  // ray query staging (cc_world_cast_rays), grown on demand
    int h_query_ovf = 0;       // the device overflow word after a shape-cast query
    DevRayHit *q_hits = nullptr;
    int q_cap = 0;
    unsigned long long *q_keys = nullptr;  // ray sort: 2 x keys, 2 x indices, radix scratch
    int *q_idx = nullptr, *q_tmp = nullptr;
    int q_sort_cap = 0;
    float *d_state_rows = nullptr;  // 16 floats per body staging for get/set state
    float *h_pinned_rows = nullptr;
    DevCounters *h_ctr = nullptr;   // pinned mirror of the device counters
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;  // bracket each cc_world_step call
    float last_call_ms = 0.f;
    // rollout gradient (cc_world_rollout_grad): tapes of one segment, checkpoints, adjoint buffers
    struct Adjoint {
        int seg_len = 0, n_ckpt = 0;
        std::vector<TapeStep> tapes;
        std::vector<float> tape_ratio;
        std::vector<Checkpoint> ckpts;  // one per segment, then the state after the rollout
        std::vector<double> ckpt_prev_dt;
        AdjBuffers buf{};
        AdjHandoff hand[2] = {{nullptr, nullptr}, {nullptr, nullptr}};
        unsigned long long *sums = nullptr;  // per world: fixed-point x, y, z sums and the count
        float *d_targets = nullptr, *d_loss = nullptr;
        std::vector<void *> allocs;
    } adj;
    int epa_packed_blocks = 0;  // packed EPA polytope blocks allocated
    // cc_world_autotune: a snapshot of the state the trials start from
    struct TuneSnapshot {
        bool ready = false;
        Checkpoint c{};
        char *joints = nullptr;  // hinges, swing-twists, then the other joint records
        size_t joint_bytes = 0;
        float2 *ccd = nullptr;
        std::vector<void *> allocs;
    } tune;
    // cc_world_step_taped: the step's rows in the C-ABI layout, grown on demand
    cc_tape_body *x_bodies = nullptr;
    cc_tape_contact *x_cons = nullptr;
    int x_cap_bodies = 0, x_cap_cons = 0;
};

static int cuda_ok(cudaError_t e) {
    if (e != cudaSuccess) {
        fprintf(stderr, "crashcat_gpu: CUDA error %s\n", cudaGetErrorString(e));
        return CC_ERR_CUDA;
    }
    return CC_OK;
}
#define CC_TRY(x)                                    \
    do {                                             \
        int _r = cuda_ok(x);                         \
        if (_r != CC_OK) return _r;                  \
    } while (0)

template <typename T>
static int dalloc(T **p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
    if (e != cudaSuccess) return cuda_ok(e);
    return cuda_ok(cudaMemset(*p, 0, sizeof(T) * count));
}

// the captured step graph holds the device world by value: drop it when a count or a
// buffer changes
static void drop_graph(cc_world *W) {
    if (W->graph_exec) {
        cudaGraphExecDestroy(W->graph_exec);
        W->graph_exec = nullptr;
    }
    if (W->graph) {
        cudaGraphDestroy(W->graph);
        W->graph = nullptr;
    }
}

// continuous-collision buffers, made when the first LINEAR_CAST body arrives
static int ensure_ccd_buffers(cc_world *W) {
    DevWorld &w = W->w;
    if (w.ccd) return CC_OK;
    const size_t cap = (size_t)w.cap, nw = (size_t)w.num_worlds;
    int r;
    if ((r = dalloc(&w.ccd_flag, cap)) != CC_OK || (r = dalloc(&w.ccd_slot, cap)) != CC_OK ||
        (r = dalloc(&w.ccd_index, cap)) != CC_OK || (r = dalloc(&w.ccd_seg, cap)) != CC_OK ||
        (r = dalloc(&w.ccd_world_off, nw + 1)) != CC_OK || (r = dalloc(&w.ccd_world_fill, nw)) != CC_OK ||
        (r = dalloc(&w.ccd_lambda, nw)) != CC_OK || (r = dalloc(&w.ccd, cap)) != CC_OK ||
        (r = dalloc(&w.ccd_scan_tmp, scan_tmp_ints((int)nw + 1))) != CC_OK)
        return r;
    drop_graph(W);
    return CC_OK;
}

// FP64 vector and quaternion helpers of the host-side shape and joint set-up
namespace {
struct D3 {
    double x, y, z;
};
struct DQ {
    double x, y, z, w;
};
D3 d3(const float *v) { return {v[0], v[1], v[2]}; }
D3 d3(float4 v) { return {v.x, v.y, v.z}; }
D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
D3 dnormalize(D3 a) {  // vec3.normalize: a zero vector stays zero
    double l = a.x * a.x + a.y * a.y + a.z * a.z;
    if (l > 0) l = 1.0 / std::sqrt(l);
    return {a.x * l, a.y * l, a.z * l};
}
DQ dq(float4 q) { return {q.x, q.y, q.z, q.w}; }
DQ dconj(DQ q) { return {-q.x, -q.y, -q.z, q.w}; }
DQ dqmul(DQ a, DQ b) {
    return {a.x * b.w + a.w * b.x + a.y * b.z - a.z * b.y, a.y * b.w + a.w * b.y + a.z * b.x - a.x * b.z,
            a.z * b.w + a.w * b.z + a.x * b.y - a.y * b.x, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
D3 drot(DQ q, D3 v) {  // q v q^-1 for a unit quaternion
    D3 u{q.x, q.y, q.z};
    D3 t = dcross(u, v);
    t = {2 * t.x, 2 * t.y, 2 * t.z};
    D3 c = dcross(u, t);
    return {v.x + q.w * t.x + c.x, v.y + q.w * t.y + c.y, v.z + q.w * t.z + c.z};
}
// rotation quaternion of the 3x3 matrix with columns c0 c1 c2 (Shoemake's method, as quat.fromMat3)
DQ quat_from_columns(D3 c0, D3 c1, D3 c2) {
    double m[3][3] = {{c0.x, c1.x, c2.x}, {c0.y, c1.y, c2.y}, {c0.z, c1.z, c2.z}};  // m[row][col]
    double tr = m[0][0] + m[1][1] + m[2][2];
    DQ o;
    if (tr > 0.0) {
        double r = std::sqrt(tr + 1.0);
        o.w = 0.5 * r;
        r = 0.5 / r;
        o.x = (m[2][1] - m[1][2]) * r;
        o.y = (m[0][2] - m[2][0]) * r;
        o.z = (m[1][0] - m[0][1]) * r;
        return o;
    }
    int i = 0;
    if (m[1][1] > m[0][0]) i = 1;
    if (m[2][2] > m[i][i]) i = 2;
    int j = (i + 1) % 3, k = (i + 2) % 3;
    double q[3];
    double r = std::sqrt(m[i][i] - m[j][j] - m[k][k] + 1.0);
    q[i] = 0.5 * r;
    r = 0.5 / r;
    o.w = (m[k][j] - m[j][k]) * r;
    q[j] = (m[j][i] + m[i][j]) * r;
    q[k] = (m[k][i] + m[i][k]) * r;
    o.x = q[0];
    o.y = q[1];
    o.z = q[2];
    return o;
}
// getInvInitialOrientationXZ (hinge-constraint.ts:166-205)
DQ inv_initial_orientation_xz(D3 n1, D3 h1, D3 n2, D3 h2) {
    const double eps = 1e-6;
    if (std::fabs(n1.x - n2.x) < eps && std::fabs(n1.y - n2.y) < eps && std::fabs(n1.z - n2.z) < eps &&
        std::fabs(h1.x - h2.x) < eps && std::fabs(h1.y - h2.y) < eps && std::fabs(h1.z - h2.z) < eps)
        return {0, 0, 0, 1};
    DQ q1 = quat_from_columns(n1, dcross(h1, n1), h1), q2 = quat_from_columns(n2, dcross(h2, n2), h2);
    return dqmul(q2, dconj(q1));
}
float3 f3d(D3 v) { return make_float3((float)v.x, (float)v.y, (float)v.z); }
bool finite3(const float *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }
bool spring_ok(const cc_spring_settings &s) {
    return (s.mode == 0 || s.mode == 1) && std::isfinite(s.frequency_or_stiffness) && std::isfinite(s.damping);
}
}  // namespace

static int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

extern "C" {

const char *cc_status_string(int status) {
    switch (status) {
        case CC_OK:
            return "ok";
        case CC_ERR_INVALID:
            return "invalid argument";
        case CC_ERR_CAPACITY:
            return "a per-step buffer overflowed (pairs, manifolds, EPA queue or contact cache)";
        case CC_ERR_TIMEOUT:
            return "a bounded device-side wait gave up";
        case CC_ERR_NAN:
            return "non-finite body state";
        case CC_ERR_CUDA:
            return "CUDA runtime error";
        case CC_ERR_UNSUPPORTED:
            return "unsupported feature";
    }
    return "unknown status";
}

// createWorldSettings world-settings.ts:224-264, with the two-layer setup of
// the reference's tests (tst/helpers.ts:5-26): MOVING (0) collides with MOVING
// and NOT_MOVING (1).
int cc_world_settings_default(cc_world_settings *o) {
    if (!o) return CC_ERR_INVALID;
    memset(o, 0, sizeof(*o));
    o->gravity[0] = 0;
    o->gravity[1] = -9.81;
    o->gravity[2] = 0;
    o->gravity_enabled = 1;
    o->speculative_contact_distance = 0.02;
    o->manifold_tolerance = 1e-3;
    o->collision_tolerance = 1e-4;
    o->penetration_tolerance = 1e-4;
    o->normal_cos_max_delta_rotation = cos((5 * M_PI) / 180);
    o->contact_point_preserve_lambda_max_dist_sq = 0.01 * 0.01;
    o->velocity_iterations = 10;
    o->position_iterations = 2;
    o->warm_starting = 1;
    o->penetration_slop = 0.02;
    o->baumgarte_factor = 0.2;
    o->max_penetration_distance = 0.2;
    o->min_velocity_for_restitution = 1;
    o->allow_sleeping = 1;
    o->time_before_sleep = 0.5;
    o->point_velocity_sleep_threshold = 0.03;
    o->num_object_layers = 2;
    o->num_broadphase_layers = 2;
    o->object_to_broadphase[0] = 0;
    o->object_to_broadphase[1] = 1;
    o->object_pairs[0] = 0b11;
    o->object_pairs[1] = 0b01;
    o->object_vs_broadphase[0] = 0b11;
    o->object_vs_broadphase[1] = 0b11;
    o->broadphase_pairs[0] = 0b11;
    o->broadphase_pairs[1] = 0b01;
    o->max_bodies = 1 << 16;
    o->num_worlds = 1;
    o->ccd_linear_cast_threshold = 0.05;  // world-settings.ts:258-262
    o->ccd_linear_cast_max_penetration = 0.25;
    o->ccd_min_velocity_for_restitution = 1.0;
    return CC_OK;
}

int cc_world_create(const cc_world_settings *s, cc_world **out) {
    if (!s || !out) return CC_ERR_INVALID;
    if (s->num_object_layers < 1 || s->num_object_layers > CC_MAX_LAYERS || s->num_broadphase_layers < 1 ||
        s->num_broadphase_layers > CC_MAX_LAYERS || s->max_bodies < 1 || s->num_worlds < 1)
        return CC_ERR_INVALID;
    cc_world *W = new (std::nothrow) cc_world();
    if (!W) return CC_ERR_INVALID;
    W->settings = *s;
    DevSettings &d = W->dev_settings;
    memset(&d, 0, sizeof(d));
    for (int k = 0; k < 3; k++) d.gravity[k] = (float)s->gravity[k];
    d.gravity_enabled = s->gravity_enabled;
    d.spec_dist = (float)s->speculative_contact_distance;
    d.manifold_tol = (float)s->manifold_tolerance;
    d.collision_tol = (float)s->collision_tolerance;
    d.penetration_tol = (float)s->penetration_tolerance;
    d.normal_cos = (float)s->normal_cos_max_delta_rotation;
    d.preserve_lambda_dsq = (float)s->contact_point_preserve_lambda_max_dist_sq;
    d.vel_iters = s->velocity_iterations;
    d.pos_iters = s->position_iterations;
    d.warm_starting = s->warm_starting;
    d.slop = (float)s->penetration_slop;
    d.baumgarte = (float)s->baumgarte_factor;
    d.max_pen = (float)s->max_penetration_distance;
    d.min_vel_restitution = (float)s->min_velocity_for_restitution;
    d.allow_sleeping = s->allow_sleeping;
    d.time_before_sleep = (float)s->time_before_sleep;
    d.sleep_threshold = (float)s->point_velocity_sleep_threshold;
    d.wait_polls = s->device_wait_polls > 0 ? (unsigned)s->device_wait_polls : (1u << 21);
    // test hook: block 0 of the whole-grid island solve leaves before its first grid barrier, so
    // the other blocks' bounded wait on that barrier runs out (a flag that nothing sets)
    d.test_withhold_block = getenv("CRASHCAT_TEST_WITHHOLD_BARRIER") ? 1 : 0;
    d.link_attempts = s->island_link_attempts > 0 ? s->island_link_attempts : (1 << 20);
    d.ccd_threshold = (float)s->ccd_linear_cast_threshold;
    d.ccd_max_penetration = (float)s->ccd_linear_cast_max_penetration;
    d.ccd_min_vel_restitution = (float)s->ccd_min_velocity_for_restitution;
    // launch-shape tunable: islands with at most this many contacts are solved by one
    // thread in the reference's exact order, larger ones by a warp (up to 256 contacts
    // and 128 bodies) or a CTA with order-preserving graph colouring
    d.small_island_max_joints = 16;
    if (const char *e = getenv("CRASHCAT_SMALL_JOINTS_MAX")) {
        int v = atoi(e);
        if (v >= 0 && v <= 16) d.small_island_max_joints = v;
    }
    d.small_island_max_cons = 8;
    if (const char *e = getenv("CRASHCAT_SMALL_ISLAND_MAX")) {
        int v = atoi(e);
        if (v >= 0 && v <= 64) d.small_island_max_cons = v;
    }
    // combined layer predicate: object layer pair enabled AND the querying
    // layer may query the other's broadphase layer AND the broadphase layers
    // collide (broadphase.ts:252-272, dbvt.ts:657-660)
    for (int a = 0; a < s->num_object_layers; a++) {
        uint32_t m = 0;
        int bpa = s->object_to_broadphase[a];
        for (int b = 0; b < s->num_object_layers; b++) {
            int bpb = s->object_to_broadphase[b];
            bool ok = (s->object_pairs[a] >> b) & 1;
            ok = ok && ((s->object_vs_broadphase[a] >> bpb) & 1);
            ok = ok && ((s->broadphase_pairs[bpa] >> bpb) & 1);
            if (ok) m |= 1u << b;
        }
        d.allowed_pairs[a] = m;
        uint32_t mc = 0;
        for (int b = 0; b < s->num_object_layers; b++)
            if (((s->object_pairs[a] >> b) & 1) && ((s->object_vs_broadphase[a] >> s->object_to_broadphase[b]) & 1))
                mc |= 1u << b;
        d.cast_pairs[a] = mc;
    }
    DevWorld &w = W->w;
    memset(&w, 0, sizeof(w));
    int cap = s->max_bodies;
    w.cap = cap;
    w.n = 0;
    w.num_worlds = s->num_worlds;
    w.max_pairs = s->max_pairs > 0 ? s->max_pairs : 16 * cap + 1024;
    w.max_manifolds = s->max_manifolds > 0 ? s->max_manifolds : 8 * cap + 1024;
    w.max_epa = w.max_manifolds;
    w.cache_cap = next_pow2(2 * w.max_manifolds);
    int r = CC_OK;
#define ALLOC(field, count)                       \
    if ((r = dalloc(&w.field, (count))) != CC_OK) { \
        cc_world_destroy(W);                      \
        return r;                                 \
    }
    ALLOC(pos, cap);
    ALLOC(quat, cap);
    ALLOC(com, cap);
    ALLOC(linvel, cap);
    ALLOC(angvel, cap);
    ALLOC(force, cap);
    ALLOC(torque, cap);
    ALLOC(inv_inertia, cap);
    ALLOC(inertia_rot, cap);
    ALLOC(shape, cap);
    ALLOC(material, cap);
    ALLOC(damping, cap);
    ALLOC(flags, cap);
    ALLOC(groups, cap);
    ALLOC(world, cap);
    ALLOC(sleep_sph, 3 * (size_t)cap);
    ALLOC(sleep_timer, cap);
    ALLOC(aabb64, 6 * (size_t)cap);
    ALLOC(aabb_lo, cap);
    ALLOC(aabb_hi, cap);
    ALLOC(wake, cap);
    ALLOC(morton, cap);
    ALLOC(morton_alt, cap);
    ALLOC(order, cap);
    ALLOC(order_alt, cap);
    ALLOC(node_parent, 2 * (size_t)cap);
    ALLOC(node_child, cap);
    ALLOC(node_lo, 2 * (size_t)cap);
    ALLOC(node_hi, 2 * (size_t)cap);
    ALLOC(node_flag, cap);
    ALLOC(pairs, w.max_pairs);
    ALLOC(pair_order, w.max_pairs);
    ALLOC(manifolds, w.max_manifolds);
    ALLOC(cons, w.max_manifolds);
    ALLOC(cons_of_manifold, w.max_manifolds);
    ALLOC(uf_parent, cap);
    ALLOC(island_of_body, cap);
    ALLOC(island_id_of_root, cap);
    ALLOC(island_body_count, cap);
    ALLOC(island_cons_count, cap);
    ALLOC(island_body_off, cap);
    ALLOC(island_cons_off, cap);
    ALLOC(island_bodies, cap);
    ALLOC(island_cons, w.max_manifolds);
    ALLOC(island_fill_b, cap);
    ALLOC(island_fill_c, cap);
    ALLOC(iter_ovr, cap);
    ALLOC(island_iters, 3 * cap);
    ALLOC(inv_inertia_world, 2 * (size_t)cap);
    {
        size_t tmp = scan_tmp_ints(cap > w.max_manifolds ? cap : w.max_manifolds);
        ALLOC(scan_tmp, tmp);
    }
    ALLOC(ctr, 1);
    ALLOC(scene, 16);
    ALLOC(node_world, 2 * (size_t)cap);
    {
        char *p = nullptr;
        if ((r = dalloc(&p, epa_item_bytes() * (size_t)w.max_epa)) != CC_OK) {
            cc_world_destroy(W);
            return r;
        }
        w.epa_items = p;
        // EPA threads scale with the world: about one per 8 bodies, 1,024 to epa_default_max_threads(),
        // and two blocks per SM (the tuner's smallest shape) once the world has that many bodies, so
        // that every SM's FP64 pipe takes part
        int et = cap / 8;
        const int two_per_sm = device_sm_count() * 2 * 64;
        if (et < two_per_sm) et = cap < two_per_sm ? cap : two_per_sm;
        et = et < 1024 ? 1024 : (et > epa_default_max_threads() ? epa_default_max_threads() : et);
        if (const char *e = getenv("CRASHCAT_EPA_THREADS")) {
            int v = atoi(e);
            if (v >= 64 && v <= epa_max_threads()) et = v;
        }
        w.epa_threads = (et + 63) / 64 * 64;
        // launch-shape tunable: the packed polytope's point limit (4 to 32); items that need
        // more support points are re-run by the pass with the reference's limits
        w.epa_packed_points = 32;
        w.epa_fetch_warp = 1;
        if (const char *e = getenv("CRASHCAT_EPA_FETCH_WARP")) w.epa_fetch_warp = atoi(e) != 0;
        if (const char *e = getenv("CRASHCAT_EPA_PACKED_POINTS")) {
            int v = atoi(e);
            if (v >= 4 && v <= 32) w.epa_packed_points = v;
        }
        w.warp_blocks_per_sm = 4;
        w.warp_carveout = 50;
        if (const char *e = getenv("CRASHCAT_WARP_BLOCKS_PER_SM")) {
            int v = atoi(e);
            if (v >= 1 && v <= 4) w.warp_blocks_per_sm = v;
        }
        if (const char *e = getenv("CRASHCAT_WARP_CARVEOUT")) {
            int v = atoi(e);
            if (v >= 0 && v <= 100) w.warp_carveout = v;
        }
        char *q = nullptr;
        if ((r = dalloc(&q, epa_packed_block_bytes() * (size_t)(w.epa_threads / 64))) != CC_OK) {
            cc_world_destroy(W);
            return r;
        }
        w.epa_packed = q;
        W->epa_packed_blocks = w.epa_threads / 64;
        char *g = nullptr;
        if ((r = dalloc(&g, epa_scratch_bytes() * (size_t)EPA_BIG_THREADS)) != CC_OK) {
            cc_world_destroy(W);
            return r;
        }
        w.epa_scratch = g;
    }
    ALLOC(epa_fallback, w.max_epa);
    for (int k = 0; k < 2; k++) {
        ALLOC(cache_keys[k], w.cache_cap);
        ALLOC(cache_recs[k], w.cache_cap);
        cudaMemset(w.cache_keys[k], 0xff, sizeof(unsigned long long) * w.cache_cap);
    }
    ALLOC(cache_parity, 1);
    ALLOC(root_flag, cap);
    ALLOC(small_list, (size_t)cap * SMALL_BUCKETS);
    ALLOC(large_list, cap);
    ALLOC(scratch_order, w.max_manifolds);
    ALLOC(scratch_colour, w.max_manifolds);
    ALLOC(scratch_claim, (size_t)cap + (size_t)w.max_manifolds + 16);
    ALLOC(mid_list, (size_t)cap * MID_BUCKETS);
    ALLOC(contact_event, w.max_manifolds);
    ALLOC(removed_keys, w.max_manifolds);
    ALLOC(body_local, cap);
    ALLOC(giant_list, cap);
    ALLOC(giant_claim, 4 * (size_t)cap);
    ALLOC(giant_count, 4 * (GIANT_COLOURS + 2));
#undef ALLOC
    // islands with more constraints than this are solved by the whole grid (launch-shape tunable)
    w.giant_min = 8192;
    if (const char *e = getenv("CRASHCAT_GIANT_MIN")) {
        int v = atoi(e);
        if (v >= 1) w.giant_min = v;
    }
    w.giant_blocks = giant_blocks_for_device();
    if (const char *e = getenv("CRASHCAT_GIANT_BLOCKS")) {  // launch-shape tunable, at most one per SM
        int v = atoi(e);
        if (v >= 1 && v < w.giant_blocks) w.giant_blocks = v;
    }
    if (w.giant_blocks <= 0) w.giant_min = 0x7fffffff;
    if ((r = cuda_ok(cudaStreamCreateWithFlags(&W->stream, cudaStreamNonBlocking))) != CC_OK ||
        (r = cuda_ok(cudaStreamCreateWithFlags(&w.aux_stream, cudaStreamNonBlocking))) != CC_OK ||
        (r = cuda_ok(cudaStreamCreateWithFlags(&w.aux2_stream, cudaStreamNonBlocking))) != CC_OK ||
        (r = cuda_ok(cudaStreamCreateWithFlags(&w.aux3_stream, cudaStreamNonBlocking))) != CC_OK ||
        (r = cuda_ok(cudaEventCreateWithFlags(&w.ev_join3, cudaEventDisableTiming))) != CC_OK ||
        (r = cuda_ok(cudaEventCreateWithFlags(&w.ev_fork, cudaEventDisableTiming))) != CC_OK ||
        (r = cuda_ok(cudaEventCreateWithFlags(&w.ev_join, cudaEventDisableTiming))) != CC_OK ||
        (r = cuda_ok(cudaEventCreateWithFlags(&w.ev_join2, cudaEventDisableTiming))) != CC_OK) {
        cc_world_destroy(W);
        return r;
    }
    if ((r = dalloc(&W->d_state_rows, 16 * (size_t)cap)) != CC_OK) {
        cc_world_destroy(W);
        return r;
    }
    if ((r = cuda_ok(cudaMallocHost((void **)&W->h_ctr, sizeof(DevCounters)))) != CC_OK) {
        cc_world_destroy(W);
        return r;
    }
    memset(W->h_ctr, 0, sizeof(DevCounters));
    *out = W;
    return CC_OK;
}

int cc_world_destroy(cc_world *W) {
    if (!W) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (W->stream) cudaStreamSynchronize(W->stream);
    if (W->graph_exec) cudaGraphExecDestroy(W->graph_exec);
    if (W->graph) cudaGraphDestroy(W->graph);
    void *ptrs[] = {w.pos, w.quat, w.com, w.linvel, w.angvel, w.force, w.torque, w.inv_inertia, w.inertia_rot,
                    w.shape, w.material, w.damping, w.flags, w.groups, w.world, w.sleep_sph, w.sleep_timer,
                    w.aabb64, w.aabb_lo, w.aabb_hi, w.wake, w.morton, w.morton_alt, w.order, w.order_alt,
                    w.node_parent, w.node_child, w.node_lo, w.node_hi, w.node_flag, w.pairs, w.pair_order, w.manifolds, w.cons,
                    w.cons_of_manifold, w.uf_parent, w.island_of_body, w.island_id_of_root, w.island_body_count,
                    w.island_cons_count, w.island_body_off, w.island_cons_off, w.island_bodies, w.island_cons,
                    w.island_fill_b, w.island_fill_c, w.iter_ovr, w.island_iters, w.inv_inertia_world, w.scan_tmp, w.ctr, w.scene,
                    w.node_world, w.epa_items, w.epa_packed, w.epa_scratch, w.epa_fallback, w.cache_keys[0], w.cache_keys[1], w.cache_recs[0],
                    w.cache_recs[1], w.cache_parity, w.root_flag, w.small_list, w.large_list, w.scratch_order,
                    w.scratch_colour, w.scratch_claim, w.mid_list, w.body_local, w.contact_event,
                    w.removed_keys, W->d_state_rows, w.hinges, w.island_joints, w.island_joint_count,
                    w.island_joint_off, w.island_fill_j, w.joint_wake, w.joint_partners, w.swings, w.others, w.sixdofs, w.frames,
                    w.giant_list, w.giant_claim, w.giant_count, w.small_joint_list, w.large_joint_list,
                    w.hulls, w.hull_points, w.hull_shrunk,
                    w.hull_planes, w.hull_faces, w.hull_vidx, w.ccd_flag, w.ccd_slot, w.ccd_index, w.ccd,
                    w.ccd_world_off, w.ccd_world_fill, w.ccd_seg, w.ccd_lambda, w.ccd_scan_tmp,
                    w.meshes, w.mesh_verts, w.mesh_tris, w.mesh_nodes, w.mesh_pairs, w.mesh_epa_base,
                    w.mesh_epa_count, w.mesh_big, w.mesh_big_red, w.compounds, w.children, w.compound_pairs};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (W->q_rays) cudaFree(W->q_rays);
    if (W->q_hits) cudaFree(W->q_hits);
    if (W->q_keys) cudaFree(W->q_keys);
    if (W->q_idx) cudaFree(W->q_idx);
    if (W->q_tmp) cudaFree(W->q_tmp);
    for (void *p : W->adj.allocs)
        if (p) cudaFree(p);
    for (void *p : W->tune.allocs)
        if (p) cudaFree(p);
    if (W->x_bodies) cudaFree(W->x_bodies);
    if (W->x_cons) cudaFree(W->x_cons);
    if (W->h_ctr) cudaFreeHost(W->h_ctr);
    if (W->ev_begin) cudaEventDestroy(W->ev_begin);
    if (W->ev_end) cudaEventDestroy(W->ev_end);
    if (W->stream) cudaStreamDestroy(W->stream);
    if (w.aux_stream) cudaStreamDestroy(w.aux_stream);
    if (w.aux2_stream) cudaStreamDestroy(w.aux2_stream);
    if (w.aux3_stream) cudaStreamDestroy(w.aux3_stream);
    if (w.ev_join3) cudaEventDestroy(w.ev_join3);
    if (w.ev_fork) cudaEventDestroy(w.ev_fork);
    if (w.ev_join) cudaEventDestroy(w.ev_join);
    if (w.ev_join2) cudaEventDestroy(w.ev_join2);
    delete W;
    return CC_OK;
}

int cc_world_num_bodies(const cc_world *W, int32_t *out) {
    if (!W || !out) return CC_ERR_INVALID;
    *out = W->w.n;
    return CC_OK;
}

// rigidBody.create rigid-body.ts:390-434: mass properties (box: setMassAndInertiaOfSolidBox
// mass-properties.ts:36-52; sphere: sphere.ts:97-123), setMassProperties
// (motion-properties.ts:419-491; the inertia of boxes and spheres is diagonal so
// the principal rotation is the identity), centre of mass, sleep spheres.
int cc_world_add_bodies(cc_world *W, const cc_body_desc *b, int32_t n, int32_t *out_index) {
    if (!W || (!b && n > 0) || n < 0) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (w.n + n > w.cap) return CC_ERR_CAPACITY;
    std::vector<float4> pos(n), quat(n), com(n), lin(n), ang(n), zero(n), ii(n), ir(n), sh(n), mat(n), damp(n),
        sph(3 * (size_t)n);
    std::vector<uint32_t> flags(n), ovr(n);
    std::vector<uint2> groups(n);
    std::vector<int> world(n);
    std::vector<float> timer(n, 0.f);
    std::vector<DevFrame> frames(n);
    bool any_decorated = false;
    for (int i = 0; i < n; i++) {
        const cc_body_desc &d = b[i];
        if (d.shape_type != CC_SHAPE_BOX && d.shape_type != CC_SHAPE_SPHERE && d.shape_type != CC_SHAPE_CAPSULE &&
            d.shape_type != CC_SHAPE_CONVEX_HULL && d.shape_type != CC_SHAPE_TRIANGLE_MESH &&
            d.shape_type != CC_SHAPE_CYLINDER && d.shape_type != CC_SHAPE_PLANE && d.shape_type != CC_SHAPE_EMPTY &&
            d.shape_type != CC_SHAPE_COMPOUND)
            return CC_ERR_UNSUPPORTED;
        if (d.mass_properties_mode < 0 || d.mass_properties_mode > 2 || !std::isfinite(d.mass)) return CC_ERR_INVALID;
        for (int k = 0; k < 6; k++)
            if (!std::isfinite(d.inertia[k])) return CC_ERR_INVALID;
        const bool plane = d.shape_type == CC_SHAPE_PLANE;
        D3 pn{0, 1, 0};
        if (plane) {  // plane.ts create :77-98; no mass (:120-122): static or kinematic only
            pn = dnormalize(d3(d.shape_params));
            if (!(pn.x * pn.x + pn.y * pn.y + pn.z * pn.z > 0) || !std::isfinite(d.shape_params[3]) ||
                d.motion_type == CC_DYNAMIC)
                return CC_ERR_INVALID;
        }
        if (d.shape_type == CC_SHAPE_CYLINDER &&  // cylinder.ts update: 0 <= convex radius <= half height, radius
            !(d.shape_params[2] >= 0.f && d.shape_params[0] >= d.shape_params[2] && d.shape_params[1] >= d.shape_params[2]))
            return CC_ERR_INVALID;
        const cc_mesh::Mesh *mesh = nullptr;
        int mesh_index = -1;
        if (d.shape_type == CC_SHAPE_TRIANGLE_MESH) {
            mesh_index = (int)d.shape_params[0];
            if (!(d.shape_params[0] == (float)mesh_index) || mesh_index < 0 || mesh_index >= (int)W->meshes.size())
                return CC_ERR_INVALID;
            // a mesh has no mass (triangle-mesh.ts:153-158): static or kinematic bodies only
            if (d.motion_type == CC_DYNAMIC) return CC_ERR_INVALID;
            // the contact key packs body indices in 21 bits
            if (w.cap >= (1 << MESH_KEY_BITS)) return CC_ERR_UNSUPPORTED;
            mesh = &W->meshes[mesh_index];
        }
        const cc_hull::Hull *hull = nullptr;
        int hull_index = -1;
        if (d.shape_type == CC_SHAPE_CONVEX_HULL) {
            hull_index = (int)d.shape_params[0];
            if (!(d.shape_params[0] == (float)hull_index) || hull_index < 0 || hull_index >= (int)W->hulls.size())
                return CC_ERR_INVALID;
            hull = &W->hulls[hull_index];
        }
        const cc_world::Compound *cmp = nullptr;
        int cmp_index = -1;
        if (d.shape_type == CC_SHAPE_COMPOUND) {
            cmp_index = (int)d.shape_params[0];
            if (!(d.shape_params[0] == (float)cmp_index) || cmp_index < 0 || cmp_index >= (int)W->compounds.size())
                return CC_ERR_INVALID;
            if (d.motion_quality == CC_MOTION_LINEAR_CAST) return CC_ERR_UNSUPPORTED;  // no compound cast
            if (w.cap >= (1 << MESH_KEY_BITS)) return CC_ERR_UNSUPPORTED;  // the contact key's 21-bit indices
            cmp = &W->compounds[cmp_index];
        }
        if (d.shape_type == CC_SHAPE_CAPSULE && !(d.shape_params[0] > 0.f && d.shape_params[1] > 0.f))
            return CC_ERR_INVALID;  // capsule.ts:55-61
        if (d.motion_type < 0 || d.motion_type > 2) return CC_ERR_INVALID;
        if (d.motion_quality != CC_MOTION_DISCRETE && d.motion_quality != CC_MOTION_LINEAR_CAST) return CC_ERR_INVALID;
        if (d.object_layer < 0 || d.object_layer >= W->settings.num_object_layers) return CC_ERR_INVALID;
        if (d.world < 0 || d.world >= w.num_worlds) return CC_ERR_INVALID;
        if (d.num_velocity_steps_override < 0 || d.num_velocity_steps_override > 255 ||
            d.num_position_steps_override < 0 || d.num_position_steps_override > 255)
            return CC_ERR_INVALID;
        ovr[i] = (uint32_t)d.num_velocity_steps_override | ((uint32_t)d.num_position_steps_override << 8);
        if (ovr[i]) W->any_iter_override = true;
        // shape decorators, OffsetCenterOfMass(Transformed(Scaled(leaf))) (scaled.ts, transformed.ts,
        // offset-center-of-mass.ts)
        if (!finite3(d.shape_scale) || !finite3(d.shape_position) || !finite3(d.com_offset) ||
            !std::isfinite(d.shape_quaternion[0]) || !std::isfinite(d.shape_quaternion[1]) ||
            !std::isfinite(d.shape_quaternion[2]) || !std::isfinite(d.shape_quaternion[3]))
            return CC_ERR_INVALID;
        double sc[3] = {d.shape_scale[0], d.shape_scale[1], d.shape_scale[2]};
        for (int k = 0; k < 3; k++)
            if (sc[k] == 0) sc[k] = 1;
        DQ tq{d.shape_quaternion[0], d.shape_quaternion[1], d.shape_quaternion[2], d.shape_quaternion[3]};
        if (tq.x == 0 && tq.y == 0 && tq.z == 0 && tq.w == 0) tq = {0, 0, 0, 1};
        const D3 tp = d3(d.shape_position), off = d3(d.com_offset);
        const bool scaled = sc[0] != 1 || sc[1] != 1 || sc[2] != 1;
        const bool transformed = tp.x != 0 || tp.y != 0 || tp.z != 0 || tq.x != 0 || tq.y != 0 || tq.z != 0 || tq.w != 1;
        const bool offset = off.x != 0 || off.y != 0 || off.z != 0;
        // a plane keeps its local bounds (computePlaneLocalBounds plane.ts:273-295) in a frame, and
        // a compound its bounds, centre of mass and inner radius (an identity transform)
        if (cmp && (scaled || transformed || offset)) return CC_ERR_UNSUPPORTED;
        const bool decorated = scaled || transformed || offset || plane || cmp;
        if (scaled && (hull || mesh || plane)) return CC_ERR_UNSUPPORTED;
        double mass;
        double idiag[3];
        double irot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // principal axes (columns)
        if (mesh || plane) {
            mass = 0.0;  // computeMassProperties triangle-mesh.ts:153-158, plane.ts:120-122
            idiag[0] = idiag[1] = idiag[2] = 0.0;
        } else if (cmp) {
            // the compound's mass and inertia (compound.ts:177-230, the children's densities),
            // principal axes
            mass = cmp->mass;
            double I[9];
            for (int k = 0; k < 9; k++) I[k] = cmp->inertia[k];
            cc_hull::principal_axes(I, idiag, irot);
        } else if (hull) {
            // computeMassProperties convex-hull.ts:453-459, principal axes of the inertia
            mass = hull->volume * d.density;
            double I[9];
            for (int k = 0; k < 9; k++) I[k] = hull->inertia[k] * d.density;
            cc_hull::principal_axes(I, idiag, irot);
        } else if (d.shape_type == CC_SHAPE_BOX) {
            double fx = 2.0 * d.shape_params[0], fy = 2.0 * d.shape_params[1], fz = 2.0 * d.shape_params[2];
            mass = fx * fy * fz * d.density;
            idiag[0] = (fy * fy + fz * fz) * (mass / 12.0);
            idiag[1] = (fx * fx + fz * fz) * (mass / 12.0);
            idiag[2] = (fx * fx + fy * fy) * (mass / 12.0);
        } else if (d.shape_type == CC_SHAPE_CYLINDER) {
            // computeMassProperties cylinder.ts
            double h = d.shape_params[0], r = d.shape_params[1];
            mass = M_PI * r * r * 2 * h * d.density;
            double iyy = 0.5 * mass * r * r;
            idiag[1] = iyy;
            idiag[0] = idiag[2] = 0.5 * iyy + (mass * 4 * h * h) / 12;
        } else if (d.shape_type == CC_SHAPE_CAPSULE) {
            // computeMassProperties capsule.ts:119-157: cylinder plus two hemispheres along Y
            double r = d.shape_params[0], h = d.shape_params[1];
            double volume = M_PI * r * r * (2 * h) + (4.0 / 3.0) * M_PI * r * r * r;
            mass = volume * d.density;
            double r2 = r * r, height = 2.0 * h;
            double cyl = M_PI * height * r2 * d.density;
            double hemi = ((2.0 * M_PI) / 3.0) * r2 * r * d.density;
            double iy = r2 * cyl * 0.5 + hemi * (2.0 / 5.0) * r2;
            double ixz = cyl * ((1.0 / 12.0) * height * height + (1.0 / 4.0) * r2) +
                         hemi * ((2.0 / 5.0) * r2 + h * h + (3.0 / 8.0) * h * r);
            idiag[0] = idiag[2] = ixz;
            idiag[1] = iy;
        } else {
            double r = d.shape_params[0];
            mass = (4.0 / 3.0) * M_PI * r * r * r * d.density;
            double in = 0.4 * mass * r * r;
            idiag[0] = idiag[1] = idiag[2] = in;
        }
        bool given_tensor = false;
        DevFrame fr;
        memset(&fr, 0, sizeof(fr));
        if (decorated && !mesh && !plane && !cmp) {
            // computeMassProperties: massProperties.scale (mass-properties.ts:59-112), rotate
            // (:121-160), translate (:168-205) of the leaf's, then the principal axes
            double t[9] = {idiag[0], 0, 0, 0, idiag[1], 0, 0, 0, idiag[2]};
            if (hull)
                for (int k = 0; k < 9; k++) t[k] = hull->inertia[k] * d.density;
            if (scaled) {
                double half = 0.5 * (t[0] + t[4] + t[8]);
                double q0 = sc[0] * sc[0] * (half - t[0]), q1 = sc[1] * sc[1] * (half - t[4]),
                       q2 = sc[2] * sc[2] * (half - t[8]);
                double ms = std::fabs(sc[0] * sc[1] * sc[2]);
                double nt[9] = {q1 + q2,           sc[0] * sc[1] * t[1], sc[0] * sc[2] * t[2],
                                sc[0] * sc[1] * t[3], q0 + q2,           sc[1] * sc[2] * t[5],
                                sc[0] * sc[2] * t[6], sc[1] * sc[2] * t[7], q0 + q1};
                for (int k = 0; k < 9; k++) t[k] = nt[k] * ms;
                mass *= ms;
            }
            if (transformed) {
                D3 cols[3] = {drot(tq, D3{1, 0, 0}), drot(tq, D3{0, 1, 0}), drot(tq, D3{0, 0, 1})};
                double R[9] = {cols[0].x, cols[1].x, cols[2].x, cols[0].y, cols[1].y, cols[2].y,
                               cols[0].z, cols[1].z, cols[2].z};  // row-major
                double rt[9], o[9];
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) {
                        rt[3 * a + c] = 0;
                        for (int k = 0; k < 3; k++) rt[3 * a + c] += R[3 * a + k] * t[3 * k + c];
                    }
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) {
                        o[3 * a + c] = 0;
                        for (int k = 0; k < 3; k++) o[3 * a + c] += rt[3 * a + k] * R[3 * c + k];
                    }
                for (int k = 0; k < 9; k++) t[k] = o[k];
            }
            if (offset) {
                double dd = off.x * off.x + off.y * off.y + off.z * off.z, v[3] = {off.x, off.y, off.z};
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) t[3 * a + c] += mass * ((a == c ? dd : 0.0) - v[a] * v[c]);
            }
            cc_hull::principal_axes(t, idiag, irot);
        }
        // MassPropertiesOverride (rigid-body.ts:309-326, 676-700): a given mass scales the shape's
        // inertia (scaleToMass mass-properties.ts:220-240); a given mass and inertia replace them
        if (d.mass_properties_mode == CC_MASS_GIVEN) {
            if (mass > 0)
                for (int k = 0; k < 3; k++) idiag[k] *= d.mass / mass;
            mass = d.mass;
        } else if (d.mass_properties_mode == CC_MASS_AND_INERTIA_GIVEN) {
            const float *t = d.inertia;
            double g[9] = {t[0], t[1], t[2], t[1], t[3], t[4], t[2], t[4], t[5]};
            cc_hull::principal_axes(g, idiag, irot);
            mass = d.mass;
            given_tensor = true;
        }
        if (decorated) {
            // the leaf's local bounds, times |s| per axis (computeScaledLocalBounds), then the corners
            // moved by the transform (computeTransformedLocalBounds); the offset moves none of them
            double lo[3], hi[3];
            if (plane) {
                // getOrthogonalBasis :210-233, getPlaneVertices :235-271: the face's corners and
                // the corners one half extent behind it
                const double he = 1000.0, c = d.shape_params[3];
                D3 p1 = dcross(pn, D3{0, 1, 0});
                double l = p1.x * p1.x + p1.y * p1.y + p1.z * p1.z;
                p1 = l < 1e-6 ? D3{1, 0, 0} : D3{p1.x / std::sqrt(l), p1.y / std::sqrt(l), p1.z / std::sqrt(l)};
                D3 p2 = dnormalize(dcross(p1, pn));
                p1 = dnormalize(dcross(pn, p2));
                D3 pt{-c * pn.x, -c * pn.y, -c * pn.z};
                for (int k = 0; k < 3; k++) lo[k] = 1e300, hi[k] = -1e300;
                for (int v = 0; v < 4; v++) {
                    const double s1 = (v == 0 || v == 1) ? he : -he, s2 = (v == 0 || v == 3) ? he : -he;
                    D3 q{pt.x + s1 * p1.x + s2 * p2.x, pt.y + s1 * p1.y + s2 * p2.y, pt.z + s1 * p1.z + s2 * p2.z};
                    for (int back = 0; back < 2; back++) {
                        double e[3] = {q.x - back * he * pn.x, q.y - back * he * pn.y, q.z - back * he * pn.z};
                        for (int k = 0; k < 3; k++) lo[k] = std::min(lo[k], e[k]), hi[k] = std::max(hi[k], e[k]);
                    }
                }
            } else if (mesh) {
                for (int k = 0; k < 3; k++) {
                    lo[k] = mesh->lo[k];
                    hi[k] = mesh->hi[k];
                }
            } else if (cmp) {
                for (int k = 0; k < 3; k++) {
                    lo[k] = cmp->lo[k];
                    hi[k] = cmp->hi[k];
                }
            } else if (hull) {
                lo[0] = hull->lo.x, lo[1] = hull->lo.y, lo[2] = hull->lo.z;
                hi[0] = hull->hi.x, hi[1] = hull->hi.y, hi[2] = hull->hi.z;
            } else {
                const float *q = d.shape_params;
                double e[3] = {q[0], q[0], q[0]};
                if (d.shape_type == CC_SHAPE_BOX) e[0] = q[0], e[1] = q[1], e[2] = q[2];
                if (d.shape_type == CC_SHAPE_CAPSULE) e[1] = (double)q[1] + (double)q[0];
                if (d.shape_type == CC_SHAPE_CYLINDER) e[0] = e[2] = q[1], e[1] = q[0];
                for (int k = 0; k < 3; k++) lo[k] = -e[k], hi[k] = e[k];
            }
            for (int k = 0; k < 3; k++) {
                lo[k] *= std::fabs(sc[k]);
                hi[k] *= std::fabs(sc[k]);
            }
            if (transformed) {
                double nlo[3] = {1e300, 1e300, 1e300}, nhi[3] = {-1e300, -1e300, -1e300};
                for (int c = 0; c < 8; c++) {
                    D3 k = drot(tq, D3{(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]});
                    double v[3] = {k.x + tp.x, k.y + tp.y, k.z + tp.z};
                    for (int a = 0; a < 3; a++) {
                        nlo[a] = std::min(nlo[a], v[a]);
                        nhi[a] = std::max(nhi[a], v[a]);
                    }
                }
                for (int a = 0; a < 3; a++) lo[a] = nlo[a], hi[a] = nhi[a];
            }
            for (int k = 0; k < 3; k++) fr.lo[k] = lo[k], fr.hi[k] = hi[k];
            // centre of mass: computeTransformedCenterOfMass + the offset (a scaled shape's is zero)
            D3 c{0, 0, 0};
            if (hull && !scaled) c = D3{hull->com.x, hull->com.y, hull->com.z};
            if (cmp) c = D3{cmp->com[0], cmp->com[1], cmp->com[2]};
            if (transformed) {
                D3 r = drot(tq, c);
                c = {r.x + tp.x, r.y + tp.y, r.z + tp.z};
            }
            c = {c.x + off.x, c.y + off.y, c.z + off.z};
            fr.com = make_float4((float)c.x, (float)c.y, (float)c.z, 0.f);
            // getInnerRadius: min|s| x the leaf's
            double inner = hull ? hull->inner_radius
                                : (d.shape_type == CC_SHAPE_BOX
                                       ? std::min((double)d.shape_params[0],
                                                  std::min((double)d.shape_params[1], (double)d.shape_params[2]))
                                       : (double)d.shape_params[0]);
            if (d.shape_type == CC_SHAPE_CYLINDER)
                inner = std::min((double)d.shape_params[0], (double)d.shape_params[1]);
            if (mesh || plane) inner = 0;
            if (cmp) inner = cmp->inner;
            double minScale = std::min(std::fabs(sc[0]), std::min(std::fabs(sc[1]), std::fabs(sc[2])));
            fr.t_pos = make_float4((float)tp.x, (float)tp.y, (float)tp.z, (float)(minScale * inner));
            fr.t_rot = make_float4((float)tq.x, (float)tq.y, (float)tq.z, (float)tq.w);
            any_decorated = true;
        }
        frames[i] = fr;
        int dof = d.allowed_dofs & 63;
        float inv_mass = 0.f;
        float3 inv_i = f3(0.f, 0.f, 0.f);
        if (d.motion_type != CC_STATIC && !mesh && !plane) {
            if ((dof & 7) != 0) {
                if (!(mass > 0)) return CC_ERR_INVALID;
                inv_mass = (float)(1.0 / mass);
            }
            if (((dof >> 3) & 7) != 0) {
                double l = idiag[0] * idiag[0] + idiag[1] * idiag[1] + idiag[2] * idiag[2];
                if (l > 1e-20)
                    inv_i = f3(idiag[0] != 0 ? (float)(1.0 / idiag[0]) : 0.f, idiag[1] != 0 ? (float)(1.0 / idiag[1]) : 0.f,
                               idiag[2] != 0 ? (float)(1.0 / idiag[2]) : 0.f);
                else
                    inv_i = f3(2.5f * inv_mass, 2.5f * inv_mass, 2.5f * inv_mass);
            }
        }
        pos[i] = make_float4(d.position[0], d.position[1], d.position[2], 0.f);
        quat[i] = make_float4(d.quaternion[0], d.quaternion[1], d.quaternion[2], d.quaternion[3]);
        com[i] = pos[i];  // the shape's centre of mass is its origin, hulls aside
        if (decorated) {  // updateCenterOfMassPosition rigid-body.ts:527-536: position + rotation x com
            D3 c = drot(dq(quat[i]), D3{fr.com.x, fr.com.y, fr.com.z});
            com[i] = make_float4((float)(d.position[0] + c.x), (float)(d.position[1] + c.y), (float)(d.position[2] + c.z),
                                 0.f);
        } else if (hull) {  // updateCenterOfMassPosition rigid-body.ts:527-536: position + rotation x com
            DQ q = dq(quat[i]);
            D3 c = drot(q, D3{hull->com.x, hull->com.y, hull->com.z});
            com[i] = make_float4((float)(d.position[0] + c.x), (float)(d.position[1] + c.y), (float)(d.position[2] + c.z),
                                 0.f);
        }
        lin[i] = make_float4(d.linear_velocity[0], d.linear_velocity[1], d.linear_velocity[2], 0.f);
        ang[i] = make_float4(d.angular_velocity[0], d.angular_velocity[1], d.angular_velocity[2], 0.f);
        zero[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        ii[i] = make_float4(inv_i.x, inv_i.y, inv_i.z, inv_mass);
        ir[i] = make_float4(0.f, 0.f, 0.f, 1.f);
        sh[i] = make_float4(d.shape_params[0], d.shape_params[1], d.shape_params[2], d.shape_params[3]);
        if (plane) sh[i] = make_float4((float)pn.x, (float)pn.y, (float)pn.z, d.shape_params[3]);
        if (scaled) {  // the scale baked into the leaf (setBoxSupport support.ts:343-372, sphere.ts:195-197,
                       // capsule.ts:308-318)
            const double ax = std::fabs(sc[0]), ay = std::fabs(sc[1]), az = std::fabs(sc[2]);
            if (d.shape_type == CC_SHAPE_BOX)
                sh[i] = make_float4((float)(ax * d.shape_params[0]), (float)(ay * d.shape_params[1]),
                                    (float)(az * d.shape_params[2]),
                                    (float)std::min(d.shape_params[3] * std::min(ax, std::min(ay, az)), 0.05));
            else if (d.shape_type == CC_SHAPE_CYLINDER)  // setCylinder*Support cylinder.ts: |s.x| throughout
                sh[i] = make_float4((float)(ax * d.shape_params[0]), (float)(ax * d.shape_params[1]),
                                    (float)(ax * d.shape_params[2]), 0.f);
            else
                sh[i] = make_float4((float)(ax * d.shape_params[0]), (float)(ax * d.shape_params[1]), 0.f, 0.f);
        }
        if (hull || (decorated && !mesh && !plane) || given_tensor) {  // principal axes of a full inertia tensor
            DQ r = quat_from_columns(D3{irot[0], irot[3], irot[6]}, D3{irot[1], irot[4], irot[7]},
                                     D3{irot[2], irot[5], irot[8]});
            ir[i] = make_float4((float)r.x, (float)r.y, (float)r.z, (float)r.w);
        }
        if (hull) {
            float hi_bits;
            memcpy(&hi_bits, &hull_index, sizeof(float));
            sh[i] = make_float4(hi_bits, (float)hull->convex_radius, 0.f, 0.f);
        }
        if (mesh) {
            float mi_bits;
            memcpy(&mi_bits, &mesh_index, sizeof(float));
            sh[i] = make_float4(mi_bits, 0.f, 0.f, 0.f);
        }
        if (cmp) {
            float ci_bits;
            memcpy(&ci_bits, &cmp_index, sizeof(float));
            sh[i] = make_float4(ci_bits, 0.f, 0.f, 0.f);
        }
        mat[i] = make_float4(d.friction, d.restitution, d.gravity_factor, 0.f);
        damp[i] = make_float4(d.linear_damping, d.angular_damping, d.max_linear_velocity, d.max_angular_velocity);
        uint32_t f = (uint32_t)d.motion_type;
        if (d.allow_sleeping) f |= F_ALLOW_SLEEP;
        f |= shape_bits(d.shape_type);
        f |= (uint32_t)dof << F_DOF_SHIFT;
        f |= (uint32_t)(d.friction_combine & 7) << F_FCOMB_SHIFT;
        f |= (uint32_t)(d.restitution_combine & 7) << F_RCOMB_SHIFT;
        f |= (uint32_t)(d.object_layer & 31) << F_LAYER_SHIFT;
        if (d.motion_quality == CC_MOTION_LINEAR_CAST) f |= F_LINEAR_CAST;
        if (decorated) f |= F_DECORATED;
        flags[i] = f;
        groups[i] = make_uint2(d.collision_groups, d.collision_mask);
        world[i] = d.world;
        // resetSleepTimer sleep.ts:123-130
        float3 e = mesh   ? f3((float)(0.5 * (mesh->hi[0] - mesh->lo[0])), (float)(0.5 * (mesh->hi[1] - mesh->lo[1])),
                               (float)(0.5 * (mesh->hi[2] - mesh->lo[2])))
                   : hull ? f3((float)(0.5 * (hull->hi.x - hull->lo.x)), (float)(0.5 * (hull->hi.y - hull->lo.y)),
                             (float)(0.5 * (hull->hi.z - hull->lo.z)))
                   : d.shape_type == CC_SHAPE_BOX
                       ? f3(d.shape_params[0], d.shape_params[1], d.shape_params[2])
                       : (d.shape_type == CC_SHAPE_CAPSULE
                              ? f3(d.shape_params[0], d.shape_params[1] + d.shape_params[0], d.shape_params[0])
                              : (d.shape_type == CC_SHAPE_CYLINDER
                                     ? f3(d.shape_params[1], d.shape_params[0], d.shape_params[1])
                                     : f3(d.shape_params[0], d.shape_params[0], d.shape_params[0])));
        if (decorated)  // half extents of the decorated shape's bounds
            e = f3((float)(0.5 * (fr.hi[0] - fr.lo[0])), (float)(0.5 * (fr.hi[1] - fr.lo[1])),
                   (float)(0.5 * (fr.hi[2] - fr.lo[2])));
        float3 c = xyz(com[i]);
        float3 p[3];
        p[0] = c;
        int lowest = (e.x <= e.y && e.x <= e.z) ? 0 : (e.y <= e.z ? 1 : 2);
        float3 X = f3(1, 0, 0), Y = f3(0, 1, 0), Z = f3(0, 0, 1);
        float4 q = quat[i];
        if (lowest == 0) {
            p[1] = c + qrot(q, Y) * e.y;
            p[2] = c + qrot(q, Z) * e.z;
        } else if (lowest == 1) {
            p[1] = c + qrot(q, X) * e.x;
            p[2] = c + qrot(q, Z) * e.z;
        } else {
            p[1] = c + qrot(q, X) * e.x;
            p[2] = c + qrot(q, Y) * e.y;
        }
        for (int k = 0; k < 3; k++) sph[3 * i + k] = make_float4(p[k].x, p[k].y, p[k].z, 0.f);
        if (out_index) out_index[i] = w.n + i;
    }
    size_t o = w.n;
    cudaStream_t s = W->stream;
    if (any_decorated && !w.frames) {  // the decorator records, allocated with the first decorated body
        int r = dalloc(&w.frames, w.cap);
        if (r != CC_OK) return r;
        CC_TRY(cudaMemset(w.frames, 0, sizeof(DevFrame) * (size_t)w.cap));
        drop_graph(W);
    }
    if (w.frames) CC_TRY(cudaMemcpyAsync(w.frames + o, frames.data(), sizeof(DevFrame) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.pos + o, pos.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.quat + o, quat.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.com + o, com.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.linvel + o, lin.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.angvel + o, ang.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.force + o, zero.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.torque + o, zero.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.inv_inertia + o, ii.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.inertia_rot + o, ir.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.shape + o, sh.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.material + o, mat.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.damping + o, damp.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.flags + o, flags.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.iter_ovr + o, ovr.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.groups + o, groups.data(), sizeof(uint2) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.world + o, world.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.sleep_sph + 3 * o, sph.data(), sizeof(float4) * 3 * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaMemcpyAsync(w.sleep_timer + o, timer.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    CC_TRY(cudaStreamSynchronize(s));
    int lc = 0, mc = 0, cc = 0;
    for (int i = 0; i < n; i++) {
        lc += (flags[i] & F_LINEAR_CAST) != 0;
        mc += shape_of(flags[i]) == SHAPE_MESH;
        cc += shape_of(flags[i]) == SHAPE_COMPOUND;
    }
    if (cc > 0 && !w.compound_pairs) {  // the compound pairs' list and their 32-manifold slots
        int r;
        if ((r = dalloc(&w.compound_pairs, (size_t)w.max_pairs)) != CC_OK) return r;
        if (!w.mesh_big_red) {
            char *big = nullptr;
            if ((r = dalloc(&big, mesh_big_slot_bytes() * (size_t)MESH_BIG_THREADS)) != CC_OK) return r;
            w.mesh_big_red = big;
        }
    }
    w.num_compound_bodies += cc;
    if (mc > 0 && !w.mesh_pairs) {
        int r;
        if ((r = dalloc(&w.mesh_pairs, (size_t)w.max_pairs)) != CC_OK ||
            (r = dalloc(&w.mesh_epa_base, (size_t)w.max_pairs)) != CC_OK ||
            (r = dalloc(&w.mesh_epa_count, (size_t)w.max_pairs)) != CC_OK ||
            (r = dalloc(&w.mesh_big, (size_t)w.max_pairs)) != CC_OK)
            return r;
        if (!w.mesh_big_red) {
            char *big = nullptr;
            if ((r = dalloc(&big, mesh_big_slot_bytes() * (size_t)MESH_BIG_THREADS)) != CC_OK) return r;
            w.mesh_big_red = big;
        }
    }
    w.num_mesh_bodies += mc;
    if (lc > 0) {
        int r = ensure_ccd_buffers(W);
        if (r != CC_OK) return r;
    }
    w.num_linear_cast += lc;
    w.n += n;
    drop_graph(W);  // body count changed: the captured step graph no longer matches
    return CC_OK;
}

}  // extern "C"

// one step's launch sequence (update.ts:45-239); `ev` (optional, CC_PROFILE_STAGES + 1
// events) brackets the stages for the stage profiler
constexpr int CC_PROFILE_STAGES = 7;
static void enqueue_step(cc_world *W, float dt, float ratio, cudaEvent_t *ev = nullptr, TapeStep *tape = nullptr) {
    DevWorld &w = W->w;
    cudaStream_t s = W->stream;
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], s);
    };
    mark(0);
    cudaMemsetAsync(w.ctr, 0, sizeof(DevCounters), s);
    launch_cache_begin(w, s);
    launch_integrate_forces(w, dt, s);
    mark(1);
    launch_broadphase(w, s);
    mark(2);
    launch_narrowphase(w, dt, s, ev ? ev[3] : nullptr);
    mark(4);
    launch_contacts_and_islands(w, dt, ratio, s);
    if (tape) launch_tape_record(w, *tape, s);
    mark(5);
    if (dt > 0.f) {
        if (w.num_linear_cast > 0) {
            // LINEAR_CAST bodies: velocities and integration, the continuous-collision pass, then
            // the position solve (update.ts:168-227)
            launch_solver(w, dt, ratio, s, ev ? ev[6] : nullptr, SOLVE_VELOCITY);
            launch_ccd(w, dt, s);
            launch_solver(w, dt, ratio, s, nullptr, SOLVE_POSITION);
        } else {
            launch_solver(w, dt, ratio, s, ev ? ev[6] : nullptr);
        }
    }
    if (ev && !(dt > 0.f)) mark(6);
    mark(7);
    cudaMemcpyAsync(W->h_ctr, w.ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, s);
}

// hulls and meshes added since the last launch go to the device in one upload each
static int upload_hulls(cc_world *W);
static int upload_meshes(cc_world *W);
static int upload_compounds(cc_world *W);
static int sync_shapes(cc_world *W) {
    int r = CC_OK;
    if (W->compounds_dirty) {
        if ((r = upload_compounds(W)) != CC_OK) return r;
        W->compounds_dirty = false;
    }
    if (W->hulls_dirty) {
        if ((r = upload_hulls(W)) != CC_OK) return r;
        W->hulls_dirty = false;
    }
    if (W->meshes_dirty) {
        if ((r = upload_meshes(W)) != CC_OK) return r;
        W->meshes_dirty = false;
    }
    return r;
}

static int run_steps(cc_world *W, float dt, int n_steps) {
    if (W->w.n == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    upload_settings(W->dev_settings, W->settings.speculative_contact_distance, W->stream);
    int status = CC_OK;
    if (!W->ev_begin) {
        CC_TRY(cudaEventCreate(&W->ev_begin));
        CC_TRY(cudaEventCreate(&W->ev_end));
    }
    CC_TRY(cudaEventRecord(W->ev_begin, W->stream));
    for (int i = 0; i < n_steps; i++) {
        // warm start ratio dt / previous dt, 0 on the first step (update.ts:118-124)
        float ratio = (W->settings.warm_starting && W->prev_dt > 0) ? (float)(dt / W->prev_dt) : 0.f;
        if (dt <= 0.f) ratio = 0.f;
        bool use_graph = ratio != 0.f;  // the first step after creation runs eagerly
        if (use_graph) {
            if (!W->graph_exec || W->graph_dt != dt || W->graph_ratio != ratio) {
                if (W->graph_exec) cudaGraphExecDestroy(W->graph_exec);
                if (W->graph) cudaGraphDestroy(W->graph);
                W->graph_exec = nullptr;
                W->graph = nullptr;
                CC_TRY(cudaStreamBeginCapture(W->stream, cudaStreamCaptureModeThreadLocal));
                enqueue_step(W, dt, ratio);
                CC_TRY(cudaStreamEndCapture(W->stream, &W->graph));
                CC_TRY(cudaGraphInstantiate(&W->graph_exec, W->graph, 0));
                W->graph_dt = dt;
                W->graph_ratio = ratio;
            }
            CC_TRY(cudaGraphLaunch(W->graph_exec, W->stream));
        } else {
            enqueue_step(W, dt, ratio);
        }
        if (dt > 0.f) W->prev_dt = dt;
        W->steps_done++;
    }
    CC_TRY(cudaEventRecord(W->ev_end, W->stream));
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaGetLastError());
    cudaEventElapsedTime(&W->last_call_ms, W->ev_begin, W->ev_end);
    W->last_ctr = *W->h_ctr;
    if (W->last_ctr.overflow) status = (W->last_ctr.overflow & OVF_TIMEOUT) ? CC_ERR_TIMEOUT : CC_ERR_CAPACITY;
    W->last_status = status;
    return status;
}

__global__ void k_pack_state(DevWorld w, float *rows, unsigned char *sleeping) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        float *o = rows + (size_t)i * 16;
        float4 p = w.pos[i], q = w.quat[i], v = w.linvel[i], a = w.angvel[i], c = w.com[i];
        o[0] = p.x;
        o[1] = p.y;
        o[2] = p.z;
        o[3] = q.x;
        o[4] = q.y;
        o[5] = q.z;
        o[6] = q.w;
        o[7] = v.x;
        o[8] = v.y;
        o[9] = v.z;
        o[10] = a.x;
        o[11] = a.y;
        o[12] = a.z;
        o[13] = c.x;
        o[14] = c.y;
        o[15] = c.z;
        if (sleeping) sleeping[i] = sleeping_of(w.flags[i]) ? 1 : 0;
    }
}

// setTransform / setLinearVelocity / setAngularVelocity: pose, velocity and the
// derived centre of mass (rigid-body.ts:527-536, 758-774)
__global__ void k_unpack_state(DevWorld w, const float *rows) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        const float *o = rows + (size_t)i * 16;
        w.pos[i] = make_float4(o[0], o[1], o[2], 0.f);
        w.quat[i] = make_float4(o[3], o[4], o[5], o[6]);
        w.linvel[i] = make_float4(o[7], o[8], o[9], 0.f);
        w.angvel[i] = make_float4(o[10], o[11], o[12], 0.f);
        float3 c = qrot(w.quat[i], shape_com(w, i, w.flags[i], w.shape[i]));
        w.com[i] = make_float4(o[0] + c.x, o[1] + c.y, o[2] + c.z, 0.f);
    }
}

extern "C" {

int cc_world_step(cc_world *W, float dt, int32_t n_steps) {
    if (!W || n_steps < 0 || !std::isfinite(dt)) return CC_ERR_INVALID;
    return run_steps(W, dt, n_steps);
}

int cc_world_get_state(cc_world *W, float *rows, uint8_t *sleeping) {
    if (!W || !rows) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (w.n == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    k_pack_state<<<grid_for(w.n, 256), 256, 0, W->stream>>>(w, W->d_state_rows, nullptr);
    CC_TRY(cudaMemcpyAsync(rows, W->d_state_rows, sizeof(float) * 16 * w.n, cudaMemcpyDeviceToHost, W->stream));
    if (sleeping) {
        std::vector<uint32_t> f(w.n);
        CC_TRY(cudaMemcpyAsync(f.data(), w.flags, sizeof(uint32_t) * w.n, cudaMemcpyDeviceToHost, W->stream));
        CC_TRY(cudaStreamSynchronize(W->stream));
        for (int i = 0; i < w.n; i++) sleeping[i] = sleeping_of(f[i]) ? 1 : 0;
    }
    CC_TRY(cudaStreamSynchronize(W->stream));
    return CC_OK;
}

int cc_world_set_state(cc_world *W, const float *rows) {
    if (!W || !rows) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (w.n == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    CC_TRY(cudaMemcpyAsync(W->d_state_rows, rows, sizeof(float) * 16 * w.n, cudaMemcpyHostToDevice, W->stream));
    k_unpack_state<<<grid_for(w.n, 256), 256, 0, W->stream>>>(w, W->d_state_rows);
    CC_TRY(cudaStreamSynchronize(W->stream));
    return CC_OK;
}

int cc_world_step_host(cc_world *W, float dt, const float *state_in, float *state_out) {
    if (!W || !state_in || !state_out) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (w.n == 0) return CC_OK;
    CC_TRY(cudaMemcpyAsync(W->d_state_rows, state_in, sizeof(float) * 16 * w.n, cudaMemcpyHostToDevice, W->stream));
    k_unpack_state<<<grid_for(w.n, 256), 256, 0, W->stream>>>(w, W->d_state_rows);
    int st = run_steps(W, dt, 1);
    k_pack_state<<<grid_for(w.n, 256), 256, 0, W->stream>>>(w, W->d_state_rows, nullptr);
    CC_TRY(cudaMemcpyAsync(state_out, W->d_state_rows, sizeof(float) * 16 * w.n, cudaMemcpyDeviceToHost, W->stream));
    CC_TRY(cudaStreamSynchronize(W->stream));
    return st;
}

int cc_world_get_pairs(cc_world *W, int32_t *out, int32_t capacity, int32_t *count) {
    if (!W || !count) return CC_ERR_INVALID;
    int np = W->last_ctr.num_pairs;
    if (np > W->w.max_pairs) np = W->w.max_pairs;
    *count = np;
    if (!out) return CC_OK;
    if (capacity < np) return CC_ERR_CAPACITY;
    if (np > 0) CC_TRY(cudaMemcpy(out, W->w.pairs, sizeof(int2) * np, cudaMemcpyDeviceToHost));
    return CC_OK;
}

int cc_world_get_manifold_sub_shapes(cc_world *W, uint32_t *out, int32_t capacity, int32_t *count) {
    if (!W || !count) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    int nm = W->last_ctr.num_manifolds;
    if (nm > w.max_manifolds) nm = w.max_manifolds;
    std::vector<Manifold> ms(nm);
    std::vector<int> cm(nm);
    if (nm > 0) {
        CC_TRY(cudaMemcpy(ms.data(), w.manifolds, sizeof(Manifold) * nm, cudaMemcpyDeviceToHost));
        CC_TRY(cudaMemcpy(cm.data(), w.cons_of_manifold, sizeof(int) * nm, cudaMemcpyDeviceToHost));
    }
    int k = 0;
    for (int i = 0; i < nm; i++) {
        if (cm[i] < 0) continue;
        if (out && k >= capacity) return CC_ERR_CAPACITY;
        if (out) {
            bool swap = ms[i].a > ms[i].b;
            out[2 * k] = swap ? ms[i].sub_b : ms[i].sub_a;
            out[2 * k + 1] = swap ? ms[i].sub_a : ms[i].sub_b;
        }
        k++;
    }
    *count = k;
    return CC_OK;
}

static_assert(sizeof(cc_ray) == sizeof(DevRay) && sizeof(cc_ray_hit) == sizeof(DevRayHit), "ray layouts");

static int queue_cast_rays(cc_world *W, const DevRay *rays, int n, const cc_query_filter *f, DevRayHit *hits,
                           int mode = COLLECT_CLOSEST, int cap = 1, int *counts = nullptr) {
    if (int r = sync_shapes(W)) return r;
    DevWorld &w = W->w;
    DevRayFilter flt{f->object_layer_mask, f->collision_group, f->collision_mask, f->flags};
    if (n > W->q_sort_cap) {
        if (W->q_keys) cudaFree(W->q_keys);
        if (W->q_idx) cudaFree(W->q_idx);
        if (W->q_tmp) cudaFree(W->q_tmp);
        W->q_keys = nullptr;
        W->q_idx = W->q_tmp = nullptr;
        W->q_sort_cap = 0;
        CC_TRY(cudaMalloc(&W->q_keys, sizeof(unsigned long long) * 2 * (size_t)n));
        CC_TRY(cudaMalloc(&W->q_idx, sizeof(int) * 2 * (size_t)n));
        CC_TRY(cudaMalloc(&W->q_tmp, sizeof(int) * radix_tmp_ints(n)));
        W->q_sort_cap = n;
    }
    launch_query_tree(w, W->stream);
    launch_ray_order(w, rays, n, W->q_keys, W->q_idx, W->q_tmp, W->stream);
    launch_cast_rays(w, rays, W->q_idx, n, flt, hits, W->stream, mode, cap, counts);
    return cuda_ok(cudaGetLastError());
}

int cc_world_collide_points_device(cc_world *W, const cc_point *points, int32_t count, const cc_query_filter *filter,
                                   float collision_tolerance, cc_point_hit *hits) {
    if (!W || count < 0 || !filter || (count > 0 && (!points || !hits))) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    DevRayFilter flt{filter->object_layer_mask, filter->collision_group, filter->collision_mask, filter->flags};
    launch_query_tree(W->w, W->stream);
    launch_collide_points(W->w, (const float4 *)points, count, flt, collision_tolerance, (int4 *)hits, W->stream);
    return cuda_ok(cudaGetLastError());
}

int cc_world_collide_points(cc_world *W, const cc_point *points, int32_t count, const cc_query_filter *filter,
                            float collision_tolerance, cc_point_hit *hits) {
    if (!W || count < 0 || !filter || (count > 0 && (!points || !hits))) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    static_assert(sizeof(cc_point) == sizeof(DevRayHit) && sizeof(cc_point_hit) == sizeof(DevRayHit), "16 bytes");
    if (count > W->q_cap) {
        if (W->q_rays) cudaFree(W->q_rays);
        if (W->q_hits) cudaFree(W->q_hits);
        W->q_rays = nullptr;
        W->q_hits = nullptr;
        W->q_cap = 0;
        CC_TRY(cudaMalloc(&W->q_rays, sizeof(DevRay) * (size_t)count));
        CC_TRY(cudaMalloc(&W->q_hits, sizeof(DevRayHit) * (size_t)count));
        W->q_cap = count;
    }
    CC_TRY(cudaMemcpyAsync(W->q_rays, points, sizeof(cc_point) * (size_t)count, cudaMemcpyHostToDevice, W->stream));
    if (int r = cc_world_collide_points_device(W, (const cc_point *)W->q_rays, count, filter, collision_tolerance,
                                               (cc_point_hit *)W->q_hits))
        return r;
    CC_TRY(cudaMemcpyAsync(hits, W->q_hits, sizeof(cc_point_hit) * (size_t)count, cudaMemcpyDeviceToHost, W->stream));
    CC_TRY(cudaStreamSynchronize(W->stream));
    return CC_OK;
}

static_assert(sizeof(cc_shape_cast) == sizeof(DevShapeCast) && sizeof(cc_shape_cast_hit) == sizeof(DevShapeCastHit),
              "shape cast layouts");

// A cast or collide query's shape: a sphere, box or capsule, a cylinder within cylinder.ts's
// limits, or a convex hull of this world named by its index in shape_params[0].
static bool query_shape_valid(const cc_world *W, int t, const float *p) {
    if (t == CC_SHAPE_SPHERE || t == CC_SHAPE_BOX || t == CC_SHAPE_CAPSULE) return true;
    if (t == CC_SHAPE_CYLINDER) return p[2] >= 0.f && p[0] >= p[2] && p[1] >= p[2];
    if (t == CC_SHAPE_CONVEX_HULL) {
        const int h = (int)p[0];
        return p[0] == (float)h && h >= 0 && h < (int)W->hulls.size();
    }
    return false;
}
}  // extern "C"
// the queries as the device reads them: a hull index as int bits, as the bodies' shape records keep it
template <class Q>
static std::vector<Q> device_queries(const Q *q, int n) {
    std::vector<Q> out(q, q + n);
    for (Q &x : out)
        if (x.shape_type == CC_SHAPE_CONVEX_HULL) {
            const int h = (int)x.shape_params[0];
            memcpy(&x.shape_params[0], &h, sizeof(int));
        }
    return out;
}
extern "C" {

int cc_world_cast_shapes_device(cc_world *W, const cc_shape_cast *casts, int32_t count, const cc_query_filter *filter,
                                cc_shape_cast_hit *hits) {
    if (!W || count < 0 || !filter || (count > 0 && (!casts || !hits))) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    DevRayFilter flt{filter->object_layer_mask, filter->collision_group, filter->collision_mask, filter->flags};
    launch_query_tree(W->w, W->stream);
    launch_cast_shapes(W->w, (const DevShapeCast *)casts, count, flt, (DevShapeCastHit *)hits, W->stream);
    return cuda_ok(cudaGetLastError());
}

int cc_world_cast_shapes(cc_world *W, const cc_shape_cast *casts, int32_t count, const cc_query_filter *filter,
                         cc_shape_cast_hit *hits) {
    if (!W || count < 0 || !filter || (count > 0 && (!casts || !hits))) return CC_ERR_INVALID;
    for (int i = 0; i < count; i++)
        if (!query_shape_valid(W, casts[i].shape_type, casts[i].shape_params)) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    const std::vector<cc_shape_cast> dq = device_queries(casts, count);
    void *d = nullptr;
    const size_t in_b = sizeof(cc_shape_cast) * (size_t)count, out_b = sizeof(cc_shape_cast_hit) * (size_t)count;
    CC_TRY(cudaMallocAsync(&d, in_b + out_b, W->stream));
    int r = cuda_ok(cudaMemcpyAsync(d, dq.data(), in_b, cudaMemcpyHostToDevice, W->stream));
    cc_shape_cast_hit *dh = (cc_shape_cast_hit *)((char *)d + in_b);
    if (r == CC_OK) r = cc_world_cast_shapes_device(W, (const cc_shape_cast *)d, count, filter, dh);
    if (r == CC_OK) r = cuda_ok(cudaMemcpyAsync(hits, dh, out_b, cudaMemcpyDeviceToHost, W->stream));
    int ovf = 0;
    if (r == CC_OK)
        r = cuda_ok(cudaMemcpyAsync(&W->h_query_ovf, &W->w.ctr->overflow, sizeof(int), cudaMemcpyDeviceToHost,
                                    W->stream));
    cudaFreeAsync(d, W->stream);
    if (r == CC_OK) r = cuda_ok(cudaStreamSynchronize(W->stream));
    ovf = W->h_query_ovf;
    // a tree walk of these casts outgrew its stack (the step's own flags are in last_ctr)
    if (r == CC_OK && (ovf & OVF_SLOTS) && !(W->last_ctr.overflow & OVF_SLOTS)) r = CC_ERR_CAPACITY;
    return r;
}

int cc_world_cast_rays_device(cc_world *W, const cc_ray *rays, int32_t count, const cc_query_filter *filter,
                              cc_ray_hit *hits) {
    if (!W || count < 0 || !filter || (count > 0 && (!rays || !hits))) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    return queue_cast_rays(W, (const DevRay *)rays, count, filter, (DevRayHit *)hits);
}

int cc_world_cast_rays(cc_world *W, const cc_ray *rays, int32_t count, const cc_query_filter *filter,
                       cc_ray_hit *hits) {
    if (!W || count < 0 || !filter || (count > 0 && (!rays || !hits))) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    if (count > W->q_cap) {
        if (W->q_rays) cudaFree(W->q_rays);
        if (W->q_hits) cudaFree(W->q_hits);
        W->q_rays = nullptr;
        W->q_hits = nullptr;
        W->q_cap = 0;
        CC_TRY(cudaMalloc(&W->q_rays, sizeof(DevRay) * (size_t)count));
        CC_TRY(cudaMalloc(&W->q_hits, sizeof(DevRayHit) * (size_t)count));
        W->q_cap = count;
    }
    CC_TRY(cudaMemcpyAsync(W->q_rays, rays, sizeof(DevRay) * (size_t)count, cudaMemcpyHostToDevice, W->stream));
    if (int r = queue_cast_rays(W, W->q_rays, count, filter, W->q_hits)) return r;
    CC_TRY(cudaMemcpyAsync(hits, W->q_hits, sizeof(DevRayHit) * (size_t)count, cudaMemcpyDeviceToHost, W->stream));
    CC_TRY(cudaStreamSynchronize(W->stream));
    return CC_OK;
}

// ---- the collectors of the batched queries ---------------------------------------
static_assert(sizeof(cc_collide_shape) == sizeof(DevCollideShape) && sizeof(cc_collide_shape_hit) == sizeof(DevCollideHit),
              "collide shape layouts");
static_assert(CC_COLLECT_CLOSEST == COLLECT_CLOSEST && CC_COLLECT_ANY == COLLECT_ANY && CC_COLLECT_ALL == COLLECT_ALL,
              "collector ids");

}  // extern "C"

// One query batch through the device: the inputs copied in, the kernels queued by run(d_in,
// d_hits, d_counts, cap), the hits copied out into count x max_hits records (closest and any: the
// first record of each query) and the counts (the closest collector's from its hit).  Mode ALL
// returns CC_ERR_CAPACITY when a query found more than max_hits hits.
template <typename In, typename Hit, typename Run>
static int run_collect(cc_world *W, const In *in, int count, int mode, int max_hits, Hit *hits, int32_t *counts,
                       Run &&run) {
    const int cap = mode == COLLECT_ALL ? max_hits : 1;
    const size_t in_b = sizeof(In) * (size_t)count, hit_b = sizeof(Hit) * (size_t)count * (size_t)cap,
                 cnt_b = sizeof(int) * (size_t)count;
    const size_t off_h = (in_b + 255) / 256 * 256, off_c = off_h + (hit_b + 255) / 256 * 256;
    char *d = nullptr;
    CC_TRY(cudaMallocAsync((void **)&d, off_c + cnt_b, W->stream));
    int r = cuda_ok(cudaMemcpyAsync(d, in, in_b, cudaMemcpyHostToDevice, W->stream));
    Hit *dh = (Hit *)(d + off_h);
    int *dc = (int *)(d + off_c);
    if (r == CC_OK) r = run((const In *)d, dh, mode == COLLECT_CLOSEST ? nullptr : dc, cap);
    if (r == CC_OK) {
        if (cap == max_hits)
            r = cuda_ok(cudaMemcpyAsync(hits, dh, hit_b, cudaMemcpyDeviceToHost, W->stream));
        else
            r = cuda_ok(cudaMemcpy2DAsync(hits, sizeof(Hit) * (size_t)max_hits, dh, sizeof(Hit), sizeof(Hit), count,
                                          cudaMemcpyDeviceToHost, W->stream));
    }
    if (r == CC_OK && mode != COLLECT_CLOSEST && counts)
        r = cuda_ok(cudaMemcpyAsync(counts, dc, cnt_b, cudaMemcpyDeviceToHost, W->stream));
    cudaFreeAsync(d, W->stream);
    if (r == CC_OK) r = cuda_ok(cudaStreamSynchronize(W->stream));
    if (r != CC_OK) return r;
    if (mode == COLLECT_CLOSEST && counts)
        for (int i = 0; i < count; i++) counts[i] = hits[(size_t)i * max_hits].body >= 0 ? 1 : 0;
    if (mode == COLLECT_ALL)
        for (int i = 0; i < count; i++)
            if (counts[i] > max_hits) return CC_ERR_CAPACITY;
    return CC_OK;
}

static bool collect_args_ok(const void *in, int32_t count, const cc_query_filter *filter, int32_t collector,
                            int32_t max_hits, const void *hits, const int32_t *counts) {
    if (count < 0 || !filter || collector < CC_COLLECT_CLOSEST || collector > CC_COLLECT_ALL || max_hits < 1)
        return false;
    if (count > 0 && (!in || !hits)) return false;
    return !(collector == CC_COLLECT_ALL && count > 0 && !counts);
}

extern "C" {

int cc_world_cast_rays_collect(cc_world *W, const cc_ray *rays, int32_t count, const cc_query_filter *filter,
                               int32_t collector, int32_t max_hits, cc_ray_hit *hits, int32_t *counts) {
    if (!W || !collect_args_ok(rays, count, filter, collector, max_hits, hits, counts)) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    return run_collect(W, (const DevRay *)rays, count, collector, max_hits, (DevRayHit *)hits, counts,
                       [&](const DevRay *d, DevRayHit *h, int *c, int cap) {
                           return queue_cast_rays(W, d, count, filter, h, collector, cap, c);
                       });
}

int cc_world_cast_shapes_collect(cc_world *W, const cc_shape_cast *casts, int32_t count, const cc_query_filter *filter,
                                 int32_t collector, int32_t max_hits, cc_shape_cast_hit *hits, int32_t *counts) {
    if (!W || !collect_args_ok(casts, count, filter, collector, max_hits, hits, counts)) return CC_ERR_INVALID;
    for (int i = 0; i < count; i++)
        if (!query_shape_valid(W, casts[i].shape_type, casts[i].shape_params)) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    DevRayFilter flt{filter->object_layer_mask, filter->collision_group, filter->collision_mask, filter->flags};
    const std::vector<cc_shape_cast> dq = device_queries(casts, count);
    return run_collect(W, (const DevShapeCast *)dq.data(), count, collector, max_hits, (DevShapeCastHit *)hits, counts,
                       [&](const DevShapeCast *d, DevShapeCastHit *h, int *c, int cap) {
                           launch_query_tree(W->w, W->stream);
                           launch_cast_shapes(W->w, d, count, flt, h, W->stream, collector, cap, c);
                           return cuda_ok(cudaGetLastError());
                       });
}

int cc_world_collide_shapes(cc_world *W, const cc_collide_shape *shapes, int32_t count, const cc_query_filter *filter,
                            const cc_collide_shape_settings *settings, int32_t collector, int32_t max_hits,
                            cc_collide_shape_hit *hits, int32_t *counts) {
    if (!W || !settings || !collect_args_ok(shapes, count, filter, collector, max_hits, hits, counts))
        return CC_ERR_INVALID;
    if (!(settings->max_separation_distance >= 0.f) || !(settings->collision_tolerance > 0.f) ||
        !(settings->penetration_tolerance > 0.f))
        return CC_ERR_INVALID;
    for (int i = 0; i < count; i++)
        if (!query_shape_valid(W, shapes[i].shape_type, shapes[i].shape_params)) return CC_ERR_INVALID;
    if (count == 0) return CC_OK;
    if (!W->w.epa_scratch) return CC_ERR_UNSUPPORTED;
    const std::vector<cc_collide_shape> dq = device_queries(shapes, count);
    if (int r = sync_shapes(W)) return r;
    DevRayFilter flt{filter->object_layer_mask, filter->collision_group, filter->collision_mask, filter->flags};
    DevCollideSettings cs{settings->max_separation_distance, settings->collision_tolerance,
                          settings->penetration_tolerance, settings->collide_with_backfaces != 0};
    // every query reports its count, the closest collector's too
    const int mode = collector;
    const int cap = mode == COLLECT_ALL ? max_hits : 1;
    const size_t in_b = sizeof(DevCollideShape) * (size_t)count,
                 hit_b = sizeof(DevCollideHit) * (size_t)count * (size_t)cap, cnt_b = sizeof(int) * (size_t)count;
    const size_t off_h = (in_b + 255) / 256 * 256, off_c = off_h + (hit_b + 255) / 256 * 256;
    char *d = nullptr;
    CC_TRY(cudaMallocAsync((void **)&d, off_c + cnt_b, W->stream));
    DevCollideHit *dh = (DevCollideHit *)(d + off_h);
    int *dc = (int *)(d + off_c);
    int r = cuda_ok(cudaMemcpyAsync(d, dq.data(), in_b, cudaMemcpyHostToDevice, W->stream));
    if (r == CC_OK) {
        launch_query_tree(W->w, W->stream);
        launch_collide_shapes(W->w, (const DevCollideShape *)d, count, flt, cs, mode, cap, dh, dc, W->stream);
        r = cuda_ok(cudaGetLastError());
    }
    if (r == CC_OK) {
        if (cap == max_hits)
            r = cuda_ok(cudaMemcpyAsync(hits, dh, hit_b, cudaMemcpyDeviceToHost, W->stream));
        else
            r = cuda_ok(cudaMemcpy2DAsync(hits, sizeof(DevCollideHit) * (size_t)max_hits, dh, sizeof(DevCollideHit),
                                          sizeof(DevCollideHit), count, cudaMemcpyDeviceToHost, W->stream));
    }
    if (r == CC_OK && counts) r = cuda_ok(cudaMemcpyAsync(counts, dc, cnt_b, cudaMemcpyDeviceToHost, W->stream));
    cudaFreeAsync(d, W->stream);
    if (r == CC_OK) r = cuda_ok(cudaStreamSynchronize(W->stream));
    if (r != CC_OK) return r;
    if (mode == COLLECT_ALL)
        for (int i = 0; i < count; i++)
            if (counts[i] > max_hits) return CC_ERR_CAPACITY;
    return CC_OK;
}

int cc_world_get_manifolds(cc_world *W, float *out, int32_t capacity, int32_t *count) {
    if (!W || !count) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    int nm = W->last_ctr.num_manifolds;
    if (nm > w.max_manifolds) nm = w.max_manifolds;
    std::vector<Manifold> ms(nm);
    std::vector<int> cm(nm);
    std::vector<ContactConstraint> cs(nm);
    if (nm > 0) {
        CC_TRY(cudaMemcpy(ms.data(), w.manifolds, sizeof(Manifold) * nm, cudaMemcpyDeviceToHost));
        CC_TRY(cudaMemcpy(cm.data(), w.cons_of_manifold, sizeof(int) * nm, cudaMemcpyDeviceToHost));
        CC_TRY(cudaMemcpy(cs.data(), w.cons, sizeof(ContactConstraint) * nm, cudaMemcpyDeviceToHost));
    }
    int k = 0;
    for (int i = 0; i < nm; i++) {
        if (cm[i] < 0) continue;
        if (out && k >= capacity) return CC_ERR_CAPACITY;
        if (out) {
            const Manifold &m = ms[i];
            float *o = out + 32 * (size_t)k;
            int A = m.a, B = m.b;
            float3 n = m.normal;
            bool swap = A > B;
            float3 base = m.base;
            o[0] = (float)(swap ? B : A);
            o[1] = (float)(swap ? A : B);
            o[2] = (float)m.n;
            float3 nn = swap ? -n : n;
            o[3] = nn.x;
            o[4] = nn.y;
            o[5] = nn.z;
            o[6] = m.depth;
            float lsum = 0.f;  // accumulated normal impulse of the contact after the solve
            for (int j = 0; j < cs[i].n; j++) lsum += cs[i].p[j].lam_n;
            o[7] = lsum;
            for (int j = 0; j < 4; j++) {
                float *p = o + 8 + 6 * j;
                if (j < m.n) {
                    float3 pa = (swap ? m.rb[j] : m.ra[j]) + base;
                    float3 pb = (swap ? m.ra[j] : m.rb[j]) + base;
                    p[0] = pa.x;
                    p[1] = pa.y;
                    p[2] = pa.z;
                    p[3] = pb.x;
                    p[4] = pb.y;
                    p[5] = pb.z;
                } else {
                    for (int t = 0; t < 6; t++) p[t] = 0.f;
                }
            }
        }
        k++;
    }
    *count = k;
    return CC_OK;
}

// Diagnostic readout of the last step's islands: island index per body (-1 for
// static or sleeping bodies) and, per contact constraint, (bodyA, bodyB, island).
int cc_world_debug_islands(cc_world *W, int32_t *island_of_body, int32_t *cons_rows, int32_t capacity,
                           int32_t *count) {
    if (!W || !count) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    int nm = W->last_ctr.num_manifolds;
    if (nm > w.max_manifolds) nm = w.max_manifolds;
    std::vector<ContactConstraint> cs(nm);
    std::vector<int> cm(nm);
    if (nm > 0) {
        CC_TRY(cudaMemcpy(cs.data(), w.cons, sizeof(ContactConstraint) * nm, cudaMemcpyDeviceToHost));
        CC_TRY(cudaMemcpy(cm.data(), w.cons_of_manifold, sizeof(int) * nm, cudaMemcpyDeviceToHost));
    }
    if (island_of_body && w.n > 0)
        CC_TRY(cudaMemcpy(island_of_body, w.island_of_body, sizeof(int) * w.n, cudaMemcpyDeviceToHost));
    int k = 0;
    for (int i = 0; i < nm; i++) {
        if (cm[i] < 0) continue;
        if (cons_rows) {
            if (k >= capacity) return CC_ERR_CAPACITY;
            cons_rows[3 * k] = cs[i].a;
            cons_rows[3 * k + 1] = cs[i].b;
            cons_rows[3 * k + 2] = cs[i].island;
        }
        k++;
    }
    *count = k;
    return CC_OK;
}

int cc_world_get_island_iterations(cc_world *W, int32_t *out) {
    if (!W || !out) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (w.n == 0) return CC_OK;
    int ni = W->last_ctr.num_islands;
    std::vector<int> iob((size_t)w.n), it(3 * (size_t)(ni > 0 ? ni : 1));
    CC_TRY(cudaMemcpy(iob.data(), w.island_of_body, sizeof(int) * w.n, cudaMemcpyDeviceToHost));
    if (ni > 0) CC_TRY(cudaMemcpy(it.data(), w.island_iters, sizeof(int) * 3 * (size_t)ni, cudaMemcpyDeviceToHost));
    for (int i = 0; i < w.n; i++) {
        int isl = iob[i];
        if (isl < 0 || isl >= ni) {
            out[2 * i] = out[2 * i + 1] = -1;
            continue;
        }
        int v = it[3 * isl], p = it[3 * isl + 1], f = it[3 * isl + 2];
        if (f & 1) v = v > W->settings.velocity_iterations ? v : W->settings.velocity_iterations;
        if (f & 2) p = p > W->settings.position_iterations ? p : W->settings.position_iterations;
        out[2 * i] = v;
        out[2 * i + 1] = p;
    }
    return CC_OK;
}

// Stage profiler: runs n_steps with CUDA events between the stages and returns the
// mean milliseconds of each stage: integrate forces, broadphase, narrowphase (GJK,
// faces, clipping), EPA, contacts + islands, per-thread island solve, per-CTA island
// solve.
int cc_world_profile_steps(cc_world *W, float dt, int32_t n_steps, float *stage_ms, int32_t n_stages) {
    if (!W || !stage_ms || n_steps <= 0 || n_stages < CC_PROFILE_STAGES) return CC_ERR_INVALID;
    if (W->w.n == 0) return CC_OK;
    if (int r = sync_shapes(W)) return r;
    upload_settings(W->dev_settings, W->settings.speculative_contact_distance, W->stream);
    cudaEvent_t ev[CC_PROFILE_STAGES + 1];
    for (int k = 0; k <= CC_PROFILE_STAGES; k++) CC_TRY(cudaEventCreate(&ev[k]));
    double acc[CC_PROFILE_STAGES] = {};
    int st = CC_OK;
    for (int i = 0; i < n_steps; i++) {
        float ratio = (W->settings.warm_starting && W->prev_dt > 0) ? (float)(dt / W->prev_dt) : 0.f;
        enqueue_step(W, dt, ratio, ev);
        if (dt > 0.f) W->prev_dt = dt;
        W->steps_done++;
        CC_TRY(cudaEventSynchronize(ev[CC_PROFILE_STAGES]));
        for (int k = 0; k < CC_PROFILE_STAGES; k++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            acc[k] += ms;
        }
    }
    CC_TRY(cudaStreamSynchronize(W->stream));
    W->last_ctr = *W->h_ctr;
    if (W->last_ctr.overflow) st = CC_ERR_CAPACITY;
    for (int k = 0; k <= CC_PROFILE_STAGES; k++) cudaEventDestroy(ev[k]);
    for (int k = 0; k < CC_PROFILE_STAGES; k++) stage_ms[k] = (float)(acc[k] / n_steps);
    for (int k = CC_PROFILE_STAGES; k < n_stages; k++) stage_ms[k] = 0.f;
    return st;
}

int cc_world_get_contact_events(cc_world *W, int32_t *out, int32_t capacity, int32_t *count) {
    if (!W || !count || capacity < 0 || (capacity > 0 && !out)) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    const DevCounters &c = W->last_ctr;
    int nm = c.num_manifolds < w.max_manifolds ? c.num_manifolds : w.max_manifolds;
    int nr = c.num_removed < w.max_manifolds ? c.num_removed : w.max_manifolds;
    std::vector<int> ev((size_t)nm);
    std::vector<Manifold> man((size_t)nm);
    std::vector<unsigned long long> rk((size_t)nr);
    if (nm > 0) {
        CC_TRY(cudaMemcpyAsync(ev.data(), w.contact_event, sizeof(int) * nm, cudaMemcpyDeviceToHost, W->stream));
        CC_TRY(cudaMemcpyAsync(man.data(), w.manifolds, sizeof(Manifold) * nm, cudaMemcpyDeviceToHost, W->stream));
    }
    if (nr > 0)
        CC_TRY(cudaMemcpyAsync(rk.data(), w.removed_keys, sizeof(unsigned long long) * nr, cudaMemcpyDeviceToHost,
                               W->stream));
    CC_TRY(cudaStreamSynchronize(W->stream));
    // (type, body A, body B) with A < B, sorted for a deterministic order
    std::vector<std::array<int32_t, 3>> rows;
    rows.reserve((size_t)nm + nr);
    for (int i = 0; i < nm; i++) {
        if (ev[i] == 0) continue;
        int a = man[i].a, b = man[i].b;
        rows.push_back({ev[i], a < b ? a : b, a < b ? b : a});
    }
    for (int i = 0; i < nr; i++) {
        const unsigned long long k = rk[i];
        if (k >> 63) {  // a mesh triangle's contact: A, B and the triangle in 21 bits each
            const unsigned long long M = (1ull << MESH_KEY_BITS) - 1ull;
            rows.push_back({3, (int32_t)((k >> 42) & M), (int32_t)((k >> 21) & M)});
        } else {
            rows.push_back({3, (int32_t)(k >> 32), (int32_t)(k & 0xffffffffu)});
        }
    }
    std::sort(rows.begin(), rows.end());
    *count = (int32_t)rows.size();
    int32_t k = 0;
    for (const auto &r : rows) {
        if (k >= capacity) break;
        out[3 * k] = r[0];
        out[3 * k + 1] = r[1];
        out[3 * k + 2] = r[2];
        k++;
    }
    return (c.overflow & OVF_CACHE) || c.num_removed > w.max_manifolds ? CC_ERR_CAPACITY : CC_OK;
}

int cc_world_get_stats(cc_world *W, cc_stats *o) {
    if (!W || !o) return CC_ERR_INVALID;
    memset(o, 0, sizeof(*o));
    const DevCounters &c = W->last_ctr;
    o->num_bodies = W->w.n;
    o->num_awake = c.num_awake;
    o->num_pairs = c.num_pairs;
    o->num_manifolds = c.num_manifolds;
    o->num_contact_points = c.num_points;
    o->num_epa = c.num_epa;
    o->num_islands = c.num_islands;
    o->max_island_constraints = c.max_island_constraints;
    o->overflow_flags = c.overflow;
    o->gpu_launches_per_step = 0;
    if (W->graph) {  // kernel nodes of the captured step
        size_t nn = 0;
        cudaGraphGetNodes(W->graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(W->graph, nodes.data(), &nn);
        int k = 0;
        for (size_t i = 0; i < nn; i++) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
        }
        o->gpu_launches_per_step = k;
    }
    o->last_call_ms = W->last_call_ms;
    o->num_giant_islands = c.num_giant_islands;
    o->giant_colours = c.giant_colours;
    o->num_ccd = c.num_ccd;
    o->num_ccd_hits = c.num_ccd_hits;
    o->num_mesh_pairs = c.num_mesh_pairs;
    o->num_mesh_hits = c.num_mesh_hits;
    o->mesh_reduced = c.mesh_reduced;
    o->mesh_big = c.num_mesh_big;
    return CC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// rollout gradient
// ---------------------------------------------------------------------------
template <typename T>
static int adj_alloc(cc_world *W, T **p, size_t count) {
    int r = dalloc(p, count);
    if (r == CC_OK) W->adj.allocs.push_back((void *)*p);
    return r;
}

static int ensure_adjoint(cc_world *W, int seg_len, int n_ckpt) {
    auto &A = W->adj;
    if (A.seg_len >= seg_len && A.n_ckpt >= n_ckpt) return CC_OK;
    for (void *p : A.allocs) cudaFree(p);
    A = cc_world::Adjoint{};
    DevWorld &w = W->w;
    size_t cap = (size_t)w.cap, nm = (size_t)w.max_manifolds, cc = (size_t)w.cache_cap;
    int r;
#define AA(ptr, count)                                  \
    if ((r = adj_alloc(W, &(ptr), (count))) != CC_OK) { \
        return r;                                       \
    }
    A.tapes.resize(seg_len);
    A.tape_ratio.assign(seg_len, 0.f);
    for (auto &t : A.tapes) {
        AA(t.cons, nm);
        AA(t.valid, nm);
        AA(t.v, cap);
        AA(t.w, cap);
        AA(t.q, cap);
        AA(t.flags, cap);
        AA(t.isl_off, cap);
        AA(t.isl_cnt, cap);
        AA(t.isl_cons, nm);
        AA(t.counts, 2);
    }
    A.ckpts.resize(n_ckpt);
    A.ckpt_prev_dt.assign(n_ckpt, 0.0);
    for (auto &c : A.ckpts) {
        AA(c.pos, cap);
        AA(c.quat, cap);
        AA(c.com, cap);
        AA(c.linvel, cap);
        AA(c.angvel, cap);
        AA(c.force, cap);
        AA(c.torque, cap);
        AA(c.sleep_sph, 3 * cap);
        AA(c.sleep_timer, cap);
        AA(c.flags, cap);
        AA(c.keys, cc);
        AA(c.recs, cc);
        AA(c.parity, 1);
    }
    AdjBuffers &b = A.buf;
    AA(b.vbar, cap);
    AA(b.wbar, cap);
    AA(b.xbar, cap);
    AA(b.vwork, cap);
    AA(b.wwork, cap);
    AA(b.iw, 2 * cap);
    AA(b.u_tape, (size_t)W->settings.velocity_iterations * nm * 12);
    AA(b.lam_bar, nm * 12);
    AA(b.mu_con, nm);
    AA(b.mu_body, cap);
    for (int k = 0; k < 2; k++) {
        AA(A.hand[k].keys, cc);
        AA(A.hand[k].vals, cc * 12);
    }
    AA(A.sums, 4 * (size_t)w.num_worlds);
    AA(A.d_targets, 3 * (size_t)w.num_worlds);
    AA(A.d_loss, (size_t)w.num_worlds);
#undef AA
    A.seg_len = seg_len;
    A.n_ckpt = n_ckpt;
    return CC_OK;
}

static float warm_ratio(const cc_world *W, float dt) {
    if (!(dt > 0.f)) return 0.f;
    return (W->settings.warm_starting && W->prev_dt > 0) ? (float)(dt / W->prev_dt) : 0.f;
}

extern "C" int cc_world_rollout_grad(cc_world *W, float dt, int32_t n_steps, int32_t checkpoint_every,
                                     const float *targets, float *loss, float *grad_linvel, float *grad_angvel,
                                     float *grad_friction) {
    if (!W || !targets || n_steps <= 0 || checkpoint_every <= 0 || !(dt > 0.f)) return CC_ERR_INVALID;
    if (int r = sync_shapes(W)) return r;
    DevWorld &w = W->w;
    if (w.n == 0) return CC_ERR_INVALID;
    // the adjoint covers contacts and the discrete integration only
    if (w.num_hinges + w.num_swings + w.num_others + w.num_sixdofs > 0 || w.num_linear_cast > 0 || W->any_iter_override)
        return CC_ERR_UNSUPPORTED;
    int K = checkpoint_every < n_steps ? checkpoint_every : n_steps;
    int nseg = (n_steps + K - 1) / K;
    int r = ensure_adjoint(W, K, nseg + 1);
    if (r != CC_OK) return r;
    auto &A = W->adj;
    cudaStream_t s = W->stream;
    upload_settings(W->dev_settings, W->settings.speculative_contact_distance, s);
    if (!W->ev_begin) {
        CC_TRY(cudaEventCreate(&W->ev_begin));
        CC_TRY(cudaEventCreate(&W->ev_end));
    }
    CC_TRY(cudaEventRecord(W->ev_begin, s));
    // forward with a checkpoint at the start of every segment
    for (int t = 0; t < n_steps; t++) {
        if (t % K == 0) {
            checkpoint_save(w, A.ckpts[t / K], s);
            A.ckpt_prev_dt[t / K] = W->prev_dt;
        }
        enqueue_step(W, dt, warm_ratio(W, dt));
        W->prev_dt = dt;
    }
    checkpoint_save(w, A.ckpts[nseg], s);
    A.ckpt_prev_dt[nseg] = W->prev_dt;
    CC_TRY(cudaMemcpyAsync(A.d_targets, targets, sizeof(float) * 3 * w.num_worlds, cudaMemcpyHostToDevice, s));
    launch_rollout_loss(w, A.d_targets, A.sums, A.d_loss, A.buf, s);
    CC_TRY(cudaMemsetAsync(A.hand[0].keys, 0xff, sizeof(unsigned long long) * (size_t)w.cache_cap, s));
    int in = 0;
    // backward: recompute each segment with tapes, then reverse its steps
    for (int seg = nseg - 1; seg >= 0; seg--) {
        checkpoint_restore(w, A.ckpts[seg], s);
        W->prev_dt = A.ckpt_prev_dt[seg];
        int len = n_steps - seg * K < K ? n_steps - seg * K : K;
        for (int j = 0; j < len; j++) {
            A.tape_ratio[j] = warm_ratio(W, dt);
            enqueue_step(W, dt, A.tape_ratio[j], nullptr, &A.tapes[j]);
            W->prev_dt = dt;
        }
        for (int j = len - 1; j >= 0; j--) {
            launch_adjoint_step(w, A.tapes[j], A.buf, dt, A.tape_ratio[j], A.hand[in], A.hand[in ^ 1], s);
            in ^= 1;
        }
    }
    // the world ends where the forward rollout ended
    checkpoint_restore(w, A.ckpts[nseg], s);
    W->prev_dt = A.ckpt_prev_dt[nseg];
    W->steps_done += n_steps;
    CC_TRY(cudaEventRecord(W->ev_end, s));
    std::vector<float4> tmp((size_t)w.n);
    if (loss) CC_TRY(cudaMemcpyAsync(loss, A.d_loss, sizeof(float) * w.num_worlds, cudaMemcpyDeviceToHost, s));
    std::vector<unsigned long long> mu_fx;
    if (grad_friction) {
        mu_fx.resize((size_t)w.n);
        CC_TRY(cudaMemcpyAsync(mu_fx.data(), A.buf.mu_body, sizeof(unsigned long long) * w.n, cudaMemcpyDeviceToHost,
                               s));
    }
    for (int k = 0; k < 2; k++) {
        float *out = k == 0 ? grad_linvel : grad_angvel;
        if (!out) continue;
        CC_TRY(cudaMemcpyAsync(tmp.data(), k == 0 ? A.buf.vbar : A.buf.wbar, sizeof(float4) * w.n,
                               cudaMemcpyDeviceToHost, s));
        CC_TRY(cudaStreamSynchronize(s));
        for (int i = 0; i < w.n; i++) {
            out[3 * i] = tmp[i].x;
            out[3 * i + 1] = tmp[i].y;
            out[3 * i + 2] = tmp[i].z;
        }
    }
    CC_TRY(cudaStreamSynchronize(s));
    CC_TRY(cudaGetLastError());
    if (grad_friction)
        for (int i = 0; i < w.n; i++) grad_friction[i] = (float)((double)(long long)mu_fx[i] / ADJ_MU_SCALE);
    cudaEventElapsedTime(&W->last_call_ms, W->ev_begin, W->ev_end);
    W->last_ctr = *W->h_ctr;
    return CC_OK;
}

// ---------------------------------------------------------------------------
// launch-shape autotuner
// ---------------------------------------------------------------------------
struct TuneShape {
    int epa_blocks_per_sm, epa_lockstep, warp_blocks_per_sm, small_max, giant_min;
};
static TuneShape tune_shape_of(const cc_world *W) {
    const DevWorld &w = W->w;
    return TuneShape{w.epa_threads / 64 / device_sm_count(), w.epa_fetch_warp, w.warp_blocks_per_sm,
                     W->dev_settings.small_island_max_cons, w.giant_min};
}
static int tune_apply(cc_world *W, const TuneShape &t) {
    DevWorld &w = W->w;
    int blocks = t.epa_blocks_per_sm * device_sm_count();
    if (blocks > W->epa_packed_blocks) {
        if (w.epa_packed) cudaFree(w.epa_packed);
        w.epa_packed = nullptr;
        W->epa_packed_blocks = 0;
        char *q = nullptr;
        if (int r = dalloc(&q, epa_packed_block_bytes() * (size_t)blocks)) return r;
        w.epa_packed = q;
        W->epa_packed_blocks = blocks;
    }
    w.epa_threads = blocks * 64;
    w.epa_fetch_warp = t.epa_lockstep;
    w.warp_blocks_per_sm = t.warp_blocks_per_sm;
    W->dev_settings.small_island_max_cons = t.small_max;
    w.giant_min = t.giant_min;
    drop_graph(W);
    return CC_OK;
}
static int tune_snapshot(cc_world *W, bool save) {
    DevWorld &w = W->w;
    auto &T = W->tune;
    cudaStream_t s = W->stream;
    if (!T.ready) {
        size_t cap = (size_t)w.cap, cc = (size_t)w.cache_cap;
        int r;
#define TA(ptr, count)                                                \
    if ((r = dalloc(&(ptr), (count))) != CC_OK) return r;             \
    T.allocs.push_back((void *)(ptr));
        Checkpoint &c = T.c;
        TA(c.pos, cap) TA(c.quat, cap) TA(c.com, cap) TA(c.linvel, cap) TA(c.angvel, cap) TA(c.force, cap)
        TA(c.torque, cap) TA(c.sleep_sph, 3 * cap) TA(c.sleep_timer, cap) TA(c.flags, cap) TA(c.keys, cc)
        TA(c.recs, cc) TA(c.parity, 1)
        if (w.ccd_lambda) {
            TA(T.ccd, (size_t)w.num_worlds)
        }
#undef TA
        T.ready = true;
    }
    // joint records carry their accumulated impulses from step to step
    size_t jb = sizeof(DevHinge) * (size_t)w.num_hinges + sizeof(DevSwing) * (size_t)w.num_swings +
                sizeof(DevJoint) * (size_t)w.num_others + sizeof(DevSixDof) * (size_t)w.num_sixdofs;
    if (save && jb > T.joint_bytes) {
        if (T.joints) cudaFree(T.joints);
        T.joints = nullptr;
        T.joint_bytes = 0;
        if (int r = dalloc(&T.joints, jb)) return r;
        T.joint_bytes = jb;
    }
    if (save) {
        checkpoint_save(w, T.c, s);
    } else {
        checkpoint_restore(w, T.c, s);
    }
    size_t hb = sizeof(DevHinge) * (size_t)w.num_hinges, sb = sizeof(DevSwing) * (size_t)w.num_swings;
    if (hb) CC_TRY(cudaMemcpyAsync(save ? (void *)T.joints : (void *)w.hinges, save ? (void *)w.hinges : (void *)T.joints,
                                   hb, cudaMemcpyDeviceToDevice, s));
    if (sb)
        CC_TRY(cudaMemcpyAsync(save ? (void *)(T.joints + hb) : (void *)w.swings,
                               save ? (void *)w.swings : (void *)(T.joints + hb), sb, cudaMemcpyDeviceToDevice, s));
    size_t ob = sizeof(DevJoint) * (size_t)w.num_others;
    if (ob)
        CC_TRY(cudaMemcpyAsync(save ? (void *)(T.joints + hb + sb) : (void *)w.others,
                               save ? (void *)w.others : (void *)(T.joints + hb + sb), ob, cudaMemcpyDeviceToDevice, s));
    size_t xb = sizeof(DevSixDof) * (size_t)w.num_sixdofs;
    if (xb)
        CC_TRY(cudaMemcpyAsync(save ? (void *)(T.joints + hb + sb + ob) : (void *)w.sixdofs,
                               save ? (void *)w.sixdofs : (void *)(T.joints + hb + sb + ob), xb,
                               cudaMemcpyDeviceToDevice, s));
    if (w.ccd_lambda && T.ccd)
        CC_TRY(cudaMemcpyAsync(save ? (void *)T.ccd : (void *)w.ccd_lambda, save ? (void *)w.ccd_lambda : (void *)T.ccd,
                               sizeof(float2) * (size_t)w.num_worlds, cudaMemcpyDeviceToDevice, s));
    CC_TRY(cudaStreamSynchronize(s));
    return CC_OK;
}

extern "C" int cc_world_autotune(cc_world *W, float dt, int32_t steps, cc_tune_report *rep) {
    if (!W || !(dt > 0.f) || steps <= 0 || !rep) return CC_ERR_INVALID;
    if (int r = sync_shapes(W)) return r;
    DevWorld &w = W->w;
    memset(rep, 0, sizeof(*rep));
    if (w.n == 0) return CC_OK;
    const double prev_dt = W->prev_dt;
    const int steps_done = W->steps_done;
    if (int r = tune_snapshot(W, true)) return r;
    int trials = 0;
    auto trial = [&](float &ms) -> int {
        if (int r = tune_snapshot(W, false)) return r;
        W->prev_dt = prev_dt;
        int st = run_steps(W, dt, 1);
        if (st == CC_ERR_CUDA) return st;
        st = run_steps(W, dt, steps);
        if (st == CC_ERR_CUDA) return st;
        ms = W->last_call_ms / (float)steps;
        trials++;
        return CC_OK;
    };
    TuneShape cur = tune_shape_of(W);
    float best = 0.f;
    if (int r = trial(best)) return r;
    rep->default_ms = best;
    const bool piles = W->last_ctr.max_island_constraints > 2048;
    const int sms = device_sm_count();
    const int epa_cap = epa_max_threads() / 64 / sms;
    for (int dim = 0; dim < 5; dim++) {
        std::vector<int> cand;
        if (dim == 0) cand = {2, 4, 6, 8};
        if (dim == 1) cand = {1, 0};
        if (dim == 2) cand = {1, 2, 3, 4};
        if (dim == 3) cand = {4, 8, 16};
        if (dim == 4 && piles) cand = {2048, 8192, 32768};
        for (int v : cand) {
            TuneShape t = cur;
            int *field = dim == 0 ? &t.epa_blocks_per_sm
                                  : dim == 1 ? &t.epa_lockstep
                                  : dim == 2 ? &t.warp_blocks_per_sm : dim == 3 ? &t.small_max : &t.giant_min;
            if (*field == v) continue;
            if (dim == 0 && v > epa_cap) continue;
            *field = v;
            if (int r = tune_apply(W, t)) return r;
            float ms = 0.f;
            if (int r = trial(ms)) return r;
            if (ms < 0.98f * best) {
                best = ms;
                cur = t;
            }
        }
        if (int r = tune_apply(W, cur)) return r;
    }
    // keep the chosen shapes and leave the world where it was
    if (int r = tune_apply(W, cur)) return r;
    if (int r = tune_snapshot(W, false)) return r;
    W->prev_dt = prev_dt;
    W->steps_done = steps_done;
    rep->tuned_ms = best;
    rep->trials = trials;
    rep->epa_blocks_per_sm = cur.epa_blocks_per_sm;
    rep->epa_lockstep = cur.epa_lockstep;
    rep->warp_blocks_per_sm = cur.warp_blocks_per_sm;
    rep->small_island_max_contacts = cur.small_max;
    rep->giant_min = cur.giant_min;
    // kernel nodes of the step graph with the chosen shapes (captured by one more trial step)
    float ms = 0.f;
    if (int r = trial(ms)) return r;
    if (W->graph) {
        size_t nn = 0;
        cudaGraphGetNodes(W->graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(W->graph, nodes.data(), &nn);
        int k = 0;
        for (size_t i = 0; i < nn; i++) {
            cudaGraphNodeType ty;
            cudaGraphNodeGetType(nodes[i], &ty);
            k += ty == cudaGraphNodeTypeKernel;
        }
        rep->graph_kernels_per_step = k;
    }
    if (int r = tune_snapshot(W, false)) return r;
    W->prev_dt = prev_dt;
    W->steps_done = steps_done;
    drop_graph(W);
    return CC_OK;
}

// One step (the launch sequence cc_world_step runs) with the tape of its velocity solve read
// back in the C-ABI layout.
extern "C" int cc_world_step_taped(cc_world *W, float dt, cc_tape_body *bodies, cc_tape_contact *contacts,
                                   int32_t capacity, int32_t *count, float *warm_ratio_out) {
    if (!W || !count || capacity < 0 || !std::isfinite(dt)) return CC_ERR_INVALID;
    if (int r = sync_shapes(W)) return r;
    DevWorld &w = W->w;
    *count = 0;
    if (w.n == 0) return CC_OK;
    int r = ensure_adjoint(W, 1, 1);
    if (r != CC_OK) return r;
    if (W->x_cap_bodies < w.cap) {
        if (W->x_bodies) cudaFree(W->x_bodies);
        W->x_bodies = nullptr;
        W->x_cap_bodies = 0;
        CC_TRY(cudaMalloc(&W->x_bodies, sizeof(cc_tape_body) * (size_t)w.cap));
        W->x_cap_bodies = w.cap;
    }
    if (W->x_cap_cons < w.max_manifolds) {
        if (W->x_cons) cudaFree(W->x_cons);
        W->x_cons = nullptr;
        W->x_cap_cons = 0;
        CC_TRY(cudaMalloc(&W->x_cons, sizeof(cc_tape_contact) * (size_t)w.max_manifolds));
        W->x_cap_cons = w.max_manifolds;
    }
    cudaStream_t s = W->stream;
    upload_settings(W->dev_settings, W->settings.speculative_contact_distance, s);
    if (!W->ev_begin) {
        CC_TRY(cudaEventCreate(&W->ev_begin));
        CC_TRY(cudaEventCreate(&W->ev_end));
    }
    float ratio = (W->settings.warm_starting && W->prev_dt > 0) ? (float)(dt / W->prev_dt) : 0.f;
    if (dt <= 0.f) ratio = 0.f;
    TapeStep &t = W->adj.tapes[0];
    CC_TRY(cudaEventRecord(W->ev_begin, s));
    enqueue_step(W, dt, ratio, nullptr, &t);
    CC_TRY(cudaEventRecord(W->ev_end, s));
    launch_tape_export(w, t, W->x_bodies, W->x_cons, s);
    if (dt > 0.f) W->prev_dt = dt;
    W->steps_done++;
    CC_TRY(cudaStreamSynchronize(s));
    CC_TRY(cudaGetLastError());
    cudaEventElapsedTime(&W->last_call_ms, W->ev_begin, W->ev_end);
    W->last_ctr = *W->h_ctr;
    int status = CC_OK;
    if (W->last_ctr.overflow) status = (W->last_ctr.overflow & OVF_TIMEOUT) ? CC_ERR_TIMEOUT : CC_ERR_CAPACITY;
    W->last_status = status;
    if (warm_ratio_out) *warm_ratio_out = ratio;
    if (bodies) CC_TRY(cudaMemcpy(bodies, W->x_bodies, sizeof(cc_tape_body) * (size_t)w.n, cudaMemcpyDeviceToHost));
    int nm = W->last_ctr.num_manifolds < w.max_manifolds ? W->last_ctr.num_manifolds : w.max_manifolds;
    std::vector<cc_tape_contact> all((size_t)nm);
    if (nm > 0) CC_TRY(cudaMemcpy(all.data(), W->x_cons, sizeof(cc_tape_contact) * (size_t)nm, cudaMemcpyDeviceToHost));
    int k = 0;
    for (int i = 0; i < nm; i++) k += all[i].body_a >= 0;
    *count = k;
    if (!contacts) return status;
    if (k > capacity) return CC_ERR_CAPACITY;
    k = 0;
    for (int i = 0; i < nm; i++)
        if (all[i].body_a >= 0) contacts[k++] = all[i];
    return status;
}

// ---------------------------------------------------------------------------
// hinge joints: creation in FP64 from the bodies' current poses
// (hingeConstraint.create hinge-constraint.ts:240-387) and the setters
// ---------------------------------------------------------------------------

// grow the joint arrays of one type and the per-island joint lists (created on first use)
template <typename T>
static int grow_joints(cc_world *W, T *&arr, int count, int &cap_io, int need) {
    if (need <= cap_io) return CC_OK;
    int cap = std::max(need, std::max(64, 2 * cap_io));
    T *na = nullptr;
    int r;
    if ((r = dalloc(&na, cap)) != CC_OK) return r;
    CC_TRY(cudaStreamSynchronize(W->stream));
    if (count > 0) CC_TRY(cudaMemcpy(na, arr, sizeof(T) * count, cudaMemcpyDeviceToDevice));
    if (arr) cudaFree(arr);
    arr = na;
    cap_io = cap;
    return CC_OK;
}
static int ensure_joint_capacity(cc_world *W, int need_hinges, int need_swings, int need_others = -1,
                                 int need_sixdofs = -1) {
    DevWorld &w = W->w;
    int r;
    if (!w.island_joint_count) {
        if ((r = dalloc(&w.island_joint_count, w.cap)) != CC_OK || (r = dalloc(&w.island_joint_off, w.cap)) != CC_OK ||
            (r = dalloc(&w.island_fill_j, w.cap)) != CC_OK || (r = dalloc(&w.joint_wake, 1)) != CC_OK ||
            (r = dalloc(&w.small_joint_list, w.cap)) != CC_OK || (r = dalloc(&w.large_joint_list, w.cap)) != CC_OK ||
            (r = dalloc(&w.joint_partners, (size_t)w.cap * JOINT_PARTNERS)) != CC_OK)
            return r;
        CC_TRY(cudaMemset(w.joint_partners, 0xff, sizeof(int) * (size_t)w.cap * JOINT_PARTNERS));
    }
    if ((r = grow_joints(W, w.hinges, w.num_hinges, w.max_hinges, need_hinges)) != CC_OK) return r;
    if ((r = grow_joints(W, w.swings, w.num_swings, w.max_swings, need_swings)) != CC_OK) return r;
    if (need_others >= 0 && (r = grow_joints(W, w.others, w.num_others, w.max_others, need_others)) != CC_OK) return r;
    if (need_sixdofs >= 0 &&
        (r = grow_joints(W, w.sixdofs, w.num_sixdofs, w.max_sixdofs, need_sixdofs)) != CC_OK)
        return r;
    int need_lists = w.max_hinges + w.max_swings + w.max_others + w.max_sixdofs;
    if (need_lists > w.max_joints) {
        int *nl = nullptr;
        if ((r = dalloc(&nl, 5 * (size_t)need_lists)) != CC_OK) return r;
        CC_TRY(cudaStreamSynchronize(W->stream));
        if (w.island_joints) cudaFree(w.island_joints);
        w.island_joints = nl;
        w.max_joints = need_lists;
    }
    drop_graph(W);
    return CC_OK;
}

// partner lists of the broadphase joint-pair filter, from the enabled joints
static int upload_partners(cc_world *W) {
    DevWorld &w = W->w;
    if (!w.joint_partners) return CC_OK;
    std::vector<int> part((size_t)w.cap * JOINT_PARTNERS, -1);
    bool over = false;
    auto add = [&](int a, int b) {
        int *p = part.data() + (size_t)a * JOINT_PARTNERS;
        for (int k = 0; k < JOINT_PARTNERS; k++) {
            if (p[k] == b) return;
            if (p[k] < 0) {
                p[k] = b;
                return;
            }
        }
        over = true;
    };
    auto add_joint = [&](const DevJointHead &h) {
        if (!(h.flags & JF_ENABLED)) return;
        add(h.a, h.b);
        add(h.b, h.a);
    };
    for (const DevHinge &j : W->hinges) add_joint(j.h);
    for (const DevSwing &j : W->swings) add_joint(j.h);
    for (const DevJoint &j : W->others) add_joint(j.h);
    for (const DevSixDof &j : W->sixdofs) add_joint(j.h);
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaMemcpy(w.joint_partners, part.data(), sizeof(int) * part.size(), cudaMemcpyHostToDevice));
    return over && w.skip_joint_pairs ? CC_ERR_CAPACITY : CC_OK;
}

extern "C" {

int cc_world_add_hinges(cc_world *W, const cc_hinge_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++) {
        const cc_hinge_desc &h = d[i];
        if (h.body_a < 0 || h.body_b < 0 || h.body_a >= w.n || h.body_b >= w.n) return CC_ERR_INVALID;
        if (h.space != CC_SPACE_WORLD && h.space != CC_SPACE_LOCAL) return CC_ERR_INVALID;
        if (h.motor_state < 0 || h.motor_state > 2) return CC_ERR_INVALID;
        if (!spring_ok(h.limits_spring) || !spring_ok(h.motor_spring)) return CC_ERR_INVALID;
        if (!finite3(h.point_a) || !finite3(h.point_b) || !finite3(h.hinge_axis_a) || !finite3(h.hinge_axis_b) ||
            !finite3(h.normal_axis_a) || !finite3(h.normal_axis_b))
            return CC_ERR_INVALID;
        if (std::isnan(h.limits_min) || std::isnan(h.limits_max) || std::isnan(h.max_friction_torque) ||
            std::isnan(h.min_torque_limit) || std::isnan(h.max_torque_limit) ||
            !std::isfinite(h.target_angular_velocity) || !std::isfinite(h.target_angle))
            return CC_ERR_INVALID;
    }
    // current poses and worlds of the bodies
    std::vector<float4> quat((size_t)w.n), com((size_t)w.n);
    std::vector<int> world((size_t)w.n);
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaMemcpy(quat.data(), w.quat, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(com.data(), w.com, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(world.data(), w.world, sizeof(int) * w.n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++)
        if (world[d[i].body_a] != world[d[i].body_b]) return CC_ERR_INVALID;
    std::vector<DevHinge> made((size_t)n);
    const double PI = 3.14159265358979323846;
    for (int i = 0; i < n; i++) {
        const cc_hinge_desc &h = d[i];
        DevHinge j;
        memset(&j, 0, sizeof(j));
        j.h.a = h.body_a;
        j.h.b = h.body_b;
        j.h.index = w.num_hinges + i;
        if (h.num_velocity_steps_override < 0 || h.num_velocity_steps_override > 255 ||
            h.num_position_steps_override < 0 || h.num_position_steps_override > 255)
            return CC_ERR_INVALID;
        j.h.iter_ovr = (int)((uint32_t)h.num_velocity_steps_override | ((uint32_t)h.num_position_steps_override << 8));
        if (j.h.iter_ovr) W->any_iter_override = true;
        j.h.priority = h.priority;
        j.h.island = -1;
        DQ qa = dq(quat[j.h.a]), qb = dq(quat[j.h.b]);
        D3 h1 = dnormalize(d3(h.hinge_axis_a)), h2 = dnormalize(d3(h.hinge_axis_b));
        D3 n1 = dnormalize(d3(h.normal_axis_a)), n2 = dnormalize(d3(h.normal_axis_b));
        DQ inv_initial;
        if (h.space == CC_SPACE_WORLD) {
            DQ iqa = dconj(qa), iqb = dconj(qb);
            j.lp1 = f3d(drot(iqa, dsub(d3(h.point_a), d3(com[j.h.a]))));
            j.lp2 = f3d(drot(iqb, dsub(d3(h.point_b), d3(com[j.h.b]))));
            j.lh1 = f3d(drot(iqa, h1));
            j.lh2 = f3d(drot(iqb, h2));
            DQ r0 = inv_initial_orientation_xz(n1, h1, n2, h2);
            inv_initial = dqmul(dqmul(iqb, r0), qa);
        } else {
            j.lp1 = f3d(d3(h.point_a));
            j.lp2 = f3d(d3(h.point_b));
            j.lh1 = f3d(h1);
            j.lh2 = f3d(h2);
            inv_initial = inv_initial_orientation_xz(drot(qa, n1), drot(qa, h1), drot(qb, n2), drot(qb, h2));
        }
        j.inv_initial = make_float4((float)inv_initial.x, (float)inv_initial.y, (float)inv_initial.z,
                                    (float)inv_initial.w);
        double mn = h.limits_min, mx = h.limits_max;
        bool has_limits = !(mn <= -PI && mx >= PI);
        j.limits_min = has_limits ? (float)std::max(mn, -PI) : (float)-PI;
        j.limits_max = has_limits ? (float)std::min(mx, PI) : (float)PI;
        j.h.flags = (h.enabled ? JF_ENABLED : 0) | (has_limits ? JF_LIMITS : 0);
        j.limits_spring_mode = h.limits_spring.mode;
        j.limits_freq = h.limits_spring.frequency_or_stiffness;
        j.limits_damping = h.limits_spring.damping;
        j.max_friction_torque = h.max_friction_torque;
        j.motor_state = h.motor_state;
        j.target_angular_velocity = h.target_angular_velocity;
        double ta = h.target_angle;
        j.target_angle = has_limits ? (float)std::max((double)j.limits_min, std::min((double)j.limits_max, ta)) : (float)ta;
        j.motor_spring_mode = h.motor_spring.mode;
        j.motor_freq = h.motor_spring.frequency_or_stiffness;
        j.motor_damping = h.motor_spring.damping;
        j.min_torque = h.min_torque_limit;
        j.max_torque = h.max_torque_limit;
        made[i] = j;
    }
    int r = ensure_joint_capacity(W, w.num_hinges + n, w.num_swings);
    if (r != CC_OK) return r;
    CC_TRY(cudaMemcpy(w.hinges + w.num_hinges, made.data(), sizeof(DevHinge) * n, cudaMemcpyHostToDevice));
    for (int i = 0; i < n; i++) {
        W->hinges.push_back(made[i]);
        if (out_index) out_index[i] = w.num_hinges + i;
    }
    w.num_hinges += n;
    w.type_count[JT_HINGE] = w.num_hinges;
    drop_graph(W);
    return upload_partners(W);
}

}  // extern "C"

// read-modify-write of one joint's device record (the host copy follows)
template <typename T, typename F>
static int edit_joint(cc_world *W, T *dev, std::vector<T> &host, int count, int32_t index, F f) {
    if (index < 0 || index >= count) return CC_ERR_INVALID;
    T j;
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaMemcpy(&j, dev + index, sizeof(T), cudaMemcpyDeviceToHost));
    f(j);
    f(host[index]);
    CC_TRY(cudaMemcpy(dev + index, &j, sizeof(T), cudaMemcpyHostToDevice));
    return CC_OK;
}
template <typename F>
static int edit_hinge(cc_world *W, int32_t index, F f) {
    return edit_joint(W, W->w.hinges, W->hinges, W->w.num_hinges, index, f);
}
template <typename F>
static int edit_swing(cc_world *W, int32_t index, F f) {
    return edit_joint(W, W->w.swings, W->swings, W->w.num_swings, index, f);
}

// SwingTwistConstraintPart.setLimits (swing-twist-constraint-part.ts:140-236) in FP64: a limit
// inside +-0.5 degrees locks its axis, one beyond +-179.5 degrees frees it
template <class P>
static void st_set_limits(P &p, double twist_min, double twist_max, double ymin, double ymax, double zmin,
                          double zmax) {
    const double PI = 3.14159265358979323846;
    const double locked = 0.5 * PI / 180.0, free_a = 179.5 * PI / 180.0;
    p.y_half_min = (float)(0.5 * ymin);
    p.y_half_max = (float)(0.5 * ymax);
    p.z_half_min = (float)(0.5 * zmin);
    p.z_half_max = (float)(0.5 * zmax);
    p.rotation_flags = 0;
    auto axis = [&](double mn, double mx, int lock_flag, int free_flag, float &smin, float &smax, float &cmin,
                    float &cmax) {
        if (mn > -locked && mx < locked) {
            p.rotation_flags |= lock_flag;
            smin = smax = 0.f;
            cmin = cmax = 1.f;
        } else if (mn < -free_a && mx > free_a) {
            p.rotation_flags |= free_flag;
            smin = -1.f;
            smax = 1.f;
            cmin = cmax = 0.f;
        } else {
            smin = (float)std::sin(0.5 * mn);
            smax = (float)std::sin(0.5 * mx);
            cmin = (float)std::cos(0.5 * mn);
            cmax = (float)std::cos(0.5 * mx);
        }
    };
    axis(twist_min, twist_max, ST_TWIST_LOCKED, ST_TWIST_FREE, p.sin_twist_min, p.sin_twist_max, p.cos_twist_min,
         p.cos_twist_max);
    axis(ymin, ymax, ST_SWING_Y_LOCKED, ST_SWING_Y_FREE, p.sin_y_min, p.sin_y_max, p.cos_y_min, p.cos_y_max);
    axis(zmin, zmax, ST_SWING_Z_LOCKED, ST_SWING_Z_FREE, p.sin_z_min, p.sin_z_max, p.cos_z_min, p.cos_z_max);
}
// the swing-twist constraint's limits: twist [min, max], swing Y +-plane, swing Z +-normal half cone
static void swing_set_limits(DevSwing &p) {
    st_set_limits(p, p.twist_min, p.twist_max, -(double)p.plane_half_cone, (double)p.plane_half_cone,
                  -(double)p.normal_half_cone, (double)p.normal_half_cone);
}
// setTargetOrientationCS (swing-twist-constraint.ts:405-416): the target clamped into the limits
static void swing_set_target(DevSwing &p, const float *q) {
    float4 o = make_float4(q[0], q[1], q[2], q[3]), sw, tw;
    get_swing_twist(o, sw, tw);
    p.target_q = clamp_swing_twist(p, sw, tw) != 0 ? qmul(sw, tw) : o;
}

extern "C" {

int cc_world_set_hinge_limits(cc_world *W, int32_t index, float limits_min, float limits_max) {
    if (!W || std::isnan(limits_min) || std::isnan(limits_max)) return CC_ERR_INVALID;
    const double PI = 3.14159265358979323846;
    return edit_hinge(W, index, [&](DevHinge &j) {  // setLimits hinge-constraint.ts:429-439
        double mn = std::max((double)limits_min, -PI), mx = std::min((double)limits_max, PI);
        j.limits_min = (float)mn;
        j.limits_max = (float)mx;
        bool has = mn > -PI || mx < PI;
        j.h.flags = has ? (j.h.flags | JF_LIMITS) : (j.h.flags & ~JF_LIMITS);
        if (has) j.target_angle = (float)std::max(mn, std::min(mx, (double)j.target_angle));
    });
}

int cc_world_set_hinge_motor(cc_world *W, int32_t index, int32_t motor_state, float target_angular_velocity,
                             float target_angle) {
    if (!W || motor_state < 0 || motor_state > 2 || !std::isfinite(target_angular_velocity) ||
        !std::isfinite(target_angle))
        return CC_ERR_INVALID;
    return edit_hinge(W, index, [&](DevHinge &j) {  // hinge-constraint.ts:441-465
        j.motor_state = motor_state;
        j.target_angular_velocity = target_angular_velocity;
        j.target_angle = (j.h.flags & JF_LIMITS)
                             ? (float)std::max((double)j.limits_min, std::min((double)j.limits_max, (double)target_angle))
                             : target_angle;
    });
}

int cc_world_set_hinge_enabled(cc_world *W, int32_t index, int32_t enabled) {
    if (!W) return CC_ERR_INVALID;
    int r = edit_hinge(W, index,
                       [&](DevHinge &j) { j.h.flags = enabled ? (j.h.flags | JF_ENABLED) : (j.h.flags & ~JF_ENABLED); });
    if (r != CC_OK) return r;
    return upload_partners(W);
}

int cc_world_get_hinge_angles(cc_world *W, float *out, int32_t capacity) {
    if (!W || capacity < 0 || (capacity > 0 && !out)) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    int n = std::min(capacity, w.num_hinges);
    if (n == 0) return capacity < w.num_hinges ? CC_ERR_CAPACITY : CC_OK;
    CC_TRY(cudaMemcpy2DAsync(out, sizeof(float), (const char *)w.hinges + offsetof(DevHinge, theta), sizeof(DevHinge),
                             sizeof(float), n, cudaMemcpyDeviceToHost, W->stream));
    CC_TRY(cudaStreamSynchronize(W->stream));
    return capacity < w.num_hinges ? CC_ERR_CAPACITY : CC_OK;
}

int cc_world_add_swing_twists(cc_world *W, const cc_swing_twist_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++) {
        const cc_swing_twist_desc &h = d[i];
        if (h.body_a < 0 || h.body_b < 0 || h.body_a >= w.n || h.body_b >= w.n) return CC_ERR_INVALID;
        if (h.space != CC_SPACE_WORLD && h.space != CC_SPACE_LOCAL) return CC_ERR_INVALID;
        if (h.swing_type != CC_SWING_CONE && h.swing_type != CC_SWING_PYRAMID) return CC_ERR_INVALID;
        if (h.swing_motor_state < 0 || h.swing_motor_state > 2 || h.twist_motor_state < 0 || h.twist_motor_state > 2)
            return CC_ERR_INVALID;
        if (!spring_ok(h.swing_motor_spring) || !spring_ok(h.twist_motor_spring)) return CC_ERR_INVALID;
        if (!finite3(h.position_a) || !finite3(h.position_b) || !finite3(h.twist_axis_a) || !finite3(h.plane_axis_a) ||
            !finite3(h.twist_axis_b) || !finite3(h.plane_axis_b) || !finite3(h.target_angular_velocity))
            return CC_ERR_INVALID;
        if (!std::isfinite(h.normal_half_cone_angle) || !std::isfinite(h.plane_half_cone_angle) ||
            !std::isfinite(h.twist_min_angle) || !std::isfinite(h.twist_max_angle) || std::isnan(h.max_friction_torque))
            return CC_ERR_INVALID;
        for (int k = 0; k < 4; k++)
            if (!std::isfinite(h.target_orientation[k])) return CC_ERR_INVALID;
    }
    std::vector<float4> quat((size_t)w.n), com((size_t)w.n);
    std::vector<int> world((size_t)w.n);
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaMemcpy(quat.data(), w.quat, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(com.data(), w.com, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(world.data(), w.world, sizeof(int) * w.n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++)
        if (world[d[i].body_a] != world[d[i].body_b]) return CC_ERR_INVALID;
    std::vector<DevSwing> made((size_t)n);
    for (int i = 0; i < n; i++) {
        const cc_swing_twist_desc &h = d[i];
        DevSwing j;
        memset(&j, 0, sizeof(j));
        j.h.a = h.body_a;
        j.h.b = h.body_b;
        j.h.index = w.num_swings + i;
        if (h.num_velocity_steps_override < 0 || h.num_velocity_steps_override > 255 ||
            h.num_position_steps_override < 0 || h.num_position_steps_override > 255)
            return CC_ERR_INVALID;
        j.h.iter_ovr = (int)((uint32_t)h.num_velocity_steps_override | ((uint32_t)h.num_position_steps_override << 8));
        if (j.h.iter_ovr) W->any_iter_override = true;
        j.h.priority = h.priority;
        j.h.island = -1;
        j.h.flags = h.enabled ? JF_ENABLED : 0;
        // constraint space: X twist, Y normal = plane x twist, Z plane (create :218-260)
        D3 t1 = dnormalize(d3(h.twist_axis_a)), p1 = dnormalize(d3(h.plane_axis_a));
        D3 t2 = dnormalize(d3(h.twist_axis_b)), p2 = dnormalize(d3(h.plane_axis_b));
        DQ c1 = quat_from_columns(t1, dcross(p1, t1), p1), c2 = quat_from_columns(t2, dcross(p2, t2), p2);
        if (h.space == CC_SPACE_WORLD) {
            DQ iqa = dconj(dq(quat[j.h.a])), iqb = dconj(dq(quat[j.h.b]));
            j.lp1 = f3d(drot(iqa, dsub(d3(h.position_a), d3(com[j.h.a]))));
            j.lp2 = f3d(drot(iqb, dsub(d3(h.position_b), d3(com[j.h.b]))));
            c1 = dqmul(iqa, c1);
            c2 = dqmul(iqb, c2);
        } else {
            j.lp1 = f3d(d3(h.position_a));
            j.lp2 = f3d(d3(h.position_b));
        }
        j.c2b1 = make_float4((float)c1.x, (float)c1.y, (float)c1.z, (float)c1.w);
        j.c2b2 = make_float4((float)c2.x, (float)c2.y, (float)c2.z, (float)c2.w);
        j.swing_type = h.swing_type;
        j.normal_half_cone = h.normal_half_cone_angle;
        j.plane_half_cone = h.plane_half_cone_angle;
        j.twist_min = h.twist_min_angle;
        j.twist_max = h.twist_max_angle;
        swing_set_limits(j);
        j.max_friction_torque = h.max_friction_torque;
        j.swing_motor_state = h.swing_motor_state;
        j.twist_motor_state = h.twist_motor_state;
        j.target_w = make_float3(h.target_angular_velocity[0], h.target_angular_velocity[1], h.target_angular_velocity[2]);
        swing_set_target(j, h.target_orientation);
        j.swing_spring_mode = h.swing_motor_spring.mode;
        j.swing_freq = h.swing_motor_spring.frequency_or_stiffness;
        j.swing_damping = h.swing_motor_spring.damping;
        j.twist_spring_mode = h.twist_motor_spring.mode;
        j.twist_freq = h.twist_motor_spring.frequency_or_stiffness;
        j.twist_damping = h.twist_motor_spring.damping;
        j.swing_min_torque = h.swing_min_torque_limit;
        j.swing_max_torque = h.swing_max_torque_limit;
        j.twist_min_torque = h.twist_min_torque_limit;
        j.twist_max_torque = h.twist_max_torque_limit;
        made[i] = j;
    }
    int r = ensure_joint_capacity(W, w.num_hinges, w.num_swings + n);
    if (r != CC_OK) return r;
    CC_TRY(cudaMemcpy(w.swings + w.num_swings, made.data(), sizeof(DevSwing) * n, cudaMemcpyHostToDevice));
    for (int i = 0; i < n; i++) {
        W->swings.push_back(made[i]);
        if (out_index) out_index[i] = w.num_swings + i;
    }
    w.num_swings += n;
    w.type_count[JT_SWING] = w.num_swings;
    drop_graph(W);
    return upload_partners(W);
}

int cc_world_set_swing_twist_limits(cc_world *W, int32_t index, float normal_half_cone_angle,
                                    float plane_half_cone_angle, float twist_min_angle, float twist_max_angle) {
    if (!W || !std::isfinite(normal_half_cone_angle) || !std::isfinite(plane_half_cone_angle) ||
        !std::isfinite(twist_min_angle) || !std::isfinite(twist_max_angle))
        return CC_ERR_INVALID;
    return edit_swing(W, index, [&](DevSwing &j) {  // setNormalHalfConeAngle ... setTwistMaxAngle :319-341
        j.normal_half_cone = normal_half_cone_angle;
        j.plane_half_cone = plane_half_cone_angle;
        j.twist_min = twist_min_angle;
        j.twist_max = twist_max_angle;
        swing_set_limits(j);
    });
}

int cc_world_set_swing_twist_motor(cc_world *W, int32_t index, int32_t swing_motor_state, int32_t twist_motor_state,
                                   const float *target_angular_velocity, const float *target_orientation,
                                   float max_friction_torque) {
    if (!W || swing_motor_state < 0 || swing_motor_state > 2 || twist_motor_state < 0 || twist_motor_state > 2 ||
        !target_angular_velocity || !target_orientation || !finite3(target_angular_velocity) ||
        std::isnan(max_friction_torque))
        return CC_ERR_INVALID;
    for (int k = 0; k < 4; k++)
        if (!std::isfinite(target_orientation[k])) return CC_ERR_INVALID;
    return edit_swing(W, index, [&](DevSwing &j) {  // :343-416
        if (j.swing_motor_state != swing_motor_state) {  // setSwingMotorState resets all three motor parts
            j.swing_motor_state = swing_motor_state;
            for (int k = 0; k < 3; k++) j.motor[k].eff = j.motor[k].lambda = 0.f;
        }
        if (j.twist_motor_state != twist_motor_state) {  // setTwistMotorState resets the twist part
            j.twist_motor_state = twist_motor_state;
            j.motor[0].eff = j.motor[0].lambda = 0.f;
        }
        j.target_w = make_float3(target_angular_velocity[0], target_angular_velocity[1], target_angular_velocity[2]);
        swing_set_target(j, target_orientation);
        j.max_friction_torque = max_friction_torque;
    });
}

int cc_world_set_swing_twist_enabled(cc_world *W, int32_t index, int32_t enabled) {
    if (!W) return CC_ERR_INVALID;
    int r = edit_swing(W, index,
                       [&](DevSwing &j) { j.h.flags = enabled ? (j.h.flags | JF_ENABLED) : (j.h.flags & ~JF_ENABLED); });
    if (r != CC_OK) return r;
    return upload_partners(W);
}

int cc_world_set_skip_joint_pairs(cc_world *W, int32_t on) {
    if (!W) return CC_ERR_INVALID;
    W->w.skip_joint_pairs = on ? 1 : 0;
    int r = ensure_joint_capacity(W, 0, 0);
    if (r != CC_OK) return r;
    drop_graph(W);
    return upload_partners(W);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// convex hull shapes (convexHull.create convex-hull.ts:106-446)
// ---------------------------------------------------------------------------
// every hull's arrays, concatenated and uploaded again whenever a hull is added
static int upload_hulls(cc_world *W) {
    DevWorld &w = W->w;
    std::vector<DevHull> hdr;
    std::vector<float4> pts, shr, pln;
    std::vector<int2> faces;
    std::vector<int> vidx;
    for (const cc_hull::Hull &h : W->hulls) {
        DevHull d;
        memset(&d, 0, sizeof(d));
        d.first_point = (int)pts.size();
        d.num_points = (int)h.points.size();
        d.first_face = (int)faces.size();
        d.num_faces = (int)h.face_first.size();
        d.convex_radius = (float)h.convex_radius;
        d.inner_radius = (float)h.inner_radius;
        d.com = make_float4((float)h.com.x, (float)h.com.y, (float)h.com.z, 0.f);
        d.lo = make_float4((float)h.lo.x, (float)h.lo.y, (float)h.lo.z, 0.f);
        d.hi = make_float4((float)h.hi.x, (float)h.hi.y, (float)h.hi.z, 0.f);
        int vbase = (int)vidx.size();
        for (size_t k = 0; k < h.points.size(); k++) {
            pts.push_back(make_float4((float)h.points[k].x, (float)h.points[k].y, (float)h.points[k].z, 0.f));
            shr.push_back(make_float4((float)h.shrunk[k].x, (float)h.shrunk[k].y, (float)h.shrunk[k].z, 0.f));
        }
        for (size_t f = 0; f < h.face_first.size(); f++) {
            faces.push_back(make_int2(vbase + h.face_first[f], h.face_count[f]));
            pln.push_back(make_float4((float)h.plane_n[f].x, (float)h.plane_n[f].y, (float)h.plane_n[f].z,
                                      (float)h.plane_c[f]));
        }
        for (int v : h.vidx) vidx.push_back(d.first_point + v);
        hdr.push_back(d);
    }
    CC_TRY(cudaStreamSynchronize(W->stream));
    void *old[] = {w.hulls, w.hull_points, w.hull_shrunk, w.hull_planes, w.hull_faces, w.hull_vidx};
    for (void *p : old)
        if (p) cudaFree(p);
    w.hulls = nullptr;
    w.hull_points = w.hull_shrunk = w.hull_planes = nullptr;
    w.hull_faces = nullptr;
    w.hull_vidx = nullptr;
    int r;
    if ((r = dalloc(&w.hulls, hdr.size())) != CC_OK || (r = dalloc(&w.hull_points, pts.size())) != CC_OK ||
        (r = dalloc(&w.hull_shrunk, shr.size())) != CC_OK || (r = dalloc(&w.hull_planes, pln.size())) != CC_OK ||
        (r = dalloc(&w.hull_faces, faces.size())) != CC_OK || (r = dalloc(&w.hull_vidx, vidx.size())) != CC_OK)
        return r;
    CC_TRY(cudaMemcpy(w.hulls, hdr.data(), sizeof(DevHull) * hdr.size(), cudaMemcpyHostToDevice));
    CC_TRY(cudaMemcpy(w.hull_points, pts.data(), sizeof(float4) * pts.size(), cudaMemcpyHostToDevice));
    CC_TRY(cudaMemcpy(w.hull_shrunk, shr.data(), sizeof(float4) * shr.size(), cudaMemcpyHostToDevice));
    CC_TRY(cudaMemcpy(w.hull_planes, pln.data(), sizeof(float4) * pln.size(), cudaMemcpyHostToDevice));
    CC_TRY(cudaMemcpy(w.hull_faces, faces.data(), sizeof(int2) * faces.size(), cudaMemcpyHostToDevice));
    CC_TRY(cudaMemcpy(w.hull_vidx, vidx.data(), sizeof(int) * vidx.size(), cudaMemcpyHostToDevice));
    w.num_hulls = (int)hdr.size();
    drop_graph(W);
    return CC_OK;
}

extern "C" {

}  // extern "C"
// ---------------------------------------------------------------------------
// triangle meshes (triangleMesh.create triangle-mesh.ts:114-140)
// ---------------------------------------------------------------------------
static int build_mesh_from(const double *positions, int32_t nv, const int32_t *indices, int32_t nt, double degenerate,
                           double active_cos, cc_mesh::Mesh &m) {
    if (!positions || !indices || nv < 0 || nt < 0) return CC_ERR_INVALID;
    for (int i = 0; i < 3 * nt; i++)
        if (indices[i] < 0 || indices[i] >= nv) return CC_ERR_INVALID;
    std::vector<double> p((size_t)3 * nv);
    for (size_t i = 0; i < p.size(); i++) {
        p[i] = positions[i];
        if (!std::isfinite(p[i])) return CC_ERR_INVALID;
    }
    cc_mesh::BuildSettings bs;
    if (degenerate >= 0.0) bs.degenerate_tolerance = degenerate;
    if (active_cos >= -1.0) bs.active_edge_cos = active_cos;
    m = cc_mesh::build(p.data(), nv, indices, nt, nullptr, bs);
    if ((int)m.active.size() >= (1 << MESH_KEY_BITS)) return CC_ERR_UNSUPPORTED;
    return CC_OK;
}

// every mesh's arrays, concatenated and uploaded again whenever a mesh is added
static int upload_meshes(cc_world *W) {
    DevWorld &w = W->w;
    std::vector<DevMesh> hdr;
    std::vector<float4> verts, nodes;
    std::vector<int4> tris;
    for (const cc_mesh::Mesh &m : W->meshes) {
        DevMesh d;
        memset(&d, 0, sizeof(d));
        d.first_vertex = (int)verts.size();
        d.first_tri = (int)tris.size();
        d.first_node = (int)(nodes.size() / 2);
        d.num_tris = (int)m.active.size();
        unsigned maxi = d.num_tris > 0 ? (unsigned)(d.num_tris - 1) : 0u;
        d.sub_bits = maxi == 0 ? 0 : 32 - __builtin_clz(maxi);
        d.lo = make_float4((float)m.lo[0], (float)m.lo[1], (float)m.lo[2], 0.f);
        d.hi = make_float4((float)m.hi[0], (float)m.hi[1], (float)m.hi[2], 0.f);
        for (size_t k = 0; k < m.positions.size() / 3; k++)
            verts.push_back(make_float4((float)m.positions[3 * k], (float)m.positions[3 * k + 1],
                                        (float)m.positions[3 * k + 2], 0.f));
        for (int t = 0; t < d.num_tris; t++)
            tris.push_back(make_int4(d.first_vertex + m.tris[3 * t], d.first_vertex + m.tris[3 * t + 1],
                                     d.first_vertex + m.tris[3 * t + 2], m.active[t]));
        for (size_t k = 0; k < m.nodes.size() / 8; k++) {
            const double *nd = &m.nodes[8 * k];
            int a = (int)nd[6], b = (int)nd[7];
            if (b >= 0) a /= 8;  // internal node: the right child's offset in doubles, as a node index
            float fa, fb;
            memcpy(&fa, &a, sizeof(float));
            memcpy(&fb, &b, sizeof(float));
            nodes.push_back(make_float4((float)nd[0], (float)nd[1], (float)nd[2], fa));
            nodes.push_back(make_float4((float)nd[3], (float)nd[4], (float)nd[5], fb));
        }
        hdr.push_back(d);
    }
    CC_TRY(cudaStreamSynchronize(W->stream));
    void *old[] = {w.meshes, w.mesh_verts, w.mesh_tris, w.mesh_nodes};
    for (void *p : old)
        if (p) cudaFree(p);
    w.meshes = nullptr;
    w.mesh_verts = w.mesh_nodes = nullptr;
    w.mesh_tris = nullptr;
    int r;
    if ((r = dalloc(&w.meshes, hdr.size())) != CC_OK || (r = dalloc(&w.mesh_verts, verts.size())) != CC_OK ||
        (r = dalloc(&w.mesh_tris, tris.size())) != CC_OK || (r = dalloc(&w.mesh_nodes, nodes.size())) != CC_OK)
        return r;
    CC_TRY(cudaMemcpy(w.meshes, hdr.data(), sizeof(DevMesh) * hdr.size(), cudaMemcpyHostToDevice));
    if (!verts.empty()) CC_TRY(cudaMemcpy(w.mesh_verts, verts.data(), sizeof(float4) * verts.size(), cudaMemcpyHostToDevice));
    if (!tris.empty()) CC_TRY(cudaMemcpy(w.mesh_tris, tris.data(), sizeof(int4) * tris.size(), cudaMemcpyHostToDevice));
    if (!nodes.empty()) CC_TRY(cudaMemcpy(w.mesh_nodes, nodes.data(), sizeof(float4) * nodes.size(), cudaMemcpyHostToDevice));
    w.num_meshes = (int)hdr.size();
    drop_graph(W);
    return CC_OK;
}

static int export_mesh(const cc_mesh::Mesh &m, cc_mesh_info *info, float *vertices, int32_t *triangles,
                       float *normals, float *nodes) {
    if (!info) return CC_ERR_INVALID;
    memset(info, 0, sizeof(*info));
    info->num_vertices = (int32_t)(m.positions.size() / 3);
    info->num_triangles = (int32_t)m.active.size();
    info->num_nodes = (int32_t)(m.nodes.size() / 8);
    for (int k = 0; k < 3; k++) {
        info->bounds_min[k] = (float)m.lo[k];
        info->bounds_max[k] = (float)m.hi[k];
    }
    if (vertices)
        for (size_t k = 0; k < m.positions.size(); k++) vertices[k] = (float)m.positions[k];
    for (int t = 0; t < info->num_triangles; t++) {
        if (triangles) {
            for (int k = 0; k < 3; k++) triangles[4 * t + k] = m.tris[3 * t + k];
            triangles[4 * t + 3] = m.active[t];
        }
        if (normals)
            for (int k = 0; k < 3; k++) normals[3 * t + k] = (float)m.normals[3 * t + k];
    }
    if (nodes)
        for (int k = 0; k < info->num_nodes; k++) {
            const double *nd = &m.nodes[8 * k];
            for (int j = 0; j < 6; j++) nodes[8 * k + j] = (float)nd[j];
            nodes[8 * k + 6] = (float)(nd[7] >= 0 ? nd[6] / 8 : nd[6]);
            nodes[8 * k + 7] = (float)nd[7];
        }
    return CC_OK;
}

extern "C" {

int cc_world_add_triangle_mesh(cc_world *W, const double *positions, int32_t nv, const int32_t *indices, int32_t nt,
                               double degenerate_tolerance, double active_edge_cos, int32_t *out_mesh) {
    if (!W) return CC_ERR_INVALID;
    cc_mesh::Mesh m;
    int r = build_mesh_from(positions, nv, indices, nt, degenerate_tolerance, active_edge_cos, m);
    if (r != CC_OK) return r;
    W->meshes.push_back(std::move(m));
    W->meshes_dirty = true;  // uploaded with the next launch (sync_shapes)
    drop_graph(W);
    if (out_mesh) *out_mesh = (int32_t)W->meshes.size() - 1;
    return CC_OK;
}

int cc_triangle_mesh_build(const double *positions, int32_t nv, const int32_t *indices, int32_t nt,
                           double degenerate_tolerance, double active_edge_cos, cc_mesh_info *info, float *vertices,
                           int32_t *triangles, float *normals, float *nodes) {
    cc_mesh::Mesh m;
    int r = build_mesh_from(positions, nv, indices, nt, degenerate_tolerance, active_edge_cos, m);
    if (r != CC_OK) return r;
    return export_mesh(m, info, vertices, triangles, normals, nodes);
}

int cc_world_get_triangle_mesh(cc_world *W, int32_t mesh, cc_mesh_info *info, float *vertices, int32_t *triangles,
                               float *normals, float *nodes) {
    if (!W || mesh < 0 || mesh >= (int)W->meshes.size()) return CC_ERR_INVALID;
    return export_mesh(W->meshes[mesh], info, vertices, triangles, normals, nodes);
}

}  // extern "C"

static int build_hull_from(const float *points, int32_t n, float convex_radius, cc_hull::Hull &h);

// ---------------------------------------------------------------------------
// compound shapes (compound.ts)
// ---------------------------------------------------------------------------
// one convex child's mass (its own density), inertia about its centre of mass (row-major, in the
// child's frame), centre of mass and local bounds in the child's frame, and inner radius
static bool child_leaf(const cc_world *W, const cc_compound_child &c, double &m, double I[9], double com[3],
                       double lo[3], double hi[3], double &inner) {
    const float *p = c.shape_params;
    const double rho = c.density;
    for (int k = 0; k < 9; k++) I[k] = 0;
    for (int k = 0; k < 3; k++) com[k] = 0;
    switch (c.shape_type) {
        case CC_SHAPE_BOX: {  // setMassAndInertiaOfSolidBox mass-properties.ts:36-52
            double f[3] = {2.0 * p[0], 2.0 * p[1], 2.0 * p[2]};
            m = f[0] * f[1] * f[2] * rho;
            I[0] = (f[1] * f[1] + f[2] * f[2]) * (m / 12.0);
            I[4] = (f[0] * f[0] + f[2] * f[2]) * (m / 12.0);
            I[8] = (f[0] * f[0] + f[1] * f[1]) * (m / 12.0);
            for (int k = 0; k < 3; k++) lo[k] = -p[k], hi[k] = p[k];
            inner = std::min((double)p[0], std::min((double)p[1], (double)p[2]));
            return p[0] > 0 && p[1] > 0 && p[2] > 0 && p[3] >= 0;
        }
        case CC_SHAPE_SPHERE: {  // sphere.ts:97-123
            double r = p[0];
            m = (4.0 / 3.0) * M_PI * r * r * r * rho;
            I[0] = I[4] = I[8] = 0.4 * m * r * r;
            for (int k = 0; k < 3; k++) lo[k] = -r, hi[k] = r;
            inner = r;
            return r > 0;
        }
        case CC_SHAPE_CAPSULE: {  // capsule.ts:119-157
            double r = p[0], h = p[1];
            double volume = M_PI * r * r * (2 * h) + (4.0 / 3.0) * M_PI * r * r * r;
            m = volume * rho;
            double r2 = r * r, height = 2.0 * h;
            double cyl = M_PI * height * r2 * rho, hemi = ((2.0 * M_PI) / 3.0) * r2 * r * rho;
            I[4] = r2 * cyl * 0.5 + hemi * (2.0 / 5.0) * r2;
            I[0] = I[8] = cyl * ((1.0 / 12.0) * height * height + (1.0 / 4.0) * r2) +
                          hemi * ((2.0 / 5.0) * r2 + h * h + (3.0 / 8.0) * h * r);
            lo[0] = lo[2] = -r, hi[0] = hi[2] = r;
            lo[1] = -(h + r), hi[1] = h + r;
            inner = r;
            return r > 0 && h > 0;
        }
        case CC_SHAPE_CYLINDER: {  // cylinder.ts computeMassProperties, getInnerRadius
            double h = p[0], r = p[1];
            m = M_PI * r * r * 2 * h * rho;
            I[4] = 0.5 * m * r * r;
            I[0] = I[8] = 0.5 * I[4] + (m * 4 * h * h) / 12;
            lo[0] = lo[2] = -r, hi[0] = hi[2] = r;
            lo[1] = -h, hi[1] = h;
            inner = std::min(h, r);
            return p[2] >= 0.f && p[0] >= p[2] && p[1] >= p[2];
        }
        case CC_SHAPE_CONVEX_HULL: {  // convex-hull.ts:453-459, 549-558
            const int hi_ = (int)p[0];
            if (!(p[0] == (float)hi_) || hi_ < 0 || hi_ >= (int)W->hulls.size()) return false;
            const cc_hull::Hull &H = W->hulls[hi_];
            m = H.volume * rho;
            for (int k = 0; k < 9; k++) I[k] = H.inertia[k] * rho;
            com[0] = H.com.x, com[1] = H.com.y, com[2] = H.com.z;
            lo[0] = H.lo.x, lo[1] = H.lo.y, lo[2] = H.lo.z;
            hi[0] = H.hi.x, hi[1] = H.hi.y, hi[2] = H.hi.z;
            inner = H.inner_radius;
            return true;
        }
        default:
            return false;
    }
}

// every compound's children, uploaded whenever a compound is added
static int upload_compounds(cc_world *W) {
    DevWorld &w = W->w;
    std::vector<DevCompound> hdr;
    std::vector<DevChild> ch;
    for (const cc_world::Compound &c : W->compounds) {
        DevCompound d;
        d.first = (int)ch.size();
        d.count = (int)c.children.size();
        d.sub_bits = c.sub_bits;
        d.pad = 0;
        for (const cc_compound_child &k : c.children) {
            DevChild x;
            x.params = make_float4(k.shape_params[0], k.shape_params[1], k.shape_params[2], k.shape_params[3]);
            if (k.shape_type == CC_SHAPE_CONVEX_HULL) {  // the body record's form: the index as int bits
                const int h = (int)k.shape_params[0];
                float bits;
                memcpy(&bits, &h, sizeof(float));
                x.params = make_float4(bits, (float)W->hulls[h].convex_radius, 0.f, 0.f);
            }
            float tbits;
            const int t = k.shape_type;
            memcpy(&tbits, &t, sizeof(float));
            x.pos = make_float4(k.position[0], k.position[1], k.position[2], tbits);
            x.quat = make_float4(k.quaternion[0], k.quaternion[1], k.quaternion[2], k.quaternion[3]);
            ch.push_back(x);
        }
        hdr.push_back(d);
    }
    CC_TRY(cudaStreamSynchronize(W->stream));
    if (w.compounds) cudaFree(w.compounds);
    if (w.children) cudaFree(w.children);
    w.compounds = nullptr;
    w.children = nullptr;
    int r;
    if ((r = dalloc(&w.compounds, hdr.size())) != CC_OK || (r = dalloc(&w.children, ch.size())) != CC_OK) return r;
    CC_TRY(cudaMemcpy(w.compounds, hdr.data(), sizeof(DevCompound) * hdr.size(), cudaMemcpyHostToDevice));
    CC_TRY(cudaMemcpy(w.children, ch.data(), sizeof(DevChild) * ch.size(), cudaMemcpyHostToDevice));
    w.num_compounds = (int)hdr.size();
    return CC_OK;
}

extern "C" {

int cc_world_add_compound(cc_world *W, const cc_compound_child *children, int32_t n, int32_t *out_index) {
    if (!W || !children || n < 1 || n > 4096) return CC_ERR_INVALID;
    cc_world::Compound c;
    c.children.assign(children, children + n);
    std::vector<double> mass((size_t)n), inertia(9 * (size_t)n), ccom(3 * (size_t)n);
    double total = 0, acc[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        const cc_compound_child &k = children[i];
        if (!finite3(k.position) || !std::isfinite(k.density) || !(k.density > 0.f)) return CC_ERR_INVALID;
        for (int j = 0; j < 4; j++)
            if (!std::isfinite(k.shape_params[j]) || !std::isfinite(k.quaternion[j])) return CC_ERR_INVALID;
        double m, I[9], com[3], lo[3], hi[3], inner;
        if (!child_leaf(W, k, m, I, com, lo, hi, inner)) return CC_ERR_INVALID;
        const DQ q{k.quaternion[0], k.quaternion[1], k.quaternion[2], k.quaternion[3]};
        // computeCompoundLocalBounds :70-108: the child's bounds' corners through its pose
        for (int cnr = 0; cnr < 8; cnr++) {
            D3 v = drot(q, D3{(cnr & 1) ? hi[0] : lo[0], (cnr & 2) ? hi[1] : lo[1], (cnr & 4) ? hi[2] : lo[2]});
            double e[3] = {v.x + k.position[0], v.y + k.position[1], v.z + k.position[2]};
            for (int a = 0; a < 3; a++) {
                c.lo[a] = (i == 0 && cnr == 0) ? e[a] : std::min(c.lo[a], e[a]);
                c.hi[a] = (i == 0 && cnr == 0) ? e[a] : std::max(c.hi[a], e[a]);
            }
        }
        c.inner = i == 0 ? inner : std::min(c.inner, inner);  // getInnerRadius :283-289
        // the child's centre of mass in the compound's frame (computeCompoundCenterOfMass :110-141)
        const D3 cw = drot(q, D3{com[0], com[1], com[2]});
        ccom[3 * i] = cw.x + k.position[0];
        ccom[3 * i + 1] = cw.y + k.position[1];
        ccom[3 * i + 2] = cw.z + k.position[2];
        for (int a = 0; a < 3; a++) acc[a] += ccom[3 * i + a] * m;
        total += m;
        mass[i] = m;
        for (int j = 0; j < 9; j++) inertia[9 * i + j] = I[j];
    }
    for (int a = 0; a < 3; a++) c.com[a] = total > 0 ? acc[a] / total : 0.0;
    // computeMassProperties :177-230: each child's inertia rotated by its quaternion and moved
    // to the compound's centre of mass (massProperties.rotate / translate)
    for (int i = 0; i < n; i++) {
        const cc_compound_child &k = children[i];
        const DQ q{k.quaternion[0], k.quaternion[1], k.quaternion[2], k.quaternion[3]};
        const D3 cols[3] = {drot(q, D3{1, 0, 0}), drot(q, D3{0, 1, 0}), drot(q, D3{0, 0, 1})};
        const double R[9] = {cols[0].x, cols[1].x, cols[2].x, cols[0].y, cols[1].y, cols[2].y,
                             cols[0].z, cols[1].z, cols[2].z};  // row-major
        const double *t = &inertia[9 * i];
        double rt[9];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                rt[3 * a + b] = 0;
                for (int j = 0; j < 3; j++) rt[3 * a + b] += R[3 * a + j] * t[3 * j + b];
            }
        const double d[3] = {ccom[3 * i] - c.com[0], ccom[3 * i + 1] - c.com[1], ccom[3 * i + 2] - c.com[2]};
        const double dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double o = 0;
                for (int j = 0; j < 3; j++) o += rt[3 * a + j] * R[3 * b + j];
                c.inertia[3 * a + b] += o + mass[i] * ((a == b ? dd : 0.0) - d[a] * d[b]);
            }
    }
    c.mass = total;
    const unsigned maxi = (unsigned)(n - 1);
    c.sub_bits = maxi == 0 ? 0 : 32 - __builtin_clz(maxi);
    W->compounds.push_back(std::move(c));
    W->compounds_dirty = true;  // uploaded with the next launch (sync_shapes)
    drop_graph(W);
    if (out_index) *out_index = (int32_t)W->compounds.size() - 1;
    return CC_OK;
}

}  // extern "C"

extern "C" {

int cc_world_add_convex_hull(cc_world *W, const float *points, int32_t n, float convex_radius, int32_t *out_hull) {
    if (!W) return CC_ERR_INVALID;
    cc_hull::Hull h;
    int r = build_hull_from(points, n, convex_radius, h);
    if (r != CC_OK) return r;
    W->hulls.push_back(h);
    W->hulls_dirty = true;  // uploaded with the next launch (sync_shapes)
    drop_graph(W);
    if (out_hull) *out_hull = (int32_t)W->hulls.size() - 1;
    return CC_OK;
}

}  // extern "C"

static int build_hull_from(const float *points, int32_t n, float convex_radius, cc_hull::Hull &h) {
    if (!points || n < 4 || n > 65536 || std::isnan(convex_radius)) return CC_ERR_INVALID;
    std::vector<cc_hull::V> in((size_t)n);
    for (int i = 0; i < n; i++) {
        if (!finite3(points + 3 * i)) return CC_ERR_INVALID;
        in[i] = {points[3 * i], points[3 * i + 1], points[3 * i + 2]};
    }
    double radius = convex_radius < 0.f ? 0.05 : (double)convex_radius;  // DEFAULT_CONVEX_RADIUS support.ts:5
    // hullTolerance 1e-3, maxErrorConvexRadius 0.05, MAX_POINTS_IN_HULL 256 (convex-hull.ts:87, 107, 368)
    return cc_hull::build(in, radius, 1e-3, 0.05, 256, h) == 0 ? CC_OK : CC_ERR_INVALID;
}

static int export_hull(const cc_hull::Hull &h, cc_hull_info *info, float *points, float *shrunk, int32_t *faces,
                       int32_t *face_vertices, float *planes, int32_t *point_faces);

extern "C" {

int cc_convex_hull_build(const float *in_points, int32_t n, float convex_radius, cc_hull_info *info, float *points,
                         float *shrunk, int32_t *faces, int32_t *face_vertices, float *planes,
                         int32_t *point_faces) {
    if (!info) return CC_ERR_INVALID;
    cc_hull::Hull h;
    int r = build_hull_from(in_points, n, convex_radius, h);
    if (r != CC_OK) return r;
    return export_hull(h, info, points, shrunk, faces, face_vertices, planes, point_faces);
}

int cc_world_get_convex_hull(cc_world *W, int32_t hull, cc_hull_info *info, float *points, float *shrunk,
                             int32_t *faces, int32_t *face_vertices, float *planes, int32_t *point_faces) {
    if (!W || !info || hull < 0 || hull >= (int)W->hulls.size()) return CC_ERR_INVALID;
    return export_hull(W->hulls[hull], info, points, shrunk, faces, face_vertices, planes, point_faces);
}

}  // extern "C"

static int export_hull(const cc_hull::Hull &h, cc_hull_info *info, float *points, float *shrunk, int32_t *faces,
                       int32_t *face_vertices, float *planes, int32_t *point_faces) {
    memset(info, 0, sizeof(*info));
    info->num_points = (int32_t)h.points.size();
    info->num_faces = (int32_t)h.face_first.size();
    info->num_face_vertices = (int32_t)h.vidx.size();
    info->convex_radius = (float)h.convex_radius;
    info->volume = (float)h.volume;
    info->inner_radius = (float)h.inner_radius;
    info->com[0] = (float)h.com.x;
    info->com[1] = (float)h.com.y;
    info->com[2] = (float)h.com.z;
    for (int k = 0; k < 9; k++) info->inertia[k] = (float)h.inertia[k];
    info->bounds_min[0] = (float)h.lo.x;
    info->bounds_min[1] = (float)h.lo.y;
    info->bounds_min[2] = (float)h.lo.z;
    info->bounds_max[0] = (float)h.hi.x;
    info->bounds_max[1] = (float)h.hi.y;
    info->bounds_max[2] = (float)h.hi.z;
    for (size_t k = 0; k < h.points.size(); k++) {
        if (points) {
            points[3 * k] = (float)h.points[k].x;
            points[3 * k + 1] = (float)h.points[k].y;
            points[3 * k + 2] = (float)h.points[k].z;
        }
        if (shrunk) {
            shrunk[3 * k] = (float)h.shrunk[k].x;
            shrunk[3 * k + 1] = (float)h.shrunk[k].y;
            shrunk[3 * k + 2] = (float)h.shrunk[k].z;
        }
        if (point_faces)
            for (int m = 0; m < 4; m++) point_faces[4 * k + m] = h.point_faces[k][m];
    }
    for (size_t f = 0; f < h.face_first.size(); f++) {
        if (faces) {
            faces[2 * f] = h.face_first[f];
            faces[2 * f + 1] = h.face_count[f];
        }
        if (planes) {
            planes[4 * f] = (float)h.plane_n[f].x;
            planes[4 * f + 1] = (float)h.plane_n[f].y;
            planes[4 * f + 2] = (float)h.plane_n[f].z;
            planes[4 * f + 3] = (float)h.plane_c[f];
        }
    }
    if (face_vertices)
        for (size_t k = 0; k < h.vidx.size(); k++) face_vertices[k] = h.vidx[k];
    return CC_OK;
}

// ---------------------------------------------------------------------------
// point, distance, fixed, cone and slider joints: created in FP64 from the bodies' current
// poses (the create functions of point-, distance-, fixed-, cone- and slider-constraint.ts)
// into one record type, DevJoint, kept sorted by (type, per-type index)
// ---------------------------------------------------------------------------
namespace {
struct BodyPoses {
    std::vector<float4> quat, com, inv;  // inv.w: inverse mass
    std::vector<int> world;
};
int read_poses(cc_world *W, BodyPoses &p) {
    DevWorld &w = W->w;
    p.quat.resize((size_t)w.n);
    p.com.resize((size_t)w.n);
    p.inv.resize((size_t)w.n);
    p.world.resize((size_t)w.n);
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaMemcpy(p.quat.data(), w.quat, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(p.com.data(), w.com, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(p.inv.data(), w.inv_inertia, sizeof(float4) * w.n, cudaMemcpyDeviceToHost));
    CC_TRY(cudaMemcpy(p.world.data(), w.world, sizeof(int) * w.n, cudaMemcpyDeviceToHost));
    return CC_OK;
}
// the fields every joint description carries
template <typename D>
bool common_ok(const DevWorld &w, const D &d) {
    return d.body_a >= 0 && d.body_b >= 0 && d.body_a < w.n && d.body_b < w.n &&
           (d.space == CC_SPACE_WORLD || d.space == CC_SPACE_LOCAL) && d.num_velocity_steps_override >= 0 &&
           d.num_velocity_steps_override <= 255 && d.num_position_steps_override >= 0 &&
           d.num_position_steps_override <= 255 && finite3(d.point_a) && finite3(d.point_b);
}
template <typename D>
DevJoint joint_record(cc_world *W, const D &d, int type, int index) {
    DevJoint j;
    memset(&j, 0, sizeof(j));
    j.type = type;
    j.h.a = d.body_a;
    j.h.b = d.body_b;
    j.h.index = index;
    j.h.priority = d.priority;
    j.h.island = -1;
    j.h.flags = d.enabled ? JF_ENABLED : 0;
    j.h.iter_ovr = (int)((uint32_t)d.num_velocity_steps_override | ((uint32_t)d.num_position_steps_override << 8));
    if (j.h.iter_ovr) W->any_iter_override = true;
    j.inv_initial = make_float4(0.f, 0.f, 0.f, 1.f);
    j.wn = make_float3(0.f, 1.f, 0.f);
    return j;
}
// attachment points from the centres of mass in body space (world-space input taken against
// the current poses), or the inverse-mass-weighted anchor of autoDetectPoint
void attach(DevJoint &j, const BodyPoses &p, const float *pa, const float *pb, int space, bool auto_detect) {
    const int a = j.h.a, b = j.h.b;
    if (space == CC_SPACE_WORLD) {
        DQ iqa = dconj(dq(p.quat[a])), iqb = dconj(dq(p.quat[b]));
        D3 ca = d3(p.com[a]), cb = d3(p.com[b]);
        D3 wa = d3(pa), wb = d3(pb);
        if (auto_detect) {
            double ima = p.inv[a].w, imb = p.inv[b].w, im = ima + imb;
            D3 anchor = ca;
            if (im > 0) anchor = {ca.x * (ima / im) + cb.x * (imb / im), ca.y * (ima / im) + cb.y * (imb / im),
                                  ca.z * (ima / im) + cb.z * (imb / im)};
            wa = wb = anchor;
        }
        j.lp1 = f3d(drot(iqa, dsub(wa, ca)));
        j.lp2 = f3d(drot(iqb, dsub(wb, cb)));
    } else {
        j.lp1 = f3d(d3(pa));
        j.lp2 = f3d(d3(pb));
    }
}
// mathcat's (gl-matrix's) approximate vec3.equals: |a - b| <= 1e-6 max(1, |a|, |b|) per component
bool dequals(D3 a, D3 b) {
    auto eq = [](double x, double y) {
        return std::fabs(x - y) <= 1e-6 * std::max(1.0, std::max(std::fabs(x), std::fabs(y)));
    };
    return eq(a.x, b.x) && eq(a.y, b.y) && eq(a.z, b.z);
}
float4 f4q(DQ q) { return make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w); }
}  // namespace

// insert new records of one type after the existing ones of that type, keeping the device
// records' accumulated impulses
static int add_other_joints(cc_world *W, int type, const std::vector<DevJoint> &made, int32_t *out_index) {
    DevWorld &w = W->w;
    const int n = (int)made.size();
    int r = ensure_joint_capacity(W, w.num_hinges, w.num_swings, w.num_others + n);
    if (r != CC_OK) return r;
    if (w.num_others > 0) {
        CC_TRY(cudaStreamSynchronize(W->stream));
        CC_TRY(cudaMemcpy(W->others.data(), w.others, sizeof(DevJoint) * w.num_others, cudaMemcpyDeviceToHost));
    }
    auto pos = std::upper_bound(W->others.begin(), W->others.end(), type,
                                [](int t, const DevJoint &j) { return t < j.type; });
    W->others.insert(pos, made.begin(), made.end());
    for (int i = 0; i < n; i++)
        if (out_index) out_index[i] = made[i].h.index;
    w.num_others += n;
    for (int t = 0; t < JT_TYPES; t++) {
        if (t == JT_HINGE || t == JT_SWING || t == JT_SIX_DOF) continue;
        w.type_count[t] = 0;
        w.type_first[t] = 0;
    }
    for (int k = w.num_others - 1; k >= 0; k--) {
        w.type_first[W->others[k].type] = k;
        w.type_count[W->others[k].type]++;
    }
    CC_TRY(cudaMemcpy(w.others, W->others.data(), sizeof(DevJoint) * w.num_others, cudaMemcpyHostToDevice));
    drop_graph(W);
    return upload_partners(W);
}
template <typename F>
static int edit_sixdof(cc_world *W, int32_t index, F f) {
    return edit_joint(W, W->w.sixdofs, W->sixdofs, W->w.num_sixdofs, index, f);
}
template <typename F>
static int edit_other(cc_world *W, int type, int32_t index, F f) {
    DevWorld &w = W->w;
    if (type < 0 || type >= JT_TYPES || type == JT_HINGE || type == JT_SWING || type == JT_SIX_DOF)
        return CC_ERR_INVALID;
    if (index < 0 || index >= w.type_count[type]) return CC_ERR_INVALID;
    return edit_joint(W, w.others, W->others, w.num_others, w.type_first[type] + index, f);
}

extern "C" {

int cc_world_add_point_joints(cc_world *W, const cc_point_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++)
        if (!common_ok(w, d[i])) return CC_ERR_INVALID;
    BodyPoses p;
    if (int r = read_poses(W, p)) return r;
    std::vector<DevJoint> made;
    for (int i = 0; i < n; i++) {
        if (p.world[d[i].body_a] != p.world[d[i].body_b]) return CC_ERR_INVALID;
        DevJoint j = joint_record(W, d[i], JT_POINT, w.type_count[JT_POINT] + i);
        attach(j, p, d[i].point_a, d[i].point_b, d[i].space, false);
        made.push_back(j);
    }
    return add_other_joints(W, JT_POINT, made, out_index);
}

int cc_world_add_distance_joints(cc_world *W, const cc_distance_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++)
        if (!common_ok(w, d[i]) || !spring_ok(d[i].spring) || std::isnan(d[i].min_distance) ||
            std::isnan(d[i].max_distance))
            return CC_ERR_INVALID;
    BodyPoses p;
    if (int r = read_poses(W, p)) return r;
    std::vector<DevJoint> made;
    for (int i = 0; i < n; i++) {
        const cc_distance_desc &h = d[i];
        if (p.world[h.body_a] != p.world[h.body_b]) return CC_ERR_INVALID;
        DevJoint j = joint_record(W, h, JT_DISTANCE, w.type_count[JT_DISTANCE] + i);
        attach(j, p, h.point_a, h.point_b, h.space, false);
        // the current distance of the attachment points (distance-constraint.ts:166-181)
        D3 wp1, wp2;
        if (h.space == CC_SPACE_WORLD) {
            wp1 = d3(h.point_a);
            wp2 = d3(h.point_b);
        } else {
            D3 r1 = drot(dq(p.quat[h.body_a]), d3(h.point_a)), r2 = drot(dq(p.quat[h.body_b]), d3(h.point_b));
            D3 ca = d3(p.com[h.body_a]), cb = d3(p.com[h.body_b]);
            wp1 = {r1.x + ca.x, r1.y + ca.y, r1.z + ca.z};
            wp2 = {r2.x + cb.x, r2.y + cb.y, r2.z + cb.z};
        }
        D3 dd = dsub(wp2, wp1);
        double dist = std::sqrt(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
        double mn = h.min_distance, mx = h.max_distance;
        if (mn < 0 && mx < 0) {
            mn = mx = dist;
        } else {
            double m0 = mn < 0 ? std::min(dist, mx) : mn, m1 = mx < 0 ? std::max(dist, mn) : mx;
            mn = m0;
            mx = m1;
        }
        j.min_dist = (float)mn;
        j.max_dist = (float)mx;
        j.spring_mode = h.spring.mode;
        j.spring_freq = h.spring.frequency_or_stiffness;
        j.spring_damping = h.spring.damping;
        j.wp1 = f3d(wp1);
        j.wp2 = f3d(wp2);
        made.push_back(j);
    }
    return add_other_joints(W, JT_DISTANCE, made, out_index);
}

int cc_world_set_distance(cc_world *W, int32_t index, float min_distance, float max_distance) {
    if (!W || std::isnan(min_distance) || std::isnan(max_distance)) return CC_ERR_INVALID;
    return edit_other(W, JT_DISTANCE, index, [&](DevJoint &j) {  // setDistance :484-493
        if (min_distance >= 0) j.min_dist = min_distance;
        if (max_distance >= 0) j.max_dist = max_distance;
        if (j.min_dist > j.max_dist) j.min_dist = j.max_dist = (j.min_dist + j.max_dist) / 2;
    });
}

int cc_world_add_fixed_joints(cc_world *W, const cc_fixed_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++)
        if (!common_ok(w, d[i]) || !finite3(d[i].axis_x_a) || !finite3(d[i].axis_y_a) || !finite3(d[i].axis_x_b) ||
            !finite3(d[i].axis_y_b))
            return CC_ERR_INVALID;
    BodyPoses p;
    if (int r = read_poses(W, p)) return r;
    std::vector<DevJoint> made;
    for (int i = 0; i < n; i++) {
        const cc_fixed_desc &h = d[i];
        if (p.world[h.body_a] != p.world[h.body_b]) return CC_ERR_INVALID;
        DevJoint j = joint_record(W, h, JT_FIXED, w.type_count[JT_FIXED] + i);
        attach(j, p, h.point_a, h.point_b, h.space, h.auto_detect_point != 0);
        // getInvInitialOrientationXY (rotation-euler-constraint-part.ts:71-111)
        D3 x1 = dnormalize(d3(h.axis_x_a)), y1 = dnormalize(d3(h.axis_y_a));
        D3 x2 = dnormalize(d3(h.axis_x_b)), y2 = dnormalize(d3(h.axis_y_b));
        DQ r0{0, 0, 0, 1};
        if (!(dequals(x1, x2) && dequals(y1, y2)))
            r0 = dqmul(quat_from_columns(x2, y2, dcross(x2, y2)), dconj(quat_from_columns(x1, y1, dcross(x1, y1))));
        if (h.space == CC_SPACE_WORLD)
            j.inv_initial = f4q(dqmul(dqmul(dconj(dq(p.quat[h.body_b])), r0), dq(p.quat[h.body_a])));
        else
            j.inv_initial = f4q(r0);
        made.push_back(j);
    }
    return add_other_joints(W, JT_FIXED, made, out_index);
}

int cc_world_add_cone_joints(cc_world *W, const cc_cone_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++)
        if (!common_ok(w, d[i]) || !finite3(d[i].twist_axis_a) || !finite3(d[i].twist_axis_b) ||
            !std::isfinite(d[i].half_cone_angle))
            return CC_ERR_INVALID;
    BodyPoses p;
    if (int r = read_poses(W, p)) return r;
    std::vector<DevJoint> made;
    for (int i = 0; i < n; i++) {
        const cc_cone_desc &h = d[i];
        if (p.world[h.body_a] != p.world[h.body_b]) return CC_ERR_INVALID;
        DevJoint j = joint_record(W, h, JT_CONE, w.type_count[JT_CONE] + i);
        attach(j, p, h.point_a, h.point_b, h.space, false);
        D3 t1 = dnormalize(d3(h.twist_axis_a)), t2 = dnormalize(d3(h.twist_axis_b));
        j.cos_half_cone = (float)std::cos((double)h.half_cone_angle);
        // getNormalizedPerpendicular (cone-constraint.ts:118-136): the fallback limit axis
        double ax = std::fabs(t1.x), ay = std::fabs(t1.y), az = std::fabs(t1.z);
        D3 perp = (ax <= ay && ax <= az) ? D3{0, -t1.z, t1.y} : (ay <= az ? D3{t1.z, 0, -t1.x} : D3{-t1.y, t1.x, 0});
        perp = dnormalize(perp);
        if (h.space == CC_SPACE_WORLD) {
            j.lt1 = f3d(drot(dconj(dq(p.quat[h.body_a])), t1));
            j.lt2 = f3d(drot(dconj(dq(p.quat[h.body_b])), t2));
            j.w_rot_axis = f3d(perp);
        } else {
            j.lt1 = f3d(t1);
            j.lt2 = f3d(t2);
            j.w_rot_axis = f3d(drot(dq(p.quat[h.body_a]), perp));
        }
        j.cos_theta = 1.f;
        made.push_back(j);
    }
    return add_other_joints(W, JT_CONE, made, out_index);
}

int cc_world_set_cone_half_angle(cc_world *W, int32_t index, float half_cone_angle) {
    if (!W || std::isnan(half_cone_angle)) return CC_ERR_INVALID;
    const double PI = 3.14159265358979323846;
    return edit_other(W, JT_CONE, index, [&](DevJoint &j) {  // setHalfConeAngle :262-264
        j.cos_half_cone = (float)std::cos(std::max(0.0, std::min(PI, (double)half_cone_angle)));
    });
}

int cc_world_add_slider_joints(cc_world *W, const cc_slider_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++) {
        const cc_slider_desc &h = d[i];
        if (!common_ok(w, h) || !finite3(h.slider_axis_a) || !finite3(h.slider_axis_b) || !finite3(h.normal_axis_a) ||
            !finite3(h.normal_axis_b) || !spring_ok(h.limits_spring) || !spring_ok(h.motor_spring) ||
            std::isnan(h.limits_min) || std::isnan(h.limits_max) || std::isnan(h.max_friction_force) ||
            std::isnan(h.min_force_limit) || std::isnan(h.max_force_limit) || h.motor_state < 0 || h.motor_state > 2 ||
            !std::isfinite(h.target_velocity) || !std::isfinite(h.target_position))
            return CC_ERR_INVALID;
    }
    BodyPoses p;
    if (int r = read_poses(W, p)) return r;
    std::vector<DevJoint> made;
    for (int i = 0; i < n; i++) {
        const cc_slider_desc &h = d[i];
        if (p.world[h.body_a] != p.world[h.body_b]) return CC_ERR_INVALID;
        DevJoint j = joint_record(W, h, JT_SLIDER, w.type_count[JT_SLIDER] + i);
        attach(j, p, h.point_a, h.point_b, h.space, h.auto_detect_point != 0);
        D3 s1 = dnormalize(d3(h.slider_axis_a)), s2 = dnormalize(d3(h.slider_axis_b));
        D3 n1 = dnormalize(d3(h.normal_axis_a)), n2 = dnormalize(d3(h.normal_axis_b));
        // getInvInitialOrientationXY (slider-constraint.ts:203-259)
        const double eps = 1e-6;
        DQ r0{0, 0, 0, 1};
        if (!(std::fabs(s1.x - s2.x) < eps && std::fabs(s1.y - s2.y) < eps && std::fabs(s1.z - s2.z) < eps &&
              std::fabs(n1.x - n2.x) < eps && std::fabs(n1.y - n2.y) < eps && std::fabs(n1.z - n2.z) < eps))
            r0 = dqmul(quat_from_columns(s2, n2, dcross(s2, n2)), dconj(quat_from_columns(s1, n1, dcross(s1, n1))));
        D3 ls1, ln1;
        if (h.space == CC_SPACE_WORLD) {
            DQ iqa = dconj(dq(p.quat[h.body_a]));
            ls1 = dnormalize(drot(iqa, s1));
            ln1 = dnormalize(drot(iqa, n1));
            j.inv_initial = f4q(dqmul(dqmul(dconj(dq(p.quat[h.body_b])), r0), dq(p.quat[h.body_a])));
        } else {
            ls1 = s1;
            ln1 = n1;
            j.inv_initial = f4q(r0);
        }
        j.ls1 = f3d(ls1);
        j.ln1 = f3d(ln1);
        j.ln2 = f3d(dcross(ls1, ln1));
        // limits :384-388 (min raised to <= 0, max to >= 0) and the setters :495-520
        const float INF = std::numeric_limits<float>::infinity();
        j.limits_min = std::min(h.limits_min, 0.f);
        j.limits_max = std::max(h.limits_max, 0.f);
        j.slider_flags = (j.limits_min != -INF || j.limits_max != INF) ? 1 : 0;
        j.limits_spring_mode = h.limits_spring.mode;
        j.limits_freq = h.limits_spring.frequency_or_stiffness;
        j.limits_damping = h.limits_spring.damping;
        j.max_friction_force = h.max_friction_force;
        j.motor_spring_mode = h.motor_spring.mode;
        j.motor_freq = h.motor_spring.frequency_or_stiffness;
        j.motor_damping = h.motor_spring.damping;
        j.min_force = h.min_force_limit;
        j.max_force = h.max_force_limit;
        j.motor_state = h.motor_state;
        j.target_velocity = h.target_velocity;
        j.target_position =
            j.slider_flags ? std::max(j.limits_min, std::min(j.limits_max, h.target_position)) : h.target_position;
        made.push_back(j);
    }
    return add_other_joints(W, JT_SLIDER, made, out_index);
}

int cc_world_set_slider_limits(cc_world *W, int32_t index, float limits_min, float limits_max) {
    if (!W || std::isnan(limits_min) || std::isnan(limits_max)) return CC_ERR_INVALID;
    return edit_other(W, JT_SLIDER, index, [&](DevJoint &j) {  // setLimits :488-493
        const float INF = std::numeric_limits<float>::infinity();
        j.limits_min = std::min(limits_min, 0.f);
        j.limits_max = std::max(limits_max, 0.f);
        j.slider_flags = (j.limits_min != -INF || j.limits_max != INF) ? 1 : 0;
    });
}

int cc_world_set_slider_motor(cc_world *W, int32_t index, int32_t motor_state, float target_velocity,
                              float target_position) {
    if (!W || motor_state < 0 || motor_state > 2 || !std::isfinite(target_velocity) || !std::isfinite(target_position))
        return CC_ERR_INVALID;
    return edit_other(W, JT_SLIDER, index, [&](DevJoint &j) {  // setMotorState / setTargetVelocity / setTargetPosition
        j.motor_state = motor_state;
        j.target_velocity = target_velocity;
        j.target_position = j.slider_flags ? std::max(j.limits_min, std::min(j.limits_max, target_position))
                                           : target_position;
    });
}

int cc_world_get_slider_positions(cc_world *W, float *out, int32_t capacity) {
    if (!W || capacity < 0 || (capacity > 0 && !out)) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    const int ns = w.type_count[JT_SLIDER];
    const int n = std::min(capacity, ns);
    if (n > 0) {
        BodyPoses p;
        if (int r = read_poses(W, p)) return r;
        for (int k = 0; k < n; k++) {  // getCurrentPosition :460-476
            const DevJoint &j = W->others[w.type_first[JT_SLIDER] + k];
            DQ qa = dq(p.quat[j.h.a]), qb = dq(p.quat[j.h.b]);
            D3 r1 = drot(qa, {j.lp1.x, j.lp1.y, j.lp1.z}), r2 = drot(qb, {j.lp2.x, j.lp2.y, j.lp2.z});
            D3 ca = d3(p.com[j.h.a]), cb = d3(p.com[j.h.b]);
            D3 u{cb.x - ca.x + r2.x - r1.x, cb.y - ca.y + r2.y - r1.y, cb.z - ca.z + r2.z - r1.z};
            D3 ax = drot(qa, {j.ls1.x, j.ls1.y, j.ls1.z});
            out[k] = (float)(u.x * ax.x + u.y * ax.y + u.z * ax.z);
        }
    }
    return capacity < ns ? CC_ERR_CAPACITY : CC_OK;
}

int cc_world_set_joint_enabled(cc_world *W, int32_t type, int32_t index, int32_t enabled) {
    if (!W) return CC_ERR_INVALID;
    if (type == JT_HINGE) return cc_world_set_hinge_enabled(W, index, enabled);
    if (type == JT_SWING) return cc_world_set_swing_twist_enabled(W, index, enabled);
    if (type == JT_SIX_DOF) {
        int r = edit_sixdof(
            W, index, [&](DevSixDof &j) { j.h.flags = enabled ? (j.h.flags | JF_ENABLED) : (j.h.flags & ~JF_ENABLED); });
        if (r != CC_OK) return r;
        return upload_partners(W);
    }
    int r = edit_other(W, type, index,
                       [&](DevJoint &j) { j.h.flags = enabled ? (j.h.flags | JF_ENABLED) : (j.h.flags & ~JF_ENABLED); });
    if (r != CC_OK) return r;
    return upload_partners(W);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// six-DOF joints (six-dof-constraint.ts)
// ---------------------------------------------------------------------------
namespace {
// updateTranslationLimits + updateRotationLimits + updateFixedFreeAxis (:240-285) in FP64 over
// the requested limits; the swing-twist part takes the rotation limits (setLimits)
void sixdof_set_limits(DevSixDof &j, const double in_min[6], const double in_max[6]) {
    const double PI = 3.14159265358979323846;
    double mn[6], mx[6];
    for (int i = 0; i < 6; i++) {
        mn[i] = in_min[i];
        mx[i] = in_max[i];
    }
    for (int i = 0; i < 3; i++)
        if (mn[i] > mx[i]) mn[i] = mx[i] = 0.0;
    if (j.swing_type == CC_SWING_CONE) {
        mx[4] = std::max(0.0, mx[4]);
        mx[5] = std::max(0.0, mx[5]);
        mn[4] = -mx[4];
        mn[5] = -mx[5];
    }
    for (int i = 3; i < 6; i++) {
        mn[i] = std::max(-PI, std::min(PI, mn[i]));
        mx[i] = std::max(-PI, std::min(PI, mx[i]));
        if (mn[i] > mx[i]) mn[i] = mx[i] = 0.0;
    }
    st_set_limits(j, mn[3], mx[3], mn[4], mx[4], mn[5], mx[5]);
    j.free_axis = j.fixed_axis = 0;
    for (int a = 0; a < 6; a++) {
        const double lim = a >= 3 ? PI : INFINITY;
        if (mn[a] >= mx[a])
            j.fixed_axis |= 1 << a;
        else if (mn[a] <= -lim && mx[a] >= lim)
            j.free_axis |= 1 << a;
        j.limit_min[a] = (float)mn[a];
        j.limit_max[a] = (float)mx[a];
    }
}
// cacheTranslationMotorActive / cacheRotationMotorActive / cacheRotationPositionMotorActive /
// cacheHasSpringLimits (:287-323)
void sixdof_cache_motors(DevSixDof &j) {
    auto friction = [&](int a) { return !((j.fixed_axis >> a) & 1) && j.max_friction[a] > 0.f; };
    j.flags &= SD_SPRING_LIMITS;
    j.rot_pos_motor = 0;
    for (int i = 0; i < 3; i++) {
        if (j.motor_state[i] != 0 || friction(i)) j.flags |= SD_TRANS_MOTOR;
        if (j.motor_state[3 + i] != 0 || friction(3 + i)) j.flags |= SD_ROT_MOTOR;
        if (j.motor_state[3 + i] == 2) j.rot_pos_motor |= 1 << i;
    }
}
// setTargetOrientationCS (:1293-1299): the target clamped into the rotation limits
void sixdof_set_target(DevSixDof &j, const float *q) {
    float4 o = make_float4(q[0], q[1], q[2], q[3]), sw, tw;
    get_swing_twist(o, sw, tw);
    clamp_swing_twist(j, sw, tw);
    j.target_q = qmul(sw, tw);
}
bool limits_ok(const float *mn, const float *mx) {
    for (int k = 0; k < 6; k++)
        if (std::isnan(mn[k]) || std::isnan(mx[k])) return false;
    return true;
}
}  // namespace

extern "C" {

int cc_world_add_six_dof_joints(cc_world *W, const cc_six_dof_desc *d, int32_t n, int32_t *out_index) {
    if (!W || (!d && n > 0) || n < 0) return CC_ERR_INVALID;
    if (n == 0) return CC_OK;
    DevWorld &w = W->w;
    for (int i = 0; i < n; i++) {
        const cc_six_dof_desc &h = d[i];
        if (h.body_a < 0 || h.body_b < 0 || h.body_a >= w.n || h.body_b >= w.n) return CC_ERR_INVALID;
        if (h.space != CC_SPACE_WORLD && h.space != CC_SPACE_LOCAL) return CC_ERR_INVALID;
        if (h.swing_type != CC_SWING_CONE && h.swing_type != CC_SWING_PYRAMID) return CC_ERR_INVALID;
        if (h.num_velocity_steps_override < 0 || h.num_velocity_steps_override > 255 ||
            h.num_position_steps_override < 0 || h.num_position_steps_override > 255)
            return CC_ERR_INVALID;
        if (!finite3(h.position_a) || !finite3(h.position_b) || !finite3(h.axis_x_a) || !finite3(h.axis_y_a) ||
            !finite3(h.axis_x_b) || !finite3(h.axis_y_b) || !finite3(h.target_velocity) ||
            !finite3(h.target_angular_velocity) || !finite3(h.target_position) || !limits_ok(h.limit_min, h.limit_max))
            return CC_ERR_INVALID;
        for (int k = 0; k < 4; k++)
            if (!std::isfinite(h.target_orientation[k])) return CC_ERR_INVALID;
        for (int k = 0; k < 3; k++)
            if (!spring_ok(h.limits_spring[k])) return CC_ERR_INVALID;
        for (int k = 0; k < 6; k++)
            if (!spring_ok(h.motor_spring[k]) || h.motor_state[k] < 0 || h.motor_state[k] > 2 ||
                std::isnan(h.max_friction[k]) || std::isnan(h.motor_min_force[k]) || std::isnan(h.motor_max_force[k]))
                return CC_ERR_INVALID;
    }
    BodyPoses p;
    if (int r = read_poses(W, p)) return r;
    std::vector<DevSixDof> made((size_t)n);
    for (int i = 0; i < n; i++) {
        const cc_six_dof_desc &h = d[i];
        if (p.world[h.body_a] != p.world[h.body_b]) return CC_ERR_INVALID;
        DevSixDof &j = made[i];
        memset(&j, 0, sizeof(j));
        j.h.a = h.body_a;
        j.h.b = h.body_b;
        j.h.index = w.num_sixdofs + i;
        j.h.iter_ovr = (int)((uint32_t)h.num_velocity_steps_override | ((uint32_t)h.num_position_steps_override << 8));
        if (j.h.iter_ovr) W->any_iter_override = true;
        j.h.priority = h.priority;
        j.h.island = -1;
        j.h.flags = h.enabled ? JF_ENABLED : 0;
        // constraint space from the columns (X, Y, X x Y) of each body (create :376-412)
        D3 x1 = dnormalize(d3(h.axis_x_a)), y1 = dnormalize(d3(h.axis_y_a));
        D3 x2 = dnormalize(d3(h.axis_x_b)), y2 = dnormalize(d3(h.axis_y_b));
        DQ c1 = quat_from_columns(x1, y1, dcross(x1, y1)), c2 = quat_from_columns(x2, y2, dcross(x2, y2));
        if (h.space == CC_SPACE_WORLD) {
            DQ iqa = dconj(dq(p.quat[h.body_a])), iqb = dconj(dq(p.quat[h.body_b]));
            j.lp1 = f3d(drot(iqa, dsub(d3(h.position_a), d3(p.com[h.body_a]))));
            j.lp2 = f3d(drot(iqb, dsub(d3(h.position_b), d3(p.com[h.body_b]))));
            c1 = dqmul(iqa, c1);
            c2 = dqmul(iqb, c2);
        } else {
            j.lp1 = f3d(d3(h.position_a));
            j.lp2 = f3d(d3(h.position_b));
        }
        j.c2b1 = f4q(c1);
        j.c2b2 = f4q(c2);
        j.swing_type = h.swing_type;
        double mn[6], mx[6];
        for (int k = 0; k < 6; k++) {
            mn[k] = h.limit_min[k];
            mx[k] = h.limit_max[k];
            j.max_friction[k] = h.max_friction[k];
            j.motor_state[k] = h.motor_state[k];
            j.motor_spring_mode[k] = h.motor_spring[k].mode;
            j.motor_freq[k] = h.motor_spring[k].frequency_or_stiffness;
            j.motor_damping[k] = h.motor_spring[k].damping;
            j.motor_min_force[k] = h.motor_min_force[k];
            j.motor_max_force[k] = h.motor_max_force[k];
        }
        for (int k = 0; k < 3; k++) {
            j.limits_spring_mode[k] = h.limits_spring[k].mode;
            j.limits_freq[k] = h.limits_spring[k].frequency_or_stiffness;
            j.limits_damping[k] = h.limits_spring[k].damping;
            if (j.limits_freq[k] > 0.f) j.flags |= SD_SPRING_LIMITS;
        }
        sixdof_set_limits(j, mn, mx);
        sixdof_cache_motors(j);
        j.target_v = make_float3(h.target_velocity[0], h.target_velocity[1], h.target_velocity[2]);
        j.target_w = make_float3(h.target_angular_velocity[0], h.target_angular_velocity[1],
                                 h.target_angular_velocity[2]);
        j.target_p = make_float3(h.target_position[0], h.target_position[1], h.target_position[2]);
        sixdof_set_target(j, h.target_orientation);
    }
    int r = ensure_joint_capacity(W, w.num_hinges, w.num_swings, -1, w.num_sixdofs + n);
    if (r != CC_OK) return r;
    CC_TRY(cudaMemcpy(w.sixdofs + w.num_sixdofs, made.data(), sizeof(DevSixDof) * n, cudaMemcpyHostToDevice));
    for (int i = 0; i < n; i++) {
        W->sixdofs.push_back(made[i]);
        if (out_index) out_index[i] = w.num_sixdofs + i;
    }
    w.num_sixdofs += n;
    w.type_count[JT_SIX_DOF] = w.num_sixdofs;
    drop_graph(W);
    return upload_partners(W);
}

int cc_world_set_six_dof_limits(cc_world *W, int32_t index, const float *limit_min, const float *limit_max) {
    if (!W || !limit_min || !limit_max || !limits_ok(limit_min, limit_max)) return CC_ERR_INVALID;
    return edit_sixdof(W, index, [&](DevSixDof &j) {  // setTranslationLimits + setRotationLimits :1238-1260
        double mn[6], mx[6];
        for (int k = 0; k < 6; k++) {
            mn[k] = limit_min[k];
            mx[k] = limit_max[k];
        }
        sixdof_set_limits(j, mn, mx);
    });
}

int cc_world_set_six_dof_motor(cc_world *W, int32_t index, const int32_t *motor_state, const float *target_velocity,
                               const float *target_angular_velocity, const float *target_position,
                               const float *target_orientation, const float *max_friction) {
    if (!W || !motor_state || !target_velocity || !target_angular_velocity || !target_position ||
        !target_orientation || !max_friction || !finite3(target_velocity) || !finite3(target_angular_velocity) ||
        !finite3(target_position))
        return CC_ERR_INVALID;
    for (int k = 0; k < 6; k++)
        if (motor_state[k] < 0 || motor_state[k] > 2 || std::isnan(max_friction[k])) return CC_ERR_INVALID;
    for (int k = 0; k < 4; k++)
        if (!std::isfinite(target_orientation[k])) return CC_ERR_INVALID;
    return edit_sixdof(W, index, [&](DevSixDof &j) {  // setMaxFriction, setMotorState, setTarget*CS :1262-1306
        for (int k = 0; k < 6; k++) {
            j.max_friction[k] = max_friction[k];
            if (j.motor_state[k] != motor_state[k]) {  // a changed state deactivates that motor part
                j.motor_state[k] = motor_state[k];
                if (k < 3) {
                    j.motor_t[k].eff = 0.f;
                    j.motor_t[k].lambda = 0.f;
                } else {
                    j.motor_r[k - 3].eff = 0.f;
                    j.motor_r[k - 3].lambda = 0.f;
                }
            }
        }
        sixdof_cache_motors(j);
        j.target_v = make_float3(target_velocity[0], target_velocity[1], target_velocity[2]);
        j.target_w = make_float3(target_angular_velocity[0], target_angular_velocity[1], target_angular_velocity[2]);
        j.target_p = make_float3(target_position[0], target_position[1], target_position[2]);
        sixdof_set_target(j, target_orientation);
    });
}

int cc_world_get_joint_lambdas(cc_world *W, int32_t type, int32_t index, float *out, int32_t capacity,
                               int32_t *count) {
    if (!W || capacity < 0 || (capacity > 0 && !out)) return CC_ERR_INVALID;
    DevWorld &w = W->w;
    if (type < 0 || type >= JT_TYPES || type == JT_HINGE || type == JT_SWING) return CC_ERR_INVALID;
    if (index < 0 || index >= w.type_count[type]) return CC_ERR_INVALID;
    if (type == JT_SIX_DOF) {  // translation rows, point, rotation, swing Y, swing Z, twist, motors
        DevSixDof x;
        CC_TRY(cudaStreamSynchronize(W->stream));
        CC_TRY(cudaMemcpy(&x, w.sixdofs + index, sizeof(DevSixDof), cudaMemcpyDeviceToHost));
        const float v[18] = {x.trans[0].lambda, x.trans[1].lambda, x.trans[2].lambda, x.pt.lambda.x, x.pt.lambda.y,
                             x.pt.lambda.z, x.rot.lambda.x, x.rot.lambda.y, x.rot.lambda.z, x.sy.lambda, x.sz.lambda,
                             x.tw.lambda, x.motor_t[0].lambda, x.motor_t[1].lambda, x.motor_t[2].lambda,
                             x.motor_r[0].lambda, x.motor_r[1].lambda, x.motor_r[2].lambda};
        for (int k = 0; k < std::min(18, capacity); k++) out[k] = v[k];
        if (count) *count = 18;
        return capacity < 18 ? CC_ERR_CAPACITY : CC_OK;
    }
    DevJoint j;
    CC_TRY(cudaStreamSynchronize(W->stream));
    CC_TRY(cudaMemcpy(&j, w.others + w.type_first[type] + index, sizeof(DevJoint), cudaMemcpyDeviceToHost));
    float v[7];
    int m = 0;
    auto put3 = [&](float3 a) {
        v[m++] = a.x;
        v[m++] = a.y;
        v[m++] = a.z;
    };
    switch (type) {
        case JT_POINT: put3(j.pt.lambda); break;
        case JT_DISTANCE: v[m++] = j.ax.lambda; break;
        case JT_FIXED:
            put3(j.pt.lambda);
            put3(j.rot.lambda);
            break;
        case JT_CONE:
            put3(j.pt.lambda);
            v[m++] = j.ang.lambda;
            break;
        case JT_SLIDER:
            v[m++] = j.dual.lambda[0];
            v[m++] = j.dual.lambda[1];
            put3(j.rot.lambda);
            v[m++] = j.ax.lambda;
            v[m++] = j.motor.lambda;
            break;
    }
    for (int k = 0; k < std::min(m, capacity); k++) out[k] = v[k];
    if (count) *count = m;
    return capacity < m ? CC_ERR_CAPACITY : CC_OK;
}

}  // extern "C"
