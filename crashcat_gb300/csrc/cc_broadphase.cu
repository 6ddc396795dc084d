// Force integration, body bounds and the LBVH broadphase.
//
// Reference: accelerationIntegrationUpdate (src/update.ts:245-319),
// rigidBody.updateAABB (src/body/rigid-body.ts:561-674) and
// broadphase.findCollidingPairs (src/broadphase/broadphase.ts:217-277).
//
// The reference keeps one incremental DBVT per broadphase layer.  Here the
// bodies of every world held by the handle go into one Karras LBVH built from
// 64-bit keys (world index << 30 | 30-bit Morton code of the AABB centre),
// sorted with the project radix sort.  Node bounds are FP32 rounded outward,
// so the tree only proposes candidates; each candidate is re-tested with the
// reference's exact FP64 predicate (tight body AABB against the querying
// body's AABB grown by the speculative contact distance, dbvt.ts:669 and
// broadphase.ts:249) so the reported pair set equals the reference's.
#include "cc_internal.cuh"

namespace cc {

// each translation unit keeps its own copy of the settings in constant memory
static __constant__ DevSettings c_settings;
static __constant__ double c_spec_dist64;

void upload_settings_narrowphase(const DevSettings &s, cudaStream_t st);
void upload_settings_solver(const DevSettings &s, cudaStream_t st);

void upload_settings(const DevSettings &s, double spec64, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(c_settings, &s, sizeof(DevSettings), 0, cudaMemcpyHostToDevice, st);
    cudaMemcpyToSymbolAsync(c_spec_dist64, &spec64, sizeof(double), 0, cudaMemcpyHostToDevice, st);
    upload_settings_narrowphase(s, st);
    upload_settings_solver(s, st);
    upload_settings_adjoint(s, st);
}

// ---------------------------------------------------------------------------
// accelerationIntegrationUpdate (update.ts:245-319), FP32
// ---------------------------------------------------------------------------
__global__ void k_integrate_forces(DevWorld w, float dt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        uint32_t f = w.flags[i];
        if (motion_of(f) != DYNAMIC || sleeping_of(f)) continue;
        float4 v4 = w.linvel[i];
        float4 av4 = w.angvel[i];
        float4 ii = w.inv_inertia[i];
        float4 mat = w.material[i];
        float4 damp = w.damping[i];
        float4 fo = w.force[i];
        float4 to = w.torque[i];
        int dof = dof_of(f);
        float gs = c_settings.gravity_enabled ? mat.z : 0.f;
        float3 v = xyz(v4);
        v.x += (fo.x * ii.w + c_settings.gravity[0] * gs) * dt;
        v.y += (fo.y * ii.w + c_settings.gravity[1] * gs) * dt;
        v.z += (fo.z * ii.w + c_settings.gravity[2] * gs) * dt;
        float ldf = fmaxf(0.f, 1.f - damp.x * dt);
        v = v * ldf;
        float ls = lensq3(v);
        if (ls > damp.z * damp.z) v = v * (damp.z / sqrtf(ls));
        if (!(dof & 1)) v.x = 0.f;
        if (!(dof & 2)) v.y = 0.f;
        if (!(dof & 4)) v.z = 0.f;
        float3 av = xyz(av4);
        if (to.x != 0.f || to.y != 0.f || to.z != 0.f) {
            Sym3 I = world_inv_inertia(w.quat[i], w.inertia_rot[i], xyz(ii), dof);
            av = av + symmul(I, xyz(to)) * dt;
        }
        float adf = fmaxf(0.f, 1.f - damp.y * dt);
        av = av * adf;
        float as = lensq3(av);
        if (as > damp.w * damp.w) av = av * (damp.w / sqrtf(as));
        if (!(dof & 8)) av.x = 0.f;
        if (!(dof & 16)) av.y = 0.f;
        if (!(dof & 32)) av.z = 0.f;
        w.linvel[i] = make_float4(v.x, v.y, v.z, v4.w);
        w.angvel[i] = make_float4(av.x, av.y, av.z, av4.w);
    }
}

// ---------------------------------------------------------------------------
// exact FP64 bounds: mat4.fromQuat then the 8 rotated corners of the shape
// bounds plus the position, in the reference's operation order with every
// operation rounded separately (no fused multiply-add).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

__device__ void exact_aabb(float4 p4, float4 q4, const double lo[3], const double hi[3], double out[6]) {
    double x = q4.x, y = q4.y, z = q4.z, ww = q4.w;
    double x2 = da(x, x), y2 = da(y, y), z2 = da(z, z);
    double xx = dm(x, x2), yx = dm(y, x2), yy = dm(y, y2), zx = dm(z, x2), zy = dm(z, y2), zz = dm(z, z2);
    double wx = dm(ww, x2), wy = dm(ww, y2), wz = dm(ww, z2);
    double m0 = ds(ds(1.0, yy), zz), m1 = da(yx, wz), m2 = ds(zx, wy);
    double m4 = ds(yx, wz), m5 = ds(ds(1.0, xx), zz), m6 = da(zy, wx);
    double m8 = da(zx, wy), m9 = ds(zy, wx), m10 = ds(ds(1.0, xx), yy);
    double px = p4.x, py = p4.y, pz = p4.z;
    double xs[2] = {lo[0], hi[0]}, ys[2] = {lo[1], hi[1]}, zs[2] = {lo[2], hi[2]};
    double mnx = 0, mny = 0, mnz = 0, mxx = 0, mxy = 0, mxz = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        double cx = xs[c & 1], cy = ys[(c >> 1) & 1], cz = zs[(c >> 2) & 1];
        double wxv = da(da(da(dm(m0, cx), dm(m4, cy)), dm(m8, cz)), px);
        double wyv = da(da(da(dm(m1, cx), dm(m5, cy)), dm(m9, cz)), py);
        double wzv = da(da(da(dm(m2, cx), dm(m6, cy)), dm(m10, cz)), pz);
        if (c == 0) {
            mnx = mxx = wxv;
            mny = mxy = wyv;
            mnz = mxz = wzv;
        } else {
            mnx = fmin(mnx, wxv);
            mny = fmin(mny, wyv);
            mnz = fmin(mnz, wzv);
            mxx = fmax(mxx, wxv);
            mxy = fmax(mxy, wyv);
            mxz = fmax(mxz, wzv);
        }
    }
    out[0] = mnx;
    out[1] = mny;
    out[2] = mnz;
    out[3] = mxx;
    out[4] = mxy;
    out[5] = mxz;
}

// local bounds of the shape in FP64 (box.ts:77-84, sphere.ts, capsule.ts:84-94)
__device__ __forceinline__ void shape_bounds(const DevWorld &w, int i, uint32_t f, float4 sp, double lo[3],
                                             double hi[3]) {
    if (f & F_DECORATED) {  // the decorated shape's bounds (computeTransformedLocalBounds transformed.ts)
        const DevFrame &d = w.frames[i];
        for (int k = 0; k < 3; k++) {
            lo[k] = d.lo[k];
            hi[k] = d.hi[k];
        }
        return;
    }
    int s = shape_of(f);
    if (s == SHAPE_MESH) {  // the mesh's root node bounds (triangle-mesh.ts:124-130)
        const DevMesh &m = w.meshes[mesh_of(sp)];
        lo[0] = m.lo.x;
        lo[1] = m.lo.y;
        lo[2] = m.lo.z;
        hi[0] = m.hi.x;
        hi[1] = m.hi.y;
        hi[2] = m.hi.z;
        return;
    }
    if (s == SHAPE_HULL) {  // the hull's local bounds (convex-hull.ts:214-231)
        const DevHull &h = w.hulls[hull_of(sp)];
        lo[0] = h.lo.x;
        lo[1] = h.lo.y;
        lo[2] = h.lo.z;
        hi[0] = h.hi.x;
        hi[1] = h.hi.y;
        hi[2] = h.hi.z;
        return;
    }
    double ex, ey, ez;
    if (s == SHAPE_BOX) {
        ex = sp.x;
        ey = sp.y;
        ez = sp.z;
    } else if (s == SHAPE_CAPSULE) {
        ex = ez = sp.x;
        ey = da((double)sp.y, (double)sp.x);  // half height + radius
    } else if (s == SHAPE_CYLINDER) {  // cylinder.ts calculateAABB
        ex = ez = sp.y;
        ey = sp.x;
    } else {
        ex = ey = ez = sp.x;
    }
    lo[0] = -ex;
    lo[1] = -ey;
    lo[2] = -ez;
    hi[0] = ex;
    hi[1] = ey;
    hi[2] = ez;
}

__device__ __forceinline__ unsigned int f2ord(float f) {
    unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned int u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounds for every body + scene bounds of AABB centres (ordered-int atomics)
__global__ void k_update_bounds(DevWorld w, unsigned int *scene) {
    float3 cmin = f3(3.0e38f, 3.0e38f, 3.0e38f), cmax = f3(-3.0e38f, -3.0e38f, -3.0e38f);
    int awake = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        uint32_t f = w.flags[i];
        if (motion_of(f) != STATIC && !sleeping_of(f)) awake++;
        double lo[3], hi[3];
        shape_bounds(w, i, f, w.shape[i], lo, hi);
        double b[6];
        exact_aabb(w.pos[i], w.quat[i], lo, hi, b);
        double *o = w.aabb64 + (size_t)i * 6;
        o[0] = b[0];
        o[1] = b[1];
        o[2] = b[2];
        o[3] = b[3];
        o[4] = b[4];
        o[5] = b[5];
        float3 l = f3(__double2float_rd(b[0]), __double2float_rd(b[1]), __double2float_rd(b[2]));
        float3 h = f3(__double2float_ru(b[3]), __double2float_ru(b[4]), __double2float_ru(b[5]));
        w.aabb_lo[i] = make_float4(l.x, l.y, l.z, 0.f);
        w.aabb_hi[i] = make_float4(h.x, h.y, h.z, 0.f);
        float3 c = (l + h) * 0.5f;
        cmin = f3(fminf(cmin.x, c.x), fminf(cmin.y, c.y), fminf(cmin.z, c.z));
        cmax = f3(fmaxf(cmax.x, c.x), fmaxf(cmax.y, c.y), fmaxf(cmax.z, c.z));
    }
    // warp reduce then one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        cmin.x = fminf(cmin.x, __shfl_xor_sync(0xffffffffu, cmin.x, o));
        cmin.y = fminf(cmin.y, __shfl_xor_sync(0xffffffffu, cmin.y, o));
        cmin.z = fminf(cmin.z, __shfl_xor_sync(0xffffffffu, cmin.z, o));
        cmax.x = fmaxf(cmax.x, __shfl_xor_sync(0xffffffffu, cmax.x, o));
        cmax.y = fmaxf(cmax.y, __shfl_xor_sync(0xffffffffu, cmax.y, o));
        cmax.z = fmaxf(cmax.z, __shfl_xor_sync(0xffffffffu, cmax.z, o));
    }
    for (int o = 16; o > 0; o >>= 1) awake += __shfl_xor_sync(0xffffffffu, awake, o);
    if ((threadIdx.x & 31) == 0) {
        if (awake) atomicAdd(&w.ctr->num_awake, awake);
        atomicMin(&scene[0], f2ord(cmin.x));
        atomicMin(&scene[1], f2ord(cmin.y));
        atomicMin(&scene[2], f2ord(cmin.z));
        atomicMax(&scene[3], f2ord(cmax.x));
        atomicMax(&scene[4], f2ord(cmax.y));
        atomicMax(&scene[5], f2ord(cmax.z));
    }
}

__device__ __forceinline__ unsigned int expand_bits10(unsigned int v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(DevWorld w, const unsigned int *scene) {
    float3 smin = f3(ord2f(scene[0]), ord2f(scene[1]), ord2f(scene[2]));
    float3 smax = f3(ord2f(scene[3]), ord2f(scene[4]), ord2f(scene[5]));
    float3 ext = smax - smin;
    float3 inv = f3(ext.x > 0.f ? 1023.f / ext.x : 0.f, ext.y > 0.f ? 1023.f / ext.y : 0.f,
                    ext.z > 0.f ? 1023.f / ext.z : 0.f);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        float3 c = (xyz(w.aabb_lo[i]) + xyz(w.aabb_hi[i])) * 0.5f;
        float3 t = (c - smin);
        unsigned int qx = (unsigned int)fminf(fmaxf(t.x * inv.x, 0.f), 1023.f);
        unsigned int qy = (unsigned int)fminf(fmaxf(t.y * inv.y, 0.f), 1023.f);
        unsigned int qz = (unsigned int)fminf(fmaxf(t.z * inv.z, 0.f), 1023.f);
        unsigned int m = (expand_bits10(qx) << 2) | (expand_bits10(qy) << 1) | expand_bits10(qz);
        w.morton[i] = ((unsigned long long)(unsigned int)w.world[i] << 30) | m;
        w.order[i] = i;
    }
}

// ---------------------------------------------------------------------------
// Karras (2012) LBVH construction over the sorted keys
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lcp(const unsigned long long *k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll(a ^ b);
}

__global__ void k_lbvh_build(DevWorld w, int2 *node_world) {
    int n = w.n;
    const unsigned long long *k = w.morton;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        int d = (lcp(k, n, i, i + 1) - lcp(k, n, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = lcp(k, n, i, i - d);
        int lmax = 2;
        while (lcp(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (lcp(k, n, i, i + (l + t) * d) > dmin) l += t;
        int j = i + l * d;
        int dnode = lcp(k, n, i, j);
        int s = 0;
        int div = 2;
        for (int t = (l + div - 1) / div; t >= 1; div <<= 1, t = (l + div - 1) / div) {
            if (lcp(k, n, i, i + (s + t) * d) > dnode) s += t;
            if (t == 1) break;
        }
        int gamma = i + s * d + min(d, 0);
        int first = min(i, j), last = max(i, j);
        int left = (first == gamma) ? (n - 1 + gamma) : gamma;
        int right = (last == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
        w.node_child[i] = make_int2(left, right);
        w.node_parent[left] = i;
        w.node_parent[right] = i;
        w.node_flag[i] = 0;
        node_world[i] = make_int2((int)(k[first] >> 30), (int)(k[last] >> 30));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) w.node_parent[n == 1 ? 0 : 0] = -1;
}

__global__ void k_lbvh_refit(DevWorld w, int2 *node_world, const int *gate) {
    if (gate && *gate == 0) return;
    int n = w.n;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int body = w.order[j];
        int node = n - 1 + j;
        w.node_lo[node] = w.aabb_lo[body];
        w.node_hi[node] = w.aabb_hi[body];
        int wd = w.world[body];
        node_world[node] = make_int2(wd, wd);
        if (n == 1) continue;
        __threadfence();
        int p = w.node_parent[node];
        while (p >= 0) {
            if (atomicAdd(&w.node_flag[p], 1) == 0) break;  // first child to arrive stops
            __threadfence();
            int2 c = w.node_child[p];
            float4 l0 = __ldcg(&w.node_lo[c.x]), h0 = __ldcg(&w.node_hi[c.x]);
            float4 l1 = __ldcg(&w.node_lo[c.y]), h1 = __ldcg(&w.node_hi[c.y]);
            w.node_lo[p] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.f);
            w.node_hi[p] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.f);
            __threadfence();
            p = w.node_parent[p];
        }
    }
}

// ---------------------------------------------------------------------------
// pair finding: one querying body per thread, stack traversal, FP64 re-test
// ---------------------------------------------------------------------------
constexpr int PAIR_BUF = 16;
constexpr int STACK_DEPTH = 64;

__device__ __forceinline__ bool overlap_f(float4 al, float4 ah, float3 bl, float3 bh) {
    return !(ah.x < bl.x || al.x > bh.x || ah.y < bl.y || al.y > bh.y || ah.z < bl.z || al.z > bh.z);
}

__device__ void flush_pairs(DevWorld &w, int2 *buf, int cnt) {
    if (cnt == 0) return;
    int base = atomicAdd(&w.ctr->num_pairs, cnt);
    for (int k = 0; k < cnt; k++) {
        int idx = base + k;
        if (idx < w.max_pairs)
            w.pairs[idx] = buf[k];
        else
            atomicOr(&w.ctr->overflow, OVF_PAIRS);
    }
}

__global__ void __launch_bounds__(128) k_find_pairs(DevWorld w, const int2 *node_world) {
    int n = w.n;
    int nthreads = gridDim.x * blockDim.x;
    int iters = (n + nthreads - 1) / nthreads;
    for (int it = 0; it < iters; it++) {
        // query bodies in the tree's leaf (Morton) order: the lanes of a warp walk neighbouring
        // subtrees.  Pairs are appended, so the order changes no result.
        const int q = it * nthreads + blockIdx.x * blockDim.x + threadIdx.x;
        const int i = q < n ? w.order[q] : n;
        int2 buf[PAIR_BUF];
        int cnt = 0;
        uint32_t fa = i < n ? w.flags[i] : 0u;
        bool query = i < n && motion_of(fa) != STATIC && !sleeping_of(fa);
        if (query) {
            const double *a64 = w.aabb64 + (size_t)i * 6;
            double e[6];
            double sd = c_spec_dist64;
            e[0] = ds(a64[0], sd);
            e[1] = ds(a64[1], sd);
            e[2] = ds(a64[2], sd);
            e[3] = da(a64[3], sd);
            e[4] = da(a64[4], sd);
            e[5] = da(a64[5], sd);
            float3 ql = f3(__double2float_rd(e[0]), __double2float_rd(e[1]), __double2float_rd(e[2]));
            float3 qh = f3(__double2float_ru(e[3]), __double2float_ru(e[4]), __double2float_ru(e[5]));
            int wa = w.world[i];
            int la = layer_of(fa);
            uint32_t allowed = c_settings.allowed_pairs[la];
            uint2 ga = w.groups[i];
            int amotion = motion_of(fa);
            int stack[STACK_DEPTH];
            int sp = 0;
            stack[sp++] = 0;  // root (leaf 0 when n == 1)
            while (sp > 0) {
                int node = stack[--sp];
                int2 nw = node_world[node];
                if (wa < nw.x || wa > nw.y) continue;
                if (!overlap_f(w.node_lo[node], w.node_hi[node], ql, qh)) continue;
                if (node < n - 1) {
                    int2 c = w.node_child[node];
                    if (sp + 2 <= STACK_DEPTH) {
                        stack[sp++] = c.y;
                        stack[sp++] = c.x;
                    } else {
                        atomicOr(&w.ctr->overflow, OVF_SLOTS);
                    }
                    continue;
                }
                int b = w.order[node - (n - 1)];
                if (b == i) continue;
                uint32_t fb = w.flags[b];
                if (!(allowed & (1u << layer_of(fb)))) continue;
                uint2 gb = w.groups[b];
                if (!((ga.x & gb.y) != 0u && (gb.x & ga.y) != 0u)) continue;
                const double *b64 = w.aabb64 + (size_t)b * 6;
                if (b64[3] < e[0] || b64[0] > e[3] || b64[4] < e[1] || b64[1] > e[4] || b64[5] < e[2] ||
                    b64[2] > e[5])
                    continue;
                int bmotion = motion_of(fb);
                bool bquery = bmotion != STATIC && !sleeping_of(fb);
                if (bquery && b <= i) continue;  // deduplication by body index
                if (!(fa & F_KIN_VS_NONDYN) && !(fb & F_KIN_VS_NONDYN) && amotion != DYNAMIC && bmotion != DYNAMIC &&
                    !(amotion == KINEMATIC && (fb & F_SENSOR)) && !(bmotion == KINEMATIC && (fa & F_SENSOR)))
                    continue;
                // bodies that share an enabled joint: the declarative form of an onBodyPairValidate
                // that rejects them (broadphase.ts:112-123)
                if (w.skip_joint_pairs) {
                    const int *jp = w.joint_partners + (size_t)i * JOINT_PARTNERS;
                    bool joined = false;
                    for (int k = 0; k < JOINT_PARTNERS; k++) joined |= jp[k] == b;
                    if (joined) continue;
                }
                if (cnt == PAIR_BUF) {
                    flush_pairs(w, buf, cnt);
                    cnt = 0;
                }
                buf[cnt++] = make_int2(i, b);
            }
        }
        // warp-aggregated reservation for what is left in the buffers (every lane of the
        // warp runs the same number of outer iterations, so the whole warp is here)
        __syncwarp();
        const unsigned mask = 0xffffffffu;
        int lane = threadIdx.x & 31;
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(mask, incl, o);
            if (lane >= o) incl += t;
        }
        int total = __shfl_sync(mask, incl, 31);
        int base = 0;
        if (lane == 31 && total > 0) base = atomicAdd(&w.ctr->num_pairs, total);
        base = __shfl_sync(mask, base, 31);
        int off = base + incl - cnt;
        for (int k = 0; k < cnt; k++) {
            int idx = off + k;
            if (idx < w.max_pairs)
                w.pairs[idx] = buf[k];
            else
                atomicOr(&w.ctr->overflow, OVF_PAIRS);
        }
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
__global__ void k_reset_scene(unsigned int *scene) {
    if (threadIdx.x < 3) scene[threadIdx.x] = 0xffffffffu;
    else if (threadIdx.x < 6) scene[threadIdx.x] = 0u;
}

void launch_integrate_forces(DevWorld &w, float dt, cudaStream_t s) {
    k_integrate_forces<<<grid_for(w.n, 256), 256, 0, s>>>(w, dt);
}

// Continuous collision, after the velocity integration: every body's bounds where the step
// has put it so far (updatePositionFromCenterOfMass + updateAABB rigid-body.ts:545-674 for the
// bodies that moved, the cast bodies still at their old position with the new rotation), the
// record of each cast body (update.ts:940-962) and its world's record count.
__global__ void k_ccd_prepare(DevWorld w, float dt) {
    if (w.ctr->num_ccd == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
        uint32_t f = w.flags[i];
        const bool cast = w.ccd_flag[i] != 0;
        const float4 sp = w.shape[i];
        if (motion_of(f) != STATIC && !sleeping_of(f) && !cast) {
            float3 p = xyz(w.com[i]) - qrot(w.quat[i], shape_com(w, i, f, sp));
            w.pos[i] = make_float4(p.x, p.y, p.z, 0.f);
        }
        double lo[3], hi[3], b[6];
        shape_bounds(w, i, f, sp, lo, hi);
        exact_aabb(w.pos[i], w.quat[i], lo, hi, b);
        double *o = w.aabb64 + (size_t)i * 6;
        for (int k = 0; k < 6; k++) o[k] = b[k];
        w.aabb_lo[i] = make_float4(__double2float_rd(b[0]), __double2float_rd(b[1]), __double2float_rd(b[2]), 0.f);
        w.aabb_hi[i] = make_float4(__double2float_ru(b[3]), __double2float_ru(b[4]), __double2float_ru(b[5]), 0.f);
        w.ccd_index[i] = cast ? w.ccd_slot[i] : -1;
        if (!cast) continue;
        const float inner = shape_inner_radius(w, i, f, sp);
        const float thr = c_settings.ccd_threshold * inner;
        const float3 d = xyz(w.linvel[i]) * dt;
        CcdRec r;
        r.delta = make_float4(d.x, d.y, d.z, thr * thr);
        r.normal = make_float4(0.f, 0.f, 0.f, fminf(c_settings.slop, c_settings.ccd_max_penetration * inner));
        r.point = make_float4(0.f, 0.f, 0.f, 1.f);
        r.fps = 1.f;
        r.friction = r.restitution = 0.f;
        r.body = i;
        r.hit = -1;
        r.slot = 0;
        r.pad[0] = r.pad[1] = 0;
        w.ccd[w.ccd_slot[i]] = r;
        atomicAdd(&w.ccd_world_fill[w.world[i]], 1);
    }
}

void launch_ccd_bounds(DevWorld &w, float dt, cudaStream_t s) {
    int n = w.n;
    k_ccd_prepare<<<grid_for(n, 256), 256, 0, s>>>(w, dt);
    if (n > 1) cudaMemsetAsync(w.node_flag, 0, sizeof(int) * (size_t)(n - 1), s);
    k_lbvh_refit<<<grid_for(n, 256), 256, 0, s>>>(w, w.node_world, &w.ctr->num_ccd);
}

void launch_broadphase(DevWorld &w, cudaStream_t s) {
    int n = w.n;
    k_reset_scene<<<1, 32, 0, s>>>(w.scene);
    k_update_bounds<<<grid_for(n, 256), 256, 0, s>>>(w, w.scene);
    k_morton<<<grid_for(n, 256), 256, 0, s>>>(w, w.scene);
    int wbits = 0;
    while ((1 << wbits) < w.num_worlds) wbits++;
    radix_sort_pairs_u64(w.morton, w.morton_alt, w.order, w.order_alt, n, 30 + wbits, w.scan_tmp, s);
    if (n > 1) k_lbvh_build<<<grid_for(n - 1, 256), 256, 0, s>>>(w, w.node_world);
    k_lbvh_refit<<<grid_for(n, 256), 256, 0, s>>>(w, w.node_world, nullptr);
    k_find_pairs<<<grid_for(n, 128, 16), 128, 0, s>>>(w, w.node_world);
}

// ray sort keys: the ray's world above the Morton code of its origin in the bodies' centre bounds
// (origins outside are clamped to the bounds' faces)
__global__ void k_ray_keys(const DevRay *rays, int nr, const unsigned int *scene, unsigned long long *keys, int *idx) {
    float3 smin = f3(ord2f(scene[0]), ord2f(scene[1]), ord2f(scene[2]));
    float3 smax = f3(ord2f(scene[3]), ord2f(scene[4]), ord2f(scene[5]));
    float3 ext = smax - smin;
    float3 inv = f3(ext.x > 0.f ? 1023.f / ext.x : 0.f, ext.y > 0.f ? 1023.f / ext.y : 0.f,
                    ext.z > 0.f ? 1023.f / ext.z : 0.f);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nr; i += gridDim.x * blockDim.x) {
        const DevRay r = rays[i];
        float3 t = f3(r.origin[0], r.origin[1], r.origin[2]) - smin;
        unsigned int qx = (unsigned int)fminf(fmaxf(t.x * inv.x, 0.f), 1023.f);
        unsigned int qy = (unsigned int)fminf(fmaxf(t.y * inv.y, 0.f), 1023.f);
        unsigned int qz = (unsigned int)fminf(fmaxf(t.z * inv.z, 0.f), 1023.f);
        unsigned int m = (expand_bits10(qx) << 2) | (expand_bits10(qy) << 1) | expand_bits10(qz);
        const unsigned int wd = r.world < 0 ? 0u : (unsigned int)r.world;
        keys[i] = ((unsigned long long)wd << 30) | m;
        idx[i] = i;
    }
}

void launch_ray_order(DevWorld &w, const DevRay *rays, int nr, unsigned long long *keys, int *idx, int *tmp,
                      cudaStream_t s) {
    k_ray_keys<<<grid_for(nr, 256), 256, 0, s>>>(rays, nr, w.scene, keys, idx);
    int wbits = 0;
    while ((1 << wbits) < w.num_worlds) wbits++;
    radix_sort_pairs_u64(keys, keys + nr, idx, idx + nr, nr, 30 + wbits, tmp, s, nullptr);
}

// the broadphase without its pair search: current boxes, Morton order and tree
void launch_query_tree(DevWorld &w, cudaStream_t s) {
    int n = w.n;
    if (n == 0) return;
    k_reset_scene<<<1, 32, 0, s>>>(w.scene);
    k_update_bounds<<<grid_for(n, 256), 256, 0, s>>>(w, w.scene);
    k_morton<<<grid_for(n, 256), 256, 0, s>>>(w, w.scene);
    int wbits = 0;
    while ((1 << wbits) < w.num_worlds) wbits++;
    radix_sort_pairs_u64(w.morton, w.morton_alt, w.order, w.order_alt, n, 30 + wbits, w.scan_tmp, s);
    if (n > 1) k_lbvh_build<<<grid_for(n - 1, 256), 256, 0, s>>>(w, w.node_world);
    k_lbvh_refit<<<grid_for(n, 256), 256, 0, s>>>(w, w.node_world, nullptr);
}

}  // namespace cc
