// Frozen-contact replay of a rollout's velocity solves, in FP64 or in FP64 dual numbers.
//
// TEST INFRASTRUCTURE ONLY (the oracle): it checks the GPU adjoint
// (cc_world_rollout_grad), never stands in for it.
//
// A "tape" holds, for every step of a rollout, the rows the step's velocity solve
// started from: the contact constraints as addContactConstraint built them
// (contact-constraints.ts:437-857: normal, tangents, moment arms, effective masses,
// velocity biases, the warm-start impulses read from the contact cache and the cached
// point each one matched), the body velocities after the force integration and the
// world inverse inertias at the step's orientation.  The replay holds those rows fixed
// and re-runs, with its own body velocities and impulses:
//   - the force integration as the linear map it is for a fixed step
//     (accelerationIntegrationUpdate update.ts:245-319: damping factors, DOF masks);
//   - the warm start (warmStartVelocityConstraints contact-constraints.ts:906-955,
//     AxisConstraintPart.warmStart axis-constraint-part.ts:500-537), its impulses
//     handed from the previous step's final impulses through the cache match
//     (contact-constraints.ts:651-686);
//   - the velocity iterations (solveVelocityConstraintsForIsland
//     contact-constraints.ts:963-1053: friction projected onto the disc of radius
//     mu * lambda_n, then the non-negative normal row; getTotalLambda / applyLambda
//     axis-constraint-part.ts:578-707), contacts in sortContactIndices order
//     (contact-constraints.ts:1240-1264);
//   - the friction combine (combine-material.ts:40-57) when friction coefficients move;
//   - the translation x += v dt of velocityIntegrationUpdate (update.ts:896-976).
// The position-solve corrections and the contact geometry are constants of each step,
// which is the model cc_world_rollout_grad differentiates.
//
// The scalar type S is double or Dual (value + one directional derivative), so one
// pass gives a loss and its derivative along a direction of the initial linear and
// angular velocities and friction coefficients: the FP64 dual-number check of the
// adjoint.  The arithmetic follows the oracle's own solver functions (oracle.cpp
// warm_start / total_lambda / apply_lambda / solve_velocity) operation for operation,
// so a replay of the oracle's own tape reproduces its solver bit for bit.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <numeric>
#include <utility>
#include <vector>

namespace orc_frozen {

// ---------------------------------------------------------------------------
// forward-mode dual number: v + d eps, eps^2 = 0
// ---------------------------------------------------------------------------
struct Dual {
    double v = 0, d = 0;
    Dual() = default;
    Dual(double x) : v(x), d(0) {}  // NOLINT: constants promote
    Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline Dual &operator+=(Dual &a, Dual b) { return a = a + b; }
inline Dual &operator-=(Dual &a, Dual b) { return a = a - b; }
inline Dual &operator*=(Dual &a, Dual b) { return a = a * b; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator==(Dual a, double b) { return a.v == b; }
inline bool operator!=(Dual a, double b) { return a.v != b; }
// an impulse is skipped only when neither its value nor its derivative moves anything
inline bool is_zero(Dual a) { return a.v == 0 && a.d == 0; }
inline bool is_zero(double a) { return a == 0; }
inline Dual sqrt_s(Dual a) {
    double r = std::sqrt(a.v);
    return {r, r > 0 ? a.d / (2 * r) : 0.0};
}
inline double sqrt_s(double a) { return std::sqrt(a); }
inline double value(double a) { return a; }
inline double value(Dual a) { return a.v; }
inline double deriv(double) { return 0; }
inline double deriv(Dual a) { return a.d; }
inline Dual max_s(Dual a, Dual b) { return a.v >= b.v ? a : b; }  // std::max(a, b) keeps a on ties
inline double max_s(double a, double b) { return std::max(a, b); }
inline Dual min_s(Dual a, Dual b) { return b.v < a.v ? b : a; }  // std::min(a, b) keeps a on ties
inline double min_s(double a, double b) { return std::min(a, b); }
template <class S>
inline S with_value(S x, double v);
template <>
inline double with_value(double, double v) { return v; }
template <>
inline Dual with_value(Dual x, double v) { return {v, x.d}; }

template <class S>
struct V3s {
    S x, y, z;
};

// ---------------------------------------------------------------------------
// tape layout (rows of doubles, as the Python harness packs them)
// ---------------------------------------------------------------------------
constexpr int BODY_ROW = 17;     // v1[3] w1[3] inverse inertia (3x3 column-major)[9] inv_mass flags
constexpr int CONST_ROW = 6;     // world, in_loss, friction, friction combine mode, ldf, adf
constexpr int CON_HEAD = 18;     // a b n island has_prev sort_key normal[3] t1[3] t2[3] friction imA imB
constexpr int POINT_ROW = 17;    // rA[3] rB[3] eff_n eff_t1 eff_t2 bias lam_n lam_t1 lam_t2 prev final_n final_t1 final_t2
constexpr int CON_ROW = CON_HEAD + 4 * POINT_ROW;
enum : int { T_DYNAMIC = 1, T_MOVING = 2 };

struct Tape {
    int n = 0, steps = 0, worlds = 0, iters = 0;
    double dt = 0;
    const double *consts = nullptr;   // n x CONST_ROW
    const double *bodies = nullptr;   // steps x n x BODY_ROW
    const double *v0 = nullptr;       // steps x n x 6: velocities at the start of each step
    const double *ratio = nullptr;    // steps
    const int *con_off = nullptr;     // steps + 1
    const double *cons = nullptr;     // con_off[steps] x CON_ROW
    const double *x_final = nullptr;  // n x 3: positions after the last step
    const double *targets = nullptr;  // worlds x 3
};

// combine-material.ts:40-57 (the oracle's combine, generic in the scalar)
template <class S>
S combine_s(S a, S b, int ma, int mb) {
    static const int prio[5] = {0, 1, 3, 4, 2};  // AVERAGE, MULTIPLY, MIN, MAX, GEOMETRIC_MEAN
    int mode = prio[ma] >= prio[mb] ? ma : mb;
    switch (mode) {
        case 1:
            return a * b;
        case 2:
            return min_s(a, b);
        case 3:
            return max_s(a, b);
        case 4:
            return sqrt_s(a * b);
        default:
            return (a + b) / S(2.0);
    }
}

template <class S>
struct Part {  // AxisPart with the rows of one point along one axis
    V3s<double> r1xa, r2xa, invI1, invI2;
    double effMass = 0, bias = 0;
    S totalLambda = S(0.0);
};
template <class S>
struct Con {
    int a, b, n;
    uint32_t key;
    bool has_prev;
    V3s<double> ax[3];  // normal, t1, t2
    S friction;
    double imA, imB;
    Part<S> p[4][3];    // [point][normal, t1, t2]
    int prev[4];
};

template <class S>
struct Replay {
    const Tape &T;
    int mode;  // 0: real parts from the tape each step (linearised at the tape); 1: own trajectory
    std::vector<V3s<S>> v, w;  // carried body velocities
    std::vector<V3s<S>> vsum;  // sum over steps of the post-solve linear velocity
    std::vector<S> mu;
    std::vector<std::vector<Con<S>>> cons;  // per step (kept for the impulse hand-off)
    double *v2_out = nullptr;               // optional: steps x n x 6 real post-solve velocities
    double *lam_out = nullptr;              // optional: total contacts x 4 x 3 real final impulses

    explicit Replay(const Tape &t, int m) : T(t), mode(m) {}

    const double *brow(int k, int i) const { return T.bodies + ((size_t)k * T.n + i) * BODY_ROW; }
    int flags(int k, int i) const { return (int)brow(k, i)[16]; }

    static void dof_lin(V3s<S> &v, int dof) {  // apply_dof_lin
        int t = dof & 7;
        if (!(t & 1)) v.x = S(0.0);
        if (!(t & 2)) v.y = S(0.0);
        if (!(t & 4)) v.z = S(0.0);
    }

    // AxisConstraintPart.warmStart axis-constraint-part.ts:500-537
    void warm_start(Part<S> &p, int a, int b, bool dA, bool dB, double imA, double imB, const V3s<double> &ax,
                    double ratio, int dofA, int dofB) {
        p.totalLambda = p.totalLambda * S(ratio);
        if (is_zero(p.totalLambda)) return;
        if (dA) {
            S l = p.totalLambda * S(imA);
            v[a] = {v[a].x - S(ax.x) * l, v[a].y - S(ax.y) * l, v[a].z - S(ax.z) * l};
            dof_lin(v[a], dofA);
            w[a] = {w[a].x - S(p.invI1.x) * p.totalLambda, w[a].y - S(p.invI1.y) * p.totalLambda,
                    w[a].z - S(p.invI1.z) * p.totalLambda};
        }
        if (dB) {
            S l = p.totalLambda * S(imB);
            v[b] = {v[b].x + S(ax.x) * l, v[b].y + S(ax.y) * l, v[b].z + S(ax.z) * l};
            dof_lin(v[b], dofB);
            w[b] = {w[b].x + S(p.invI2.x) * p.totalLambda, w[b].y + S(p.invI2.y) * p.totalLambda,
                    w[b].z + S(p.invI2.z) * p.totalLambda};
        }
    }
    // getTotalLambda axis-constraint-part.ts:578-625 (softness 0)
    S total_lambda(const Part<S> &p, int a, int b, bool mA, bool mB, const V3s<double> &ax) {
        S jv;
        if (mA && mB) {
            S dx = v[a].x - v[b].x, dy = v[a].y - v[b].y, dz = v[a].z - v[b].z;
            jv = S(ax.x) * dx + S(ax.y) * dy + S(ax.z) * dz;
        } else if (mA) {
            jv = S(ax.x) * v[a].x + S(ax.y) * v[a].y + S(ax.z) * v[a].z;
        } else if (mB) {
            jv = -(S(ax.x) * v[b].x + S(ax.y) * v[b].y + S(ax.z) * v[b].z);
        } else {
            jv = S(0.0);
        }
        if (mA) jv = jv + (S(p.r1xa.x) * w[a].x + S(p.r1xa.y) * w[a].y + S(p.r1xa.z) * w[a].z);
        if (mB) jv = jv - (S(p.r2xa.x) * w[b].x + S(p.r2xa.y) * w[b].y + S(p.r2xa.z) * w[b].z);
        S lambda = S(p.effMass) * (jv - (S(0.0) * p.totalLambda + S(p.bias)));
        return p.totalLambda + lambda;
    }
    // applyLambda axis-constraint-part.ts:640-707
    void apply_lambda(Part<S> &p, int a, int b, bool dA, bool dB, double imA, double imB, const V3s<double> &ax, S tl,
                      int dofA, int dofB) {
        S dl = tl - p.totalLambda;
        p.totalLambda = tl;
        if (is_zero(dl)) return;
        if (dA) {
            S ls = dl * S(imA);
            v[a].x -= S(ax.x) * ls;
            v[a].y -= S(ax.y) * ls;
            v[a].z -= S(ax.z) * ls;
            dof_lin(v[a], dofA);
            w[a].x -= S(p.invI1.x) * dl;
            w[a].y -= S(p.invI1.y) * dl;
            w[a].z -= S(p.invI1.z) * dl;
        }
        if (dB) {
            S ls = dl * S(imB);
            v[b].x += S(ax.x) * ls;
            v[b].y += S(ax.y) * ls;
            v[b].z += S(ax.z) * ls;
            dof_lin(v[b], dofB);
            w[b].x += S(p.invI2.x) * dl;
            w[b].y += S(p.invI2.y) * dl;
            w[b].z += S(p.invI2.z) * dl;
        }
    }

    // the rows of one point along one axis (inv_eff_mass oracle.cpp: crosses only for dynamic bodies)
    void make_part(Part<S> &p, const double *pt, const V3s<double> &ax, bool dA, bool dB, const double *IA,
                   const double *IB, double eff, double bias) {
        p.r1xa = p.r2xa = p.invI1 = p.invI2 = {0, 0, 0};
        if (dA) {
            V3s<double> r{pt[0], pt[1], pt[2]};
            V3s<double> c{r.y * ax.z - r.z * ax.y, r.z * ax.x - r.x * ax.z, r.x * ax.y - r.y * ax.x};
            p.r1xa = c;
            p.invI1 = {IA[0] * c.x + IA[3] * c.y + IA[6] * c.z, IA[1] * c.x + IA[4] * c.y + IA[7] * c.z,
                       IA[2] * c.x + IA[5] * c.y + IA[8] * c.z};
        }
        if (dB) {
            V3s<double> r{pt[3], pt[4], pt[5]};
            V3s<double> c{r.y * ax.z - r.z * ax.y, r.z * ax.x - r.x * ax.z, r.x * ax.y - r.y * ax.x};
            p.r2xa = c;
            p.invI2 = {IB[0] * c.x + IB[3] * c.y + IB[6] * c.z, IB[1] * c.x + IB[4] * c.y + IB[7] * c.z,
                       IB[2] * c.x + IB[5] * c.y + IB[8] * c.z};
        }
        p.effMass = eff;
        p.bias = bias;
    }

    // eps, dir: the initial perturbation (dual seed = dir in every mode)
    void run(double eps, const double *dv, const double *dw, const double *dmu) {
        const int n = T.n;
        v.assign(n, {});
        w.assign(n, {});
        vsum.assign(n, {S(0.0), S(0.0), S(0.0)});
        mu.assign(n, S(0.0));
        for (int i = 0; i < n; i++) {
            const double *v0 = T.v0 + (size_t)i * 6;
            auto seed = [&](double x, double d) {
                S s = S(x + (mode == 1 ? eps * d : 0.0));
                return with_value_seed(s, d);
            };
            v[i] = {seed(v0[0], dv ? dv[3 * i] : 0), seed(v0[1], dv ? dv[3 * i + 1] : 0),
                    seed(v0[2], dv ? dv[3 * i + 2] : 0)};
            w[i] = {seed(v0[3], dw ? dw[3 * i] : 0), seed(v0[4], dw ? dw[3 * i + 1] : 0),
                    seed(v0[5], dw ? dw[3 * i + 2] : 0)};
            const double *cst = T.consts + (size_t)i * CONST_ROW;
            mu[i] = with_value_seed(S(cst[2] + (mode == 1 && dmu ? eps * dmu[i] : 0.0)), dmu ? dmu[i] : 0.0);
        }
        cons.assign(T.steps, {});
        size_t lam_base = 0;
        for (int k = 0; k < T.steps; k++) {
            step(k);
            if (v2_out)
                for (int i = 0; i < n; i++) {
                    double *o = v2_out + ((size_t)k * n + i) * 6;
                    o[0] = value(v[i].x), o[1] = value(v[i].y), o[2] = value(v[i].z);
                    o[3] = value(w[i].x), o[4] = value(w[i].y), o[5] = value(w[i].z);
                }
            if (lam_out)
                for (size_t c = 0; c < cons[k].size(); c++)
                    for (int q = 0; q < 4; q++)
                        for (int r = 0; r < 3; r++)
                            lam_out[(lam_base + c) * 12 + q * 3 + r] = value(cons[k][c].p[q][r].totalLambda);
            lam_base += cons[k].size();
            if (k >= 2) cons[k - 2].clear();  // only the previous step's impulses are handed on
        }
    }
    static S with_value_seed(S s, double d);

    void step(int k) {
        const int n = T.n;
        const double ratio = T.ratio[k];
        // force integration around the tape: v1 = v1_tape + L (v0 - v0_tape)
        for (int i = 0; i < n; i++) {
            const double *b = brow(k, i);
            const int f = (int)b[16];
            const double *v0t = T.v0 + ((size_t)k * n + i) * 6;
            if (f & T_DYNAMIC) {
                const double *cst = T.consts + (size_t)i * CONST_ROW;
                const double ldf = cst[4], adf = cst[5];
                const int dof = (f >> 8) & 63;
                S lx = (dof & 1) ? S(ldf) * (v[i].x - S(v0t[0])) : S(0.0);
                S ly = (dof & 2) ? S(ldf) * (v[i].y - S(v0t[1])) : S(0.0);
                S lz = (dof & 4) ? S(ldf) * (v[i].z - S(v0t[2])) : S(0.0);
                S ax = (dof & 8) ? S(adf) * (w[i].x - S(v0t[3])) : S(0.0);
                S ay = (dof & 16) ? S(adf) * (w[i].y - S(v0t[4])) : S(0.0);
                S az = (dof & 32) ? S(adf) * (w[i].z - S(v0t[5])) : S(0.0);
                if (mode == 0) {  // the real parts are the tape's
                    v[i] = {with_value(lx, b[0]), with_value(ly, b[1]), with_value(lz, b[2])};
                    w[i] = {with_value(ax, b[3]), with_value(ay, b[4]), with_value(az, b[5])};
                } else {
                    v[i] = {S(b[0]) + lx, S(b[1]) + ly, S(b[2]) + lz};
                    w[i] = {S(b[3]) + ax, S(b[4]) + ay, S(b[5]) + az};
                }
            } else {  // static, kinematic or sleeping: the tape's velocities, constants of the step
                v[i] = {S(b[0]), S(b[1]), S(b[2])};
                w[i] = {S(b[3]), S(b[4]), S(b[5])};
            }
        }
        // the step's constraints, their warm-start impulses handed on from the previous step
        const int c0 = T.con_off[k], c1 = T.con_off[k + 1];
        std::vector<Con<S>> &cs = cons[k];
        cs.resize(c1 - c0);
        std::map<std::pair<int, int>, int> prev_of;
        if (k > 0)
            for (size_t j = 0; j < cons[k - 1].size(); j++) prev_of[{cons[k - 1][j].a, cons[k - 1][j].b}] = (int)j;
        for (int ci = c0; ci < c1; ci++) {
            const double *r = T.cons + (size_t)ci * CON_ROW;
            Con<S> &c = cs[ci - c0];
            c.a = (int)r[0];
            c.b = (int)r[1];
            c.n = (int)r[2];
            c.has_prev = r[4] != 0;
            c.key = (uint32_t)r[5];
            for (int x = 0; x < 3; x++) c.ax[x] = {r[6 + 3 * x], r[7 + 3 * x], r[8 + 3 * x]};
            const double *ca = T.consts + (size_t)c.a * CONST_ROW, *cb = T.consts + (size_t)c.b * CONST_ROW;
            S fr = combine_s(mu[c.a], mu[c.b], (int)ca[3], (int)cb[3]);
            c.friction = mode == 0 ? with_value(fr, r[15]) : fr;
            c.imA = r[16];
            c.imB = r[17];
            const int fa = flags(k, c.a), fb = flags(k, c.b);
            const bool dA = fa & T_DYNAMIC, dB = fb & T_DYNAMIC;
            const double *IA = brow(k, c.a) + 6, *IB = brow(k, c.b) + 6;
            const Con<S> *pc = nullptr;
            if (k > 0 && c.has_prev) {
                auto it = prev_of.find({c.a, c.b});
                if (it != prev_of.end()) pc = &cons[k - 1][it->second];
            }
            for (int q = 0; q < 4; q++) {
                const double *pt = r + CON_HEAD + q * POINT_ROW;
                c.prev[q] = (int)pt[13];
                for (int x = 0; x < 3; x++) {
                    Part<S> &p = c.p[q][x];
                    make_part(p, pt, c.ax[x], dA, dB, IA, IB, pt[6 + x], x == 0 ? pt[9] : 0.0);
                    // warm-start impulse: the tape's value, its derivative through the cache match
                    // from the previous step's final impulse (contact-constraints.ts:651-686)
                    double tape_lam = pt[10 + x];
                    S lam = S(tape_lam);
                    if (q < c.n && pc && c.prev[q] >= 0 && c.prev[q] < pc->n) {
                        S from = pc->p[c.prev[q]][x].totalLambda;
                        lam = mode == 0 ? with_value(from, tape_lam) : from;
                    }
                    if (p.effMass == 0) lam = S(0.0);  // rows reset in the setup carry nothing
                    p.totalLambda = lam;
                }
            }
        }
        // warm start in the tape's order (warmStartVelocityConstraints contact-constraints.ts:906-955)
        for (Con<S> &c : cs) {
            const int fa = flags(k, c.a), fb = flags(k, c.b);
            const bool dA = fa & T_DYNAMIC, dB = fb & T_DYNAMIC;
            const int dofA = (fa >> 8) & 63, dofB = (fb >> 8) & 63;
            for (int q = 0; q < c.n; q++) {
                Part<S> *p = c.p[q];
                if (p[1].effMass != 0 || p[2].effMass != 0) {
                    warm_start(p[1], c.a, c.b, dA, dB, c.imA, c.imB, c.ax[1], ratio, dofA, dofB);
                    warm_start(p[2], c.a, c.b, dA, dB, c.imA, c.imB, c.ax[2], ratio, dofA, dofB);
                }
                warm_start(p[0], c.a, c.b, dA, dB, c.imA, c.imB, c.ax[0], ratio, dofA, dofB);
            }
        }
        // solve order: sortContactIndices (sortKey, idA, idB), stable; islands share no dynamic body,
        // so one sweep over every island's contacts gives each island's sweep
        std::vector<int> ord(cs.size());
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
            const Con<S> &a = cs[x], &b = cs[y];
            if (a.key != b.key) return a.key < b.key;
            if (a.a != b.a) return a.a < b.a;
            return a.b < b.b;
        });
        for (int it = 0; it < T.iters; it++) {
            for (int ci : ord) {
                Con<S> &c = cs[ci];
                const int fa = flags(k, c.a), fb = flags(k, c.b);
                const bool dA = fa & T_DYNAMIC, dB = fb & T_DYNAMIC;
                const bool mA = fa & T_MOVING, mB = fb & T_MOVING;
                const int dofA = (fa >> 8) & 63, dofB = (fb >> 8) & 63;
                if (!dA && !dB) continue;
                for (int q = 0; q < c.n; q++) {
                    Part<S> *p = c.p[q];
                    if (p[1].effMass != 0 || p[2].effMass != 0) {
                        S l1 = total_lambda(p[1], c.a, c.b, mA, mB, c.ax[1]);
                        S l2 = total_lambda(p[2], c.a, c.b, mA, mB, c.ax[2]);
                        S mf = c.friction * p[0].totalLambda;
                        S fm = l1 * l1 + l2 * l2;
                        S mfs = mf * mf;
                        if (fm > mfs) {
                            S s = mf / sqrt_s(fm);
                            l1 = l1 * s;
                            l2 = l2 * s;
                        }
                        apply_lambda(p[1], c.a, c.b, dA, dB, c.imA, c.imB, c.ax[1], l1, dofA, dofB);
                        apply_lambda(p[2], c.a, c.b, dA, dB, c.imA, c.imB, c.ax[2], l2, dofA, dofB);
                    }
                }
                for (int q = 0; q < c.n; q++) {
                    Part<S> &p = c.p[q][0];
                    S tl = total_lambda(p, c.a, c.b, mA, mB, c.ax[0]);
                    apply_lambda(p, c.a, c.b, dA, dB, c.imA, c.imB, c.ax[0], max_s(S(0.0), tl), dofA, dofB);
                }
            }
        }
        for (int i = 0; i < n; i++)
            if (flags(k, i) & T_DYNAMIC) {
                vsum[i].x += v[i].x;
                vsum[i].y += v[i].y;
                vsum[i].z += v[i].z;
            }
    }

    // loss = sum over worlds |centroid of x_final + dt (vsum - ref) - target|^2, the centroid over
    // each world's bodies marked in_loss; ref = the real parts (mode 0) or a nominal run's sums
    S loss(const std::vector<V3s<double>> *ref) const {
        std::vector<V3s<S>> cen(T.worlds, {S(0.0), S(0.0), S(0.0)});
        std::vector<double> cnt(T.worlds, 0.0);
        for (int i = 0; i < T.n; i++) {
            const double *cst = T.consts + (size_t)i * CONST_ROW;
            if (cst[1] == 0) continue;
            int wd = (int)cst[0];
            V3s<S> dv = vsum[i];
            V3s<double> r = ref ? (*ref)[i] : V3s<double>{value(dv.x), value(dv.y), value(dv.z)};
            const double *x = T.x_final + (size_t)i * 3;
            cen[wd].x += S(x[0]) + S(T.dt) * (dv.x - S(r.x));
            cen[wd].y += S(x[1]) + S(T.dt) * (dv.y - S(r.y));
            cen[wd].z += S(x[2]) + S(T.dt) * (dv.z - S(r.z));
            cnt[wd] += 1;
        }
        S l = S(0.0);
        for (int wd = 0; wd < T.worlds; wd++) {
            if (cnt[wd] == 0) continue;
            S c = S(cnt[wd]);
            S dx = cen[wd].x / c - S(T.targets[3 * wd]), dy = cen[wd].y / c - S(T.targets[3 * wd + 1]),
              dz = cen[wd].z / c - S(T.targets[3 * wd + 2]);
            l += dx * dx + dy * dy + dz * dz;
        }
        return l;
    }
};
template <>
inline double Replay<double>::with_value_seed(double s, double) { return s; }
template <>
inline Dual Replay<Dual>::with_value_seed(Dual s, double d) { return {s.v, d}; }

}  // namespace orc_frozen
