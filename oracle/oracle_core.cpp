// TEST INFRASTRUCTURE -- NOT THE PRODUCT. See oracle_core.hpp.
#include "oracle_core.hpp"

#include <algorithm>
#include <functional>
#include <map>
#include <set>
#include <unordered_map>

namespace orc {

static constexpr uint32_t MAX_DEPTH = 3;  // graph/mod.rs:41

// active_nodes (validate.rs:24-43): everything reachable backwards from the Output.
static std::vector<uint32_t> active_nodes(const Graph& g) {
    const sf_node* out = nullptr;
    for (auto& n : g.nodes) if (n.kind == SF_NODE_OUTPUT) { out = &n; break; }
    if (!out) return {};
    std::set<uint32_t> seen;
    std::vector<uint32_t> stack{out->id};
    while (!stack.empty()) {
        uint32_t id = stack.back();
        stack.pop_back();
        if (!seen.insert(id).second) continue;
        for (auto& l : g.links) if (l.to_node == id) stack.push_back(l.from_node);
    }
    return std::vector<uint32_t>(seen.begin(), seen.end());  // sorted ascending
}

static std::map<uint32_t, uint32_t> body_owners(const Graph& g) {
    std::map<uint32_t, uint32_t> owners;
    for (auto& n : g.nodes)
        for (uint32_t b : g.body_of(n)) owners[b] = n.id;
    return owners;
}

// topo_order (validate.rs:45-85): Kahn's algorithm, smallest ready id first.
static bool topo_order(const Graph& g, std::vector<uint32_t>& order) {
    auto act = active_nodes(g);
    std::set<uint32_t> active(act.begin(), act.end());
    auto owners = body_owners(g);
    std::map<uint32_t, size_t> indeg;
    for (uint32_t id : active) if (!owners.count(id)) indeg[id] = 0;
    for (auto& l : g.links)
        if (indeg.count(l.to_node) && active.count(l.from_node)) indeg[l.to_node] += 1;
    std::vector<uint32_t> ready;
    for (auto& [id, d] : indeg) if (d == 0) ready.push_back(id);
    auto desc = [](uint32_t a, uint32_t b) { return a > b; };
    std::sort(ready.begin(), ready.end(), desc);
    order.clear();
    while (!ready.empty()) {
        uint32_t id = ready.back();
        ready.pop_back();
        order.push_back(id);
        std::vector<uint32_t> next;
        for (auto& l : g.links) {
            if (l.from_node != id) continue;
            auto it = indeg.find(l.to_node);
            if (it != indeg.end()) {
                it->second -= 1;
                if (it->second == 0) next.push_back(l.to_node);
            }
        }
        std::sort(next.begin(), next.end(), desc);
        ready.insert(ready.end(), next.begin(), next.end());
        std::sort(ready.begin(), ready.end(), desc);
    }
    return order.size() == indeg.size();
}

static uint32_t sat_mul(uint32_t a, uint32_t b) {
    uint64_t r = uint64_t(a) * uint64_t(b);
    return r > 0xffffffffull ? 0xffffffffu : uint32_t(r);
}

// iteration_product (validate.rs:112-141).
static uint32_t product(const Graph& g, uint32_t id, std::vector<uint32_t>& seen) {
    if (std::find(seen.begin(), seen.end(), id) != seen.end()) return 0xffffffffu;
    seen.push_back(id);
    uint32_t p = 1;
    const sf_node* n = g.node(id);
    if (n && n->kind == SF_NODE_ITERATE) {
        uint32_t m = 0;
        bool any = false;
        for (uint32_t b : g.body_of(*n)) { m = std::max(m, product(g, b, seen)); any = true; }
        p = sat_mul(n->u[0], any ? m : 1);
    }
    seen.pop_back();
    return p;
}

// trap_scales walk (eval.rs:853-877).
static void trap_walk(const Graph& g, uint32_t id, uint32_t depth, float* scales) {
    if (depth > MAX_DEPTH + 1) return;
    const sf_node* n = g.node(id);
    if (!n || !n->enabled) return;
    if (n->kind == SF_NODE_TRAP) scales[std::min<uint32_t>(n->u[0], 3)] = n->f[0];
    else if (n->kind == SF_NODE_ITERATE)
        for (uint32_t b : g.body_of(*n)) trap_walk(g, b, depth + 1, scales);
}

// lipschitz visit (eval.rs:828-849).
static void lip_visit(const Graph& g, uint32_t id, float radius, uint32_t depth, float* l) {
    if (depth > MAX_DEPTH + 1) return;
    const sf_node* n = g.node(id);
    if (!n || !n->enabled) return;
    if (n->kind == SF_NODE_TWIST || n->kind == SF_NODE_BEND) {
        float x = n->f[0] * radius;
        *l *= sqrtf(1.0f + x * x);
    }
    for (uint32_t b : g.body_of(*n)) lip_visit(g, b, radius, depth + 1, l);
}

// needed (eval.rs:35-47).
static void needed(const Graph& g, uint32_t id, std::set<uint32_t>& set) {
    if (!set.insert(id).second) return;
    const sf_node* n = g.node(id);
    if (!n) return;
    if (n->enabled && n->kind == SF_NODE_INSTANCES) return;
    for (uint32_t port = 0; port < input_count(n->kind); ++port) {
        uint32_t src;
        if (g.input_of(id, port, &src)) needed(g, src, set);
    }
}

// glam Quat::from_euler(EulerRot::XYZ, a, b, c) = Qx(a) Qy(b) Qz(c) as (x, y, z, w),
// and Quat * Vec3 (glam's mul_vec3); R = float restates the reference's f32 glam.
template <class R> struct Q4 { R x, y, z, w; };
template <class R> static Q4<R> qmul(const Q4<R>& a, const Q4<R>& b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
template <class R> static Q4<R> quat_xyz(const float deg[3]) {
    const R k = R(3.14159265358979323846) / R(180);
    const R a = R(deg[0]) * k, b = R(deg[1]) * k, c = R(deg[2]) * k;
    Q4<R> qx{r_sin(a * R(0.5)), 0, 0, r_cos(a * R(0.5))};
    Q4<R> qy{0, r_sin(b * R(0.5)), 0, r_cos(b * R(0.5))};
    Q4<R> qz{0, 0, r_sin(c * R(0.5)), r_cos(c * R(0.5))};
    return qmul(qmul(qx, qy), qz);
}
template <class R> static V3<R> qrot(const Q4<R>& q, V3<R> v) {
    V3<R> b(q.x, q.y, q.z);
    R b2 = b.dot(b);
    return v * (q.w * q.w - b2) + b * (v.dot(b) * R(2)) + b.cross(v) * (q.w * R(2));
}

// bvh::build (bvh.rs:26-102), in binary32 as the reference.
static void bvh_split(std::vector<Graph::InstBounds>& leaves, size_t lo, size_t hi,
                      std::vector<Graph::InstBounds>& nodes) {
    float mn[3], mx[3];
    for (int k = 0; k < 3; ++k) { mn[k] = INFINITY; mx[k] = -INFINITY; }
    for (size_t i = lo; i < hi; ++i)
        for (int k = 0; k < 3; ++k) {
            mn[k] = std::min(mn[k], leaves[i].center[k] - leaves[i].half[k]);
            mx[k] = std::max(mx[k], leaves[i].center[k] + leaves[i].half[k]);
        }
    size_t index = nodes.size();
    Graph::InstBounds n{};
    for (int k = 0; k < 3; ++k) {
        n.center[k] = mn[k] * 0.5f + mx[k] * 0.5f;
        n.half[k] = std::max(mx[k] - n.center[k], n.center[k] - mn[k]) + 0.002f;
    }
    n.placement = -1;
    nodes.push_back(n);
    if (hi - lo == 1) {
        nodes[index].placement = leaves[lo].placement;
    } else {
        float e[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
        int axis = (e[0] >= e[1] && e[0] >= e[2]) ? 0 : (e[1] >= e[2] ? 1 : 2);
        size_t middle = lo + (hi - lo) / 2;
        std::nth_element(leaves.begin() + lo, leaves.begin() + middle, leaves.begin() + hi,
                         [axis](const Graph::InstBounds& a, const Graph::InstBounds& b) {
                             if (a.center[axis] != b.center[axis]) return a.center[axis] < b.center[axis];
                             return a.placement < b.placement;
                         });
        bvh_split(leaves, lo, middle, nodes);
        bvh_split(leaves, middle, hi, nodes);
    }
    nodes[index].escape = nodes.size();
}
std::vector<Graph::InstBounds> bvh_build(const sf_placement* pl, uint32_t count, const float* half) {
    std::vector<Graph::InstBounds> leaves(count), nodes;
    for (uint32_t i = 0; i < count; ++i) {
        Q4<float> r = quat_xyz<float>(pl[i].angles);
        V3<float> ext(0, 0, 0);
        for (int a = 0; a < 3; ++a) {
            V3<float> axis(a == 0, a == 1, a == 2);
            V3<float> c = qrot(r, axis);
            float h = half[a] * pl[i].scale[a];
            ext = ext + V3<float>(std::fabs(c.x), std::fabs(c.y), std::fabs(c.z)) * h;
        }
        float e[3] = {ext.x, ext.y, ext.z};
        for (int k = 0; k < 3; ++k) {
            float pad = (std::fabs(pl[i].position[k]) + e[k]) * (16.0f * 1.1920929e-7f) + 0.002f;
            leaves[i].center[k] = pl[i].position[k];
            leaves[i].half[k] = e[k] + pad;
        }
        leaves[i].escape = 0;
        leaves[i].placement = i;
    }
    if (count) bvh_split(leaves, 0, count, nodes);
    return nodes;
}
// InstanceBounds::distance (bvh.rs:19-24).
template <class R> static R inst_bound(const Graph::InstBounds& n, V3<R> p) {
    V3<R> q(r_abs(p.x - R(n.center[0])) - R(n.half[0]), r_abs(p.y - R(n.center[1])) - R(n.half[1]),
            r_abs(p.z - R(n.center[2])) - R(n.half[2]));
    V3<R> m(r_max(q.x, R(0)), r_max(q.y, R(0)), r_max(q.z, R(0)));
    return m.length() + r_min(r_max(q.x, r_max(q.y, q.z)), R(0));
}

bool prepare(Graph& g) {
    g.ok = false;
    if (!topo_order(g, g.order)) { g.error = "cycle"; return false; }
    g.output = 0;
    for (auto& n : g.nodes) if (n.kind == SF_NODE_OUTPUT) { g.output = n.id; break; }
    std::set<uint32_t> set;
    needed(g, g.output, set);
    g.plan.clear();
    for (uint32_t id : g.order) if (set.count(id)) g.plan.push_back(id);
    g.plans.clear();
    g.instances.clear();
    g.plans[g.output] = g.plan;
    for (auto& n : g.nodes) {
        if (!n.enabled || n.kind != SF_NODE_INSTANCES) continue;
        if (size_t(n.u[0]) + n.u[1] > g.placements.size()) { g.error = "placements out of range"; return false; }
        g.instances[n.id] = bvh_build(g.placements.data() + n.u[0], n.u[1], n.f);
        uint32_t child;
        if (g.input_of(n.id, 0, &child) && !g.plans.count(child)) {
            std::set<uint32_t> sub;
            needed(g, child, sub);
            std::vector<uint32_t> plan;
            for (uint32_t id : g.order) if (sub.count(id)) plan.push_back(id);
            g.plans[child] = plan;
        }
    }
    g.union_leaves.clear();
    {
        std::function<void(bool, uint32_t)> leaves = [&](bool has, uint32_t id) {
            const sf_node* n = has ? g.node(id) : nullptr;
            if (n && n->enabled && n->kind == SF_NODE_UNION) {
                for (uint32_t port = 0; port < 2; ++port) {
                    uint32_t from = 0;
                    const bool h = g.input_of(id, port, &from);
                    leaves(h, from);
                }
                return;
            }
            if (!n) { g.union_leaves.push_back(UINT32_MAX); return; }
            if (std::find(g.union_leaves.begin(), g.union_leaves.end(), id) != g.union_leaves.end()) return;
            g.union_leaves.push_back(id);
            if (!g.plans.count(id)) {
                std::set<uint32_t> sub;
                needed(g, id, sub);
                std::vector<uint32_t> plan;
                for (uint32_t o : g.order) if (sub.count(o)) plan.push_back(o);
                g.plans[id] = plan;
            }
        };
        uint32_t root = 0;
        const bool has = g.input_of(g.output, 0, &root);
        leaves(has, root);
    }
    for (int i = 0; i < 4; ++i) g.trap_scales[i] = 1.f;
    for (uint32_t id : g.order) trap_walk(g, id, 0, g.trap_scales);
    auto owners = body_owners(g);
    uint32_t best = 0;
    bool any = false;
    for (uint32_t id : active_nodes(g)) {
        if (owners.count(id)) continue;
        std::vector<uint32_t> seen;
        best = std::max(best, product(g, id, seen));
        any = true;
    }
    g.iteration_product = any ? best : 1;
    float l = 1.f;
    for (uint32_t id : active_nodes(g)) lip_visit(g, id, g.hint, 0, &l);
    g.lipschitz = l;
    g.step_scale = g.safety / l;
    // negative_bounds (graph_wgsl.rs:979-1006): a bound reached through an odd
    // number of Subtraction second inputs is not a lower bound there.
    std::set<uint32_t> unsafe;
    std::set<std::pair<uint32_t, bool>> seen;
    std::vector<std::pair<uint32_t, bool>> work{{g.output, false}};
    while (!work.empty()) {
        auto [id, negative] = work.back();
        work.pop_back();
        if (!seen.insert({id, negative}).second) continue;
        const sf_node* n = g.node(id);
        if (!n) continue;
        if (negative && (n->kind == SF_NODE_BOUNDED || n->kind == SF_NODE_INSTANCES)) unsafe.insert(id);
        for (uint32_t port = 0; port < input_count(n->kind); ++port) {
            uint32_t from;
            if (g.input_of(id, port, &from))
                work.push_back({from, negative != (n->enabled && n->kind == SF_NODE_SUBTRACTION && port == 1)});
        }
    }
    g.fast_bounds.clear();
    for (uint32_t id : g.order) {
        const sf_node* n = g.node(id);
        if (n && n->enabled && (n->kind == SF_NODE_BOUNDED || n->kind == SF_NODE_INSTANCES) && !unsafe.count(id))
            g.fast_bounds.insert(id);
    }
    g.ok = true;
    return true;
}

// ---------------------------------------------------------------- DE
// integral_spherical_power (eval.rs:129-178).
template <class R> static void spherical_power(V3<R> p, R r, uint32_t n, V3<R>* out, R* deriv) {
    if (n == 1) { *out = p; *deriv = R(1); return; }
    auto mul = [](V2<R> a, V2<R> b) { return V2<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
    R rho = V2<R>(p.x, p.y).length();
    V2<R> theta(r_clamp(p.z / r, R(-1), R(1)), rho / r);
    V2<R> phi = rho > R(0) ? V2<R>(p.x, p.y) / rho : V2<R>(1, 0);
    if (n == 6 || n == 8) {
        auto square = [](V2<R> a) { return V2<R>(a.x * a.x - a.y * a.y, R(2) * a.x * a.y); };
        V2<R> t2 = square(theta), f2 = square(phi);
        V2<R> t4 = square(t2), f4 = square(f2);
        R r2 = r * r;
        R r4 = r2 * r2;
        V2<R> t, f;
        R previous;
        if (n == 6) { t = mul(t2, t4); f = mul(f2, f4); previous = r4 * r; }
        else { t = square(t4); f = square(f4); previous = r4 * r2 * r; }
        *out = V3<R>(t.y * f.x, t.y * f.y, t.x) * (previous * r);
        *deriv = R(n) * previous;
        return;
    }
    V2<R> t(1, 0), f(1, 0);
    uint32_t e = n;
    while (e != 0) {
        if (e & 1) { t = mul(t, theta); f = mul(f, phi); }
        e >>= 1;
        if (e != 0) { theta = mul(theta, theta); phi = mul(phi, phi); }
    }
    R radial_previous = 1;
    for (uint32_t i = 1; i < n; ++i) radial_previous *= r;
    *out = V3<R>(t.y * f.x, t.y * f.y, t.x) * (radial_previous * r);
    *deriv = R(n) * radial_previous;
}

static inline uint32_t u32_of_f(float v) { return uint32_t(v); }

// terrain noise / rock distance (eval.rs:232-263).
static float terrain_hash(int32_t cx, int32_t cy, int32_t cz, uint32_t seed) {
    uint32_t h = (uint32_t(cx) * 0x8da6b343u) ^ (uint32_t(cy) * 0xd8163841u) ^ (uint32_t(cz) * 0xcb1ab31fu) ^ seed;
    h = (h ^ (h >> 16)) * 0x7feb352du;
    h = (h ^ (h >> 15)) * 0x846ca68bu;
    h ^= h >> 16;
    return float(h >> 8) / 16777216.0f;
}
template <class R> static R terrain_noise(V3<R> p, uint32_t seed) {
    V3<R> base(r_floor(p.x), r_floor(p.y), r_floor(p.z));
    V3<R> f = p - base;
    V3<R> t = f * f * (V3<R>::splat(3) - f * R(2));
    int32_t c0 = int32_t(base.x), c1 = int32_t(base.y), c2 = int32_t(base.z);
    auto mix = [](R a, R b, R t) { return a + (b - a) * t; };
    auto hash = [&](int x, int y, int z) { return R(terrain_hash(c0 + x, c1 + y, c2 + z, seed)); };
    R a = mix(hash(0, 0, 0), hash(1, 0, 0), t.x);
    R b = mix(hash(0, 1, 0), hash(1, 1, 0), t.x);
    R d = mix(hash(0, 0, 1), hash(1, 0, 1), t.x);
    R e = mix(hash(0, 1, 1), hash(1, 1, 1), t.x);
    return mix(mix(a, b, t.y), mix(d, e, t.y), t.z);
}
template <class R> static R rock_distance(V3<R> p, V3<R> half, R erosion, uint32_t seed) {
    R h = half.min_element();
    V3<R> q = p * (R(1.15) / h);
    R relief = R(0.57) * terrain_noise(q, seed) + R(0.29) * terrain_noise(q * R(2.03), seed + 97) +
               R(0.14) * terrain_noise(q * R(4.17), seed + 193) - R(0.5);
    return ((p / half).length() - R(1) - erosion * relief) * h / (R(1) + R(5.22) * erosion);
}

// measure (eval.rs:299-331).
template <class R> static R measure(uint32_t m, V3<R> p) {
    const R TAU = R(6.28318530717958647692);
    switch (m) {
    case SF_MEASURE_NORM: return p.length();
    case SF_MEASURE_AXIS_X: return V2<R>(p.y, p.z).length();
    case SF_MEASURE_AXIS_Y: return V2<R>(p.x, p.z).length();
    case SF_MEASURE_AXIS_Z: return V2<R>(p.x, p.y).length();
    case SF_MEASURE_PLANE_Y: return r_abs(p.y);
    case SF_MEASURE_ANGLE_XY: return (p.x == R(0) && p.y == R(0)) ? R(0.5) : r_atan2(p.y, p.x) / TAU + R(0.5);
    case SF_MEASURE_ANGLE_XZ: return (p.x == R(0) && p.z == R(0)) ? R(0.5) : r_atan2(p.z, p.x) / TAU + R(0.5);
    case SF_MEASURE_ANGLE_YZ: return (p.y == R(0) && p.z == R(0)) ? R(0.5) : r_atan2(p.z, p.y) / TAU + R(0.5);
    case SF_MEASURE_LOG_NORM: return r_log1p(p.length());
    default: return p.length();
    }
}

template <class R> static V3<R> f3(const sf_node& n, int i) { return V3<R>(R(n.f[i]), R(n.f[i + 1]), R(n.f[i + 2])); }

// glam Quat::from_euler(XYZ) * p (common.wgsl:258-265 restates it as Rx(Ry(Rz p))).
template <class R> static V3<R> rotate_euler_xyz(V3<R> p, V3<R> a) {
    V3<R> q = p;
    q = V3<R>(r_cos(a.z) * q.x - r_sin(a.z) * q.y, r_sin(a.z) * q.x + r_cos(a.z) * q.y, q.z);
    q = V3<R>(r_cos(a.y) * q.x + r_sin(a.y) * q.z, q.y, -r_sin(a.y) * q.x + r_cos(a.y) * q.z);
    q = V3<R>(q.x, r_cos(a.x) * q.y - r_sin(a.x) * q.z, r_sin(a.x) * q.y + r_cos(a.x) * q.z);
    return q;
}

// apply_seeded (eval.rs:346-556).
template <class R>
static PointState<R> apply_seeded(const Graph& g, uint32_t id, PointState<R> s, V3<R> c, V3<R> seed_p, R seed_dr) {
    const sf_node* np = g.node(id);
    if (!np || !np->enabled) return s;
    const sf_node& n = *np;
    switch (n.kind) {
    case SF_NODE_TRANSLATE: s.p = s.p + f3<R>(n, 0); break;
    case SF_NODE_ROTATE: {
        V3<R> a = f3<R>(n, 0);
        s.p = rotate_euler_xyz(s.p, V3<R>(to_radians(a.x), to_radians(a.y), to_radians(a.z)));
        break;
    }
    case SF_NODE_SCALE: s.p = s.p * R(n.f[0]); s.dr *= r_abs(R(n.f[0])); break;
    case SF_NODE_SCALE_AXES: { V3<R> f = f3<R>(n, 0); s.p = s.p * f; s.dr *= f.max_element(); break; }
    case SF_NODE_MIRROR: {
        V3<R> nn = safe_normalize(f3<R>(n, 0));
        R h = s.p.dot(nn) - R(n.f[3]);
        if (h < R(0)) s.p = s.p - nn * (R(2) * h);
        break;
    }
    case SF_NODE_BOX_FOLD: {
        R l = R(n.f[0]);
        s.p = vclamp(s.p, V3<R>::splat(-l), V3<R>::splat(l)) * R(2) - s.p;
        break;
    }
    case SF_NODE_BOX_FOLD_AXES: {
        V3<R> l = f3<R>(n, 0);
        V3<R> folded = vclamp(s.p, -l, l) * R(2) - s.p;
        for (int a = 0; a < 3; ++a) if (n.u[a]) s.p[a] = folded[a];
        break;
    }
    case SF_NODE_SPHERE_INVERSION: {
        R rad = R(n.f[0]), mr = R(n.f[1]);
        R k = rad * rad / r_max(s.p.length_squared(), mr * mr);
        s.p = s.p * k;
        s.dr *= k;
        break;
    }
    case SF_NODE_SPHERE_FOLD: {
        R r2 = s.p.dot(s.p);
        R mr = R(n.f[0]), fr = R(n.f[1]);
        R mr2 = mr * mr, fr2 = fr * fr;
        R k = r2 < mr2 ? fr2 / mr2 : (r2 < fr2 ? fr2 / r2 : R(1));
        s.p = s.p * k;
        s.dr *= k;
        break;
    }
    case SF_NODE_ABS:
        if (n.u[0]) s.p.x = r_abs(s.p.x);
        if (n.u[1]) s.p.y = r_abs(s.p.y);
        if (n.u[2]) s.p.z = r_abs(s.p.z);
        break;
    case SF_NODE_MENGER_FOLD: {
        R scale = R(n.f[0]);
        V3<R> off = f3<R>(n, 1);
        V3<R> z = s.p.abs();
        if (z.x < z.y) z = V3<R>(z.y, z.x, z.z);
        if (z.x < z.z) z = V3<R>(z.z, z.y, z.x);
        if (z.y < z.z) z = V3<R>(z.x, z.z, z.y);
        z = z * scale - off * (scale - R(1));
        if (z.z < R(-0.5) * off.z * (scale - R(1))) z.z += off.z * (scale - R(1));
        s.p = z;
        s.dr *= scale;
        break;
    }
    case SF_NODE_KALEIDO: {
        const R TAU = R(6.28318530717958647692);
        R sector = TAU / R(std::max<uint32_t>(n.u[0], 1));
        R a = r_atan2(s.p.z, s.p.x) + to_radians(R(n.f[0]));
        a = r_abs(r_rem_euclid(a + sector * R(0.5), sector) - sector * R(0.5));
        R r = V2<R>(s.p.x, s.p.z).length();
        s.p.x = r * r_cos(a);
        s.p.z = r * r_sin(a);
        break;
    }
    case SF_NODE_POWER: {
        R power = R(n.f[0]);
        R radius = s.p.length();
        float pf = n.f[0];
        if (radius >= R(1e-12) && pf >= 1.0f && pf <= 16.0f && pf == floorf(pf)) {
            V3<R> point;
            R deriv;
            spherical_power(s.p, radius, u32_of_f(pf), &point, &deriv);
            s.p = point;
            s.dr *= deriv;
        } else {
            R r = r_max(radius, R(1e-12));
            R theta = radius >= R(1e-12) ? r_atan2(V2<R>(s.p.x, s.p.y).length(), s.p.z)
                                         : r_acos(r_clamp(s.p.z / r, R(-1), R(1)));
            R phi = r_atan2(s.p.y, s.p.x);
            s.dr *= r_pow(r, power - R(1)) * power;
            R zr = r_pow(r, power);
            R st = r_sin(theta * power), ct = r_cos(theta * power);
            R sp = r_sin(phi * power), cp = r_cos(phi * power);
            s.p = V3<R>(st * cp, st * sp, ct) * zr;
        }
        break;
    }
    case SF_NODE_ADD_ORIGIN: s.p = s.p + c; s.dr += R(1); break;
    case SF_NODE_ADD_SEED: {
        V3<R> m = f3<R>(n, 0);
        s.p = s.p + seed_p * m;
        s.dr += seed_dr * m.abs().max_element();
        break;
    }
    case SF_NODE_ADD_CONSTANT: {
        V3<R> m = f3<R>(n, 0), j = f3<R>(n, 3);
        s.p = s.p + (c * m + j);
        s.dr += m.abs().max_element();
        break;
    }
    case SF_NODE_TWIST: {
        R a = R(n.f[0]) * s.p.y;
        R sn = r_sin(a), cs = r_cos(a);
        V2<R> v(cs * s.p.x - sn * s.p.z, sn * s.p.x + cs * s.p.z);
        s.p.x = v.x;
        s.p.z = v.y;
        break;
    }
    case SF_NODE_BEND: {
        R a = R(n.f[0]) * s.p.x;
        R sn = r_sin(a), cs = r_cos(a);
        V2<R> v(cs * s.p.x - sn * s.p.y, sn * s.p.x + cs * s.p.y);
        s.p.x = v.x;
        s.p.y = v.y;
        break;
    }
    case SF_NODE_TILE: {
        V3<R> per = f3<R>(n, 0);
        V3<R> half = per * R(0.5);
        s.p = V3<R>(r_rem_euclid(s.p.x + half.x, per.x) - half.x, r_rem_euclid(s.p.y + half.y, per.y) - half.y,
                    r_rem_euclid(s.p.z + half.z, per.z) - half.z);
        break;
    }
    case SF_NODE_REPEAT_FINITE: {
        V3<R> per = f3<R>(n, 0);
        V3<R> last = V3<R>(R(n.u[0]), R(n.u[1]), R(n.u[2])) - V3<R>::splat(1);
        V3<R> half = last * R(0.5);
        V3<R> q = s.p / per + half + V3<R>::splat(R(0.5));
        V3<R> cell = vclamp(V3<R>(r_floor(q.x), r_floor(q.y), r_floor(q.z)), V3<R>::splat(0), last) - half;
        s.p = s.p - cell * per;
        break;
    }
    case SF_NODE_ITERATE: {
        V3<R> lp = s.p;
        R ldr = s.dr;
        uint32_t iterations = n.u[0];
        R bailout = R(n.f[0]);
        auto b = g.body_of(n);
        for (uint32_t i = 0; i < iterations; ++i) {
            if (s.p.length() > bailout) break;
            for (uint32_t bid : b) s = apply_seeded(g, bid, s, c, lp, ldr);
            s.iter += 1;
        }
        break;
    }
    case SF_NODE_TRAP: {
        uint32_t i = std::min<uint32_t>(n.u[0], 3);
        R v = measure(n.u[1], s.p);
        switch (n.u[2]) {
        case SF_TRAP_MAXIMUM: s.traps[i] = s.traps[i] >= R(1e30) ? v : r_max(s.traps[i], v); break;
        case SF_TRAP_LAST: s.traps[i] = v; break;
        default: s.traps[i] = r_min(s.traps[i], v); break;
        }
        break;
    }
    default: break;
    }
    return s;
}

// fence (eval.rs:558-599).
template <class R> static R fence(const sf_node& n, const PointState<R>& s) {
    switch (n.kind) {
    case SF_NODE_SPHERE: return (s.p.length() - R(n.f[0])) / s.dr;
    case SF_NODE_TORUS:
        return (V2<R>(V2<R>(s.p.x, s.p.z).length() - R(n.f[0]), s.p.y).length() - R(n.f[1])) / s.dr;
    case SF_NODE_CYLINDER: {
        V2<R> q(V2<R>(s.p.x, s.p.z).length() - R(n.f[0]), r_abs(s.p.y) - R(n.f[1]));
        V2<R> qm(r_max(q.x, R(0)), r_max(q.y, R(0)));
        return (qm.length() + r_min(r_max(q.x, q.y), R(0))) / s.dr;
    }
    case SF_NODE_BOX: {
        V3<R> q = s.p.abs() - f3<R>(n, 0);
        return (vmax(q, V3<R>::splat(0)).length() + r_min(r_max(q.x, r_max(q.y, q.z)), R(0))) / s.dr;
    }
    case SF_NODE_ROUND_BOX: {
        V3<R> half = f3<R>(n, 0);
        R r = r_min(R(n.f[3]), half.min_element());
        V3<R> q = s.p.abs() - (half - V3<R>::splat(r));
        return (vmax(q, V3<R>::splat(0)).length() + r_min(q.max_element(), R(0)) - r) / s.dr;
    }
    case SF_NODE_ROCK: return rock_distance(s.p, f3<R>(n, 0), R(n.f[3]), n.u[0]) / s.dr;
    case SF_NODE_PLANE: return (s.p.dot(safe_normalize(f3<R>(n, 0))) - R(n.f[3])) / s.dr;
    case SF_NODE_NORM_FENCE: return (s.p.length() - R(n.f[0])) / r_abs(s.dr);
    case SF_NODE_BULB_FENCE: {
        R r = r_max(s.p.length(), R(1e-12));
        return R(0.5) * r_log(r) * r / s.dr;
    }
    default: return std::numeric_limits<R>::infinity();
    }
}

template <class R> static bool is_empty(R d) { return d >= R(1e30); }

// combine (eval.rs:601-657).
template <class R> static DistState<R> combine(const sf_node& n, DistState<R> a, DistState<R> b) {
    const R INF = std::numeric_limits<R>::infinity();
    auto blend = [&](R h, R d) {
        DistState<R> r;
        for (int i = 0; i < 4; ++i) {
            bool fa = r_finite(a.traps[i]), fb = r_finite(b.traps[i]);
            r.traps[i] = (fa && fb) ? b.traps[i] + (a.traps[i] - b.traps[i]) * h : fa ? a.traps[i] : fb ? b.traps[i] : INF;
        }
        r.d = d;
        r.material = h >= R(0.5) ? a.material : b.material;
        r.iter = h >= R(0.5) ? a.iter : b.iter;
        return r;
    };
    // flags (graph_wgsl.rs:845-852): a union keeps its winner's, the others join both
    DistState<R> r;
    switch (n.kind) {
    case SF_NODE_UNION: { r = a.d <= b.d ? a : b; r.d = r_min(a.d, b.d); return r; }
    case SF_NODE_INTERSECTION: { r = a.d >= b.d ? a : b; r.d = r_max(a.d, b.d); break; }
    case SF_NODE_SUBTRACTION: { r = a; r.d = r_max(a.d, -b.d); break; }
    case SF_NODE_SMOOTH_UNION: {
        if (is_empty(a.d)) { r = b; break; }
        if (is_empty(b.d)) { r = a; break; }
        R k = R(n.f[0]);
        R h = r_clamp(R(0.5) + R(0.5) * (b.d - a.d) / k, R(0), R(1));
        r = blend(h, b.d + (a.d - b.d) * h - k * h * (R(1) - h));
        break;
    }
    case SF_NODE_SMOOTH_INTERSECTION: {
        if (is_empty(a.d)) { r = b; r.d = INF; break; }
        if (is_empty(b.d)) { r = a; r.d = INF; break; }
        R k = R(n.f[0]);
        R h = r_clamp(R(0.5) - R(0.5) * (b.d - a.d) / k, R(0), R(1));
        r = blend(h, b.d + (a.d - b.d) * h + k * h * (R(1) - h));
        break;
    }
    default: return a;
    }
    r.flags = a.flags | b.flags;
    return r;
}

template <class R>
static DistState<R> eval_raw(const Graph& g, uint32_t target, V3<R> p, bool fast, int depth, bool probe = false);

// Instances (eval.rs:749-814): the nearest copy found by the seeded stackless walk
// over the fence hierarchy; with fast, the GPU's skips (graph_wgsl.rs:760-790): the
// root fence beyond the margin, and copies whose fence is beyond it. probe (the union
// search's bounds-only sample, graph_wgsl.rs:766-767): the root fence whatever the margin.
template <class R>
static DistState<R> eval_instances(const Graph& g, const sf_node& n, V3<R> p, bool fast, int depth,
                                   bool probe = false) {
    const R INF = std::numeric_limits<R>::infinity();
    DistState<R> best{INF, 0, 0, {INF, INF, INF, INF}};
    uint32_t child;
    if (!g.input_of(n.id, 0, &child) || depth > int(MAX_DEPTH)) return best;
    const auto& nodes = g.instances.at(n.id);
    if (nodes.empty()) return best;
    const bool skip = fast && g.fast_bounds.count(n.id);
    const R margin = R(n.f[3]);
    if (skip) {
        best.d = R(1e30);
        R env = inst_bound(nodes[0], p);
        if (probe || env > margin) return DistState<R>{env, 0, 0, {INF, INF, INF, INF}, 1};
    }
    size_t chosen = SIZE_MAX, seed = 0;
    while (nodes[seed].placement < 0) {
        size_t left = seed + 1, right = nodes[left].escape;
        seed = inst_bound(nodes[left], p) <= inst_bound(nodes[right], p) ? left : right;
    }
    size_t cursor = seed;
    bool seed_pass = true;
    while (cursor < nodes.size()) {
        size_t current = cursor;
        bool first = seed_pass;
        seed_pass = false;
        cursor = first ? 0 : current + 1;
        const auto& node = nodes[current];
        if (inst_bound(node, p) > best.d) {
            if (!first) cursor = node.escape;
            continue;
        }
        if (!first && current == seed) continue;
        if (node.placement < 0) continue;
        size_t index = size_t(node.placement);
        const sf_placement& pl = g.placements[n.u[0] + index];
        Q4<R> rot = quat_xyz<R>(pl.angles);
        Q4<R> conj{-rot.x, -rot.y, -rot.z, rot.w};
        V3<R> sc(R(pl.scale[0]), R(pl.scale[1]), R(pl.scale[2]));
        V3<R> q = qrot(conj, p - V3<R>(R(pl.position[0]), R(pl.position[1]), R(pl.position[2]))) / sc;
        R smin = r_min(sc.x, r_min(sc.y, sc.z));
        // the Box fence of half * scale at q * scale (eval.rs:796-804)
        V3<R> qs = q * sc;
        V3<R> e(r_abs(qs.x) - R(n.f[0]) * sc.x, r_abs(qs.y) - R(n.f[1]) * sc.y, r_abs(qs.z) - R(n.f[2]) * sc.z);
        R bound = V3<R>(r_max(e.x, R(0)), r_max(e.y, R(0)), r_max(e.z, R(0))).length() +
                  r_min(r_max(e.x, r_max(e.y, e.z)), R(0));
        if (bound > best.d) continue;
        DistState<R> d;
        if (skip && bound > margin) {
            d = DistState<R>{bound, 0, 0, {INF, INF, INF, INF}, 1};
        } else {
            // the template of a search that may not skip runs exactly (graph_wgsl.rs:
            // the `_exact` variant), so fast mode passes into it only from a skipping one
            d = eval_raw(g, child, q, skip, depth + 1);
            d.d = r_max(d.d * smin, bound);
        }
        if (d.d < best.d || (d.d == best.d && index < chosen)) {
            best = d;
            chosen = index;
        }
    }
    return best;
}

// evaluate_raw (eval.rs:671-826) + PreparedGraph::evaluate (eval.rs:98-114); with
// fast, the GPU's skippable bounds (graph_wgsl.rs:800-814); with probe as well, the
// union search's bounds-only sample (graph_wgsl.rs:808-812): every skippable bound
// whatever the margin.
template <class R>
static DistState<R> eval_raw(const Graph& g, uint32_t target, V3<R> p, bool fast, int depth, bool probe) {
    const R INF = std::numeric_limits<R>::infinity();
    DistState<R> empty{INF, 0, 0, {INF, INF, INF, INF}};
    PointState<R> start{p, R(1), 0, {INF, INF, INF, INF}};
    struct Val { bool point; PointState<R> ps; DistState<R> ds; };
    auto pit = g.plans.find(target);
    if (pit == g.plans.end()) return empty;
    const std::vector<uint32_t>& plan = pit->second;
    std::unordered_map<uint32_t, Val> values;
    values.reserve(plan.size() * 2);
    auto get_point = [&](uint32_t id, uint32_t port) {
        uint32_t from;
        if (g.input_of(id, port, &from)) {
            auto it = values.find(from);
            if (it != values.end() && it->second.point) return it->second.ps;
        }
        return start;
    };
    auto get_dist = [&](uint32_t id, uint32_t port) {
        uint32_t from;
        if (g.input_of(id, port, &from)) {
            auto it = values.find(from);
            if (it != values.end() && !it->second.point) return it->second.ds;
        }
        return empty;
    };
    for (uint32_t id : plan) {
        const sf_node& n = *g.node(id);
        Val v{};
        uint32_t k = n.kind;
        if (k == SF_NODE_INPUT) { v.point = true; v.ps = start; }
        else if (k == SF_NODE_OUTPUT) { v.point = false; v.ds = get_dist(id, 0); }
        else if (is_point_to_point(k)) {
            PointState<R> s = get_point(id, 0);
            v.point = true;
            v.ps = apply_seeded(g, id, s, p, s.p, s.dr);
        } else if (is_fence(k)) {
            PointState<R> s = get_point(id, 0);
            v.point = false;
            v.ds.d = n.enabled ? fence(n, s) : INF;
            v.ds.material = 0;
            v.ds.iter = s.iter;
            for (int i = 0; i < 4; ++i) v.ds.traps[i] = s.traps[i];
        } else if (k == SF_NODE_MATERIAL_TAG) {
            v.point = false;
            v.ds = get_dist(id, 0);
            if (n.enabled) v.ds.material = n.u[0];
        } else if (k == SF_NODE_BOUNDED) {
            v.point = false;
            v.ds = get_dist(id, 1);
            if (n.enabled) {
                sf_node box = n;
                box.kind = SF_NODE_BOX;
                const R bound = fence(box, get_point(id, 0));
                if (fast && g.fast_bounds.count(id) && (probe || bound > R(n.f[3])))
                    v.ds = DistState<R>{bound, 0, 0, {INF, INF, INF, INF}, 1};
                else
                    v.ds.d = r_max(v.ds.d, bound);
            }
        } else if (k == SF_NODE_INSTANCES && n.enabled) {
            v.point = false;
            v.ds = eval_instances(g, n, p, fast, depth, probe);
        } else if (!n.enabled) {
            v.point = false;
            v.ds = get_dist(id, 0);
        } else {
            v.point = false;
            v.ds = combine(n, get_dist(id, 0), get_dist(id, 1));
        }
        values[id] = v;
    }
    auto it = values.find(target);
    if (it != values.end() && !it->second.point) return it->second.ds;
    return empty;
}

template <class R> static Sample<R> sample_of(const Graph& g, const DistState<R>& r) {
    Sample<R> out;
    out.distance = r.d;
    out.material = r.material;
    for (int i = 0; i < 4; ++i)
        out.traps[i] = r_finite(r.traps[i]) ? r_min(r.traps[i] / R(g.trap_scales[i]), R(1)) : R(1);
    out.iterations = std::min(r.iter, g.iteration_product);
    out.flags = r.flags;
    return out;
}

// The union search (graph_wgsl.rs:1112-1154, its `_exact` function): each leaf's probe
// (a probe that took no skip is the leaf's exact sample), then the unsettled leaf with
// the lowest bound, ties to the lower index, evaluated exactly until no bound can
// reach the best; the best starts empty (+inf) where the WGSL starts from a 1e30
// sentinel, so an all-empty union keeps the plain union's +inf.
template <class R> Sample<R> evaluate_union_search(const Graph& g, V3<R> p, uint32_t* exact_leaves) {
    const size_t k = g.union_leaves.size();
    if (k < 2 || k > 128 || g.fast_bounds.empty()) return evaluate(g, p, false);
    const R INF = std::numeric_limits<R>::infinity();
    const DistState<R> empty{INF, 0, 0, {INF, INF, INF, INF}};
    auto leaf = [&](size_t i, bool probe) {
        return g.union_leaves[i] == UINT32_MAX ? empty : eval_raw(g, g.union_leaves[i], p, probe, 0, probe);
    };
    std::vector<R> lower(k);
    std::vector<char> settled(k, 0);
    DistState<R> best = empty;
    size_t winner = k;
    for (size_t i = 0; i < k; ++i) {
        const DistState<R> s = leaf(i, true);
        lower[i] = s.d;
        if (s.flags == 0) {
            settled[i] = 1;
            if (s.d < best.d || (s.d == best.d && i < winner)) { best = s; winner = i; }
        }
    }
    for (size_t step = 0; step < k; ++step) {
        size_t chosen = k;
        R bound = INF;
        for (size_t i = 0; i < k; ++i)
            if (!settled[i] && (lower[i] < bound || (lower[i] == bound && i < chosen))) { chosen = i; bound = lower[i]; }
        if (chosen == k || bound > best.d) break;
        settled[chosen] = 1;
        if (exact_leaves) ++*exact_leaves;
        const DistState<R> s = leaf(chosen, false);
        if (s.d < best.d || (s.d == best.d && chosen < winner)) { best = s; winner = chosen; }
    }
    return sample_of(g, best);
}

template <class R> Sample<R> evaluate(const Graph& g, V3<R> p, bool fast) {
    DistState<R> r = eval_raw(g, g.output, p, fast, 0);
    Sample<R> out;
    out.distance = r.d;
    out.material = r.material;
    for (int i = 0; i < 4; ++i)
        out.traps[i] = r_finite(r.traps[i]) ? r_min(r.traps[i] / R(g.trap_scales[i]), R(1)) : R(1);
    out.iterations = std::min(r.iter, g.iteration_product);
    out.flags = r.flags;
    return out;
}

// ---------------------------------------------------------------- transport
template <class R> static V3<R> v3(const float* f) { return V3<R>(R(f[0]), R(f[1]), R(f[2])); }

template <class R> Scene<R> make_scene(const Graph& g, const sf_scene_desc& d, const sf_render_config& c) {
    Scene<R> s;
    s.cam.origin = v3<R>(d.camera.origin);
    s.cam.forward = v3<R>(d.camera.forward);
    s.cam.right = v3<R>(d.camera.right);
    s.cam.up = v3<R>(d.camera.up);
    s.cam.tan_half = R(d.camera.tan_half_fov);
    s.cam.aspect = R(d.camera.aspect);
    s.cam.lens_radius = R(d.camera.lens_radius);
    s.cam.focus_distance = R(d.camera.focus_distance);
    auto mat = [](const sf_material& m) {
        Mat<R> o;
        o.albedo = v3<R>(m.albedo);
        o.roughness = R(m.roughness);
        o.metallic = R(m.metallic);
        o.specular = R(m.specular);
        o.emission = v3<R>(m.emission);
        return o;
    };
    s.material = mat(d.material);
    s.finish_count = std::min<uint32_t>(d.finish_count, SF_MAX_FINISHES);
    for (uint32_t i = 0; i < s.finish_count; ++i) s.finishes[i] = mat(d.finishes[i]);
    // the scene's lights: light_list (up to 96) when set, else the inline array
    s.light_count = d.light_list ? std::min<uint32_t>(d.light_list_count, SF_MAX_SCENE_LIGHTS)
                                 : std::min<uint32_t>(d.light_count, SF_MAX_LIGHTS);
    for (uint32_t i = 0; i < s.light_count; ++i) {
        const sf_area_light& l = d.light_list ? d.light_list[i] : d.lights[i];
        Light<R>& o = s.lights[i];
        o.kind = l.kind;
        o.color = v3<R>(l.radiance);
        if (l.kind == SF_LIGHT_HDRI) {
            const float r = l.rotation * (3.14159265f / 180.0f);
            o.pano = panorama_find(reinterpret_cast<uint64_t>(l.environment));
            o.a = V3<R>(R(std::cos(r)), R(std::sin(r)), R(o.pano && o.pano->uniform ? 1 : 0));
            o.color = V3<R>(R(l.radiance[0]), 0, 0);
        } else if (l.kind == SF_LIGHT_SUN) {
            // GpuLight::from_light (uniforms.rs:656-668), in binary32 as the reference
            o.a = v3<R>(l.direction);
            o.cos_max = R(std::cos((l.angular_size * 0.5f) * (3.14159265f / 180.0f)));
        } else if (l.kind == SF_LIGHT_ENVIRONMENT) {
            o.a = v3<R>(l.zenith);
            o.b = v3<R>(l.horizon);
            o.c = v3<R>(l.ground);
            auto lum = [](const float* c) { return R(c[0]) * R(0.2126) + R(c[1]) * R(0.7152) + R(c[2]) * R(0.0722); };
            o.energy = r_max(r_max(lum(l.zenith), lum(l.horizon)), lum(l.ground));
            R peak = 0;
            for (int k = 0; k < 3; ++k) peak = r_max(peak, r_max(R(l.zenith[k]), r_max(R(l.horizon[k]), R(l.ground[k]))));
            o.peak = peak;
        } else if (l.kind == SF_LIGHT_TUBE) {
            // GpuLight::from_light (uniforms.rs:717-729): start, end, radius, length
            o.a = v3<R>(l.center);
            o.b = v3<R>(l.edge_u);
            o.radius = R(l.edge_v[0]);
            o.length = (o.b - o.a).length();
        } else {
            // an area light; a projector adds its beam (uniforms.rs:690-715), in binary32
            o.kind = SF_LIGHT_AREA;
            o.a = v3<R>(l.center);
            o.b = v3<R>(l.edge_u);
            o.c = v3<R>(l.edge_v);
            if (l.kind == SF_LIGHT_PROJECTOR) {
                const float deg = 3.14159265f / 180.0f;
                o.projector = true;
                o.beam[0] = R(std::cos(l.direction[0] * deg));
                o.beam[1] = R(std::cos(l.direction[1] * deg));
                o.beam[2] = R(std::tan(l.direction[1] * deg));
            }
        }
    }
    const sf_coloring& col = d.coloring;
    s.coloring.slot = col.slot;
    s.coloring.n = std::min<uint32_t>(col.stop_count, SF_MAX_RAMP_STOPS);
    s.coloring.cyclic = col.cyclic != 0;
    s.coloring.smooth = col.smooth != 0;
    s.coloring.positioned = col.positioned != 0;
    s.coloring.frequency = R(col.frequency);
    s.coloring.phase = R(col.phase);
    s.coloring.gamma = R(col.gamma);
    for (uint32_t i = 0; i < s.coloring.n; ++i) {
        s.coloring.stops[i] = V3<R>(R(col.stops[i][0]), R(col.stops[i][1]), R(col.stops[i][2]));
        s.coloring.pos[i] = R(col.stops[i][3]);
    }
    for (int k = 0; k < 4; ++k) s.col_weights[k] = R(d.coloring_orbit.traps[k]);
    s.col_extra[0] = R(d.coloring_orbit.iterations);
    s.col_extra[1] = R(d.coloring_orbit.normal);
    s.col_extra[2] = R(d.coloring_orbit.logarithmic);
    // finish details and optics (uniforms.rs:797-815, :103-122)
    s.dune_wind = R(d.dune_wind * (3.14159265f / 180.0f));
    for (uint32_t i = 0; i < s.finish_count; ++i) {
        const sf_finish_detail& f = d.details[i];
        Detail<R>& o = s.details[i];
        o.kind = f.pattern;
        o.seed = f.seed;
        o.scale = R(f.scale);
        o.strength = R(f.strength);
        o.bump = R(f.bump);
        o.rough_delta = R(f.roughness_delta);
        o.tint = v3<R>(f.tint);
    }
    for (uint32_t i = 0; i <= s.finish_count; ++i) {
        const sf_optics& o = d.optics[i];
        if (!o.enabled) continue;
        Optics<R>& q = s.optics[i];
        q.surface[0] = R(o.opacity);
        q.surface[1] = R(o.transmission);
        q.surface[2] = R(o.ior);
        q.surface[3] = R(o.thin_walled ? 1 : 0);
        // sigma = -ln(max(c, 1e-4)) / distance in binary32, as GpuOptics packs it
        for (int k = 0; k < 3; ++k)
            q.absorption[k] = R(-std::log(std::max(o.absorption_color[k], 0.0001f)) / o.absorption_distance);
        q.absorption[3] = R(o.absorption_distance);
        for (int k = 0; k < 3; ++k) q.subsurface[k] = R(o.subsurface_color[k]);
        q.subsurface[3] = R(o.subsurface / o.subsurface_radius);
        s.has_optics = true;
    }
    // the texture: on the oracle side sf_texture.graph carries an oracle graph handle
    const sf_texture& t = d.texture;
    if (t.graph) {
        Texture<R>& x = s.tex;
        x.graph = reinterpret_cast<const Graph*>(t.graph);
        x.channel = t.channel;
        x.octaves = t.octaves;
        x.budget = x.graph->iteration_product;
        for (int k = 0; k < 3; ++k) x.mapping[k] = R(t.offset[k]);
        x.mapping[3] = R(t.scale);
        for (int k = 0; k < 3; ++k) x.rotation[k] = R(t.rotation[k] * (3.14159265f / 180.0f));
        x.rotation[3] = R(t.contrast);
        x.effects[0] = R(t.strength);
        x.effects[1] = R(t.roughness);
        x.effects[2] = R(t.bump);
        x.effects[3] = R(1);
        if (t.channel == 7) {
            for (int k = 0; k < 4; ++k) x.weights[k] = R(t.orbit.traps[k]);
            x.extra[0] = R(t.orbit.iterations);
            x.extra[1] = R(t.orbit.normal);
            x.extra[2] = R(t.orbit.logarithmic);
        }
        x.parallax[0] = R(t.parallax);
        x.parallax[1] = R(float(t.parallax_steps));
        if (t.fan) {
            x.fan[0] = R(t.fan_period[0]);
            x.fan[1] = R(t.fan_period[1]);
            x.fan[2] = R(float(t.fan_rays));
            x.fan[3] = R(1);
        }
        if (t.mask) {
            x.mask[0] = R(float(t.mask_slot));
            x.mask[1] = R(t.mask_value);
            x.mask[2] = R(t.mask_width);
            x.mask[3] = R(1);
        }
        const sf_coloring& rc = t.ramp;
        x.ramp.n = std::min<uint32_t>(rc.stop_count, SF_MAX_RAMP_STOPS);
        x.ramp.cyclic = rc.cyclic != 0;
        x.ramp.smooth = rc.smooth != 0;
        x.ramp.positioned = rc.positioned != 0;
        x.ramp.frequency = R(rc.frequency);
        x.ramp.phase = R(rc.phase);
        x.ramp.gamma = R(rc.gamma);
        for (uint32_t i = 0; i < x.ramp.n; ++i) {
            x.ramp.stops[i] = V3<R>(R(rc.stops[i][0]), R(rc.stops[i][1]), R(rc.stops[i][2]));
            x.ramp.pos[i] = R(rc.stops[i][3]);
        }
    }
    s.variation_slot = d.variation_slot;
    s.variation_enabled = d.variation_enabled;
    s.var_rough[0] = R(d.variation_roughness[0]);
    s.var_rough[1] = R(d.variation_roughness[1]);
    s.var_metal[0] = R(d.variation_metallic[0]);
    s.var_metal[1] = R(d.variation_metallic[1]);
    s.cavity = R(d.cavity_darkness);
    s.fog[0] = R(d.fog.density);
    s.fog[1] = R(d.fog.height);
    s.fog[2] = R(d.fog.falloff);
    s.fog[3] = R(d.fog.anisotropy);
    s.fog_color = V3<R>(R(d.fog.color[0]), R(d.fog.color[1]), R(d.fog.color[2]));
    s.seed = uint32_t(d.seed) ^ uint32_t(d.seed >> 32);
    s.pixel_tolerance = R(c.pixel_tolerance);
    s.hit_eps = R(c.hit_epsilon);
    // uniforms.rs:781-782: far = max(2*hint + |origin|, 200), computed in f32.
    float origin_len = sqrtf(d.camera.origin[0] * d.camera.origin[0] + d.camera.origin[1] * d.camera.origin[1] +
                             d.camera.origin[2] * d.camera.origin[2]);
    float far = std::max(2.0f * g.hint + origin_len, 200.0f);
    s.far = R(far);
    s.step_scale = R(g.step_scale);
    s.iteration_product = g.iteration_product;
    s.width = c.width;
    s.height = c.height;
    s.max_bounces = c.max_bounces;
    s.max_steps = c.max_steps;
    return s;
}

// march_segment (pathtrace.wgsl:78-145). absolute_rule selects the fixed-epsilon
// hit test (radius <= eps) used by the primary-ray configuration; otherwise the
// reference's cone-relative test (radius / t < hit_cone).
template <class R>
Hit<R> march_segment(const Graph& g, V3<R> ro, V3<R> rd, R safety, R hit_cone, R t_end, uint32_t max_steps,
                     bool absolute_rule, R eps, uint64_t* de_evals) {
    const R T_MAX = R(200);
    R t = 0, omega = R(1.2), prev_radius = 0, step_len = 0, cand_t = 0, cand_err = R(1e30);
    Sample<R> blank{T_MAX, {1, 1, 1, 1}, 0, 0};
    Sample<R> cand = blank;
    Hit<R> out{false, t_end, 0, blank, false, 0xffffffffu};
    R accept = absolute_rule ? eps : hit_cone;
    for (uint32_t i = 0; i < max_steps; ++i) {
        if (t >= t_end) return out;
        out.steps = i + 1;
        Sample<R> s = evaluate(g, ro + rd * t, true);
        if (de_evals) ++*de_evals;
        R radius = r_abs(s.distance) * safety;
        // a bounding box is only a stepping aid: near acceptance, the exact sample
        if (s.flags != 0 && (absolute_rule ? radius : radius / r_max(t, R(1e-6))) <= accept * R(5)) {
            s = evaluate(g, ro + rd * t, false);
            if (de_evals) ++*de_evals;
            radius = r_abs(s.distance) * safety;
        }
        bool sor_fail = omega > R(1) && (radius + prev_radius) < step_len * R(1.0001);
        if (sor_fail) { step_len = step_len - omega * step_len; omega = 1; }
        else step_len = radius * omega;
        prev_radius = radius;
        R err = absolute_rule ? radius : radius / r_max(t, R(1e-6));
        if (!sor_fail && s.flags == 0 && err < cand_err) { cand_t = t; cand = s; cand_err = err; }
        if (!sor_fail && s.flags == 0 && (absolute_rule ? err <= accept : err < accept)) {
            out.hit = true;
            out.t = t;
            out.sample = s;
            return out;
        }
        if (!sor_fail && t + step_len >= t_end) {
            if (radius >= t_end - t) return out;
            omega = 1;
            step_len = radius;
        }
        t += step_len;
    }
    if (cand_err < accept * R(4)) { out.hit = true; out.t = cand_t; out.sample = cand; }
    else out.exhausted = true;
    return out;
}

// normal_at: tetrahedral 4-tap stencil (common.wgsl:376-387).
template <class R> V3<R> normal_tetra(const Graph& g, V3<R> p, R h) {
    const V3<R> k[4] = {V3<R>(1, -1, -1), V3<R>(-1, -1, 1), V3<R>(-1, 1, -1), V3<R>(1, 1, 1)};
    V3<R> grad(0, 0, 0);
    for (int i = 0; i < 4; ++i) grad = grad + k[i] * evaluate(g, p + k[i] * h, true).distance;
    return normalize(grad);
}
// Central difference, 6 taps (the primary-ray configuration's normal).
template <class R> V3<R> normal_central(const Graph& g, V3<R> p, R h) {
    auto de = [&](V3<R> q) { return evaluate(g, q, true).distance; };
    V3<R> grad(de(p + V3<R>(h, 0, 0)) - de(p - V3<R>(h, 0, 0)), de(p + V3<R>(0, h, 0)) - de(p - V3<R>(0, h, 0)),
               de(p + V3<R>(0, 0, h)) - de(p - V3<R>(0, 0, h)));
    return normalize(grad);
}

static const double PI_W = 3.14159265358979;  // common.wgsl:6
// Lights (lights.wgsl:5-356): rectangles, projectors (a rectangle with a beam) and
// tubes (capsules) are the emitters.
template <class R> static V3<R> area_normal(const Light<R>& l) { return safe_normalize(l.b.cross(l.c)); }
template <class R> static R luminance(V3<R> c) { return c.x * R(0.2126) + c.y * R(0.7152) + c.z * R(0.0722); }
template <class R> static bool is_emitter(const Light<R>& l) { return l.kind == SF_LIGHT_AREA || l.kind == SF_LIGHT_TUBE; }
// beam_profile (lights.wgsl:11-16)
template <class R> static R beam_profile(const Light<R>& l, V3<R> direction) {
    if (!l.projector) return 1;
    const R cosine = area_normal(l).dot(direction);
    const R t = r_clamp((cosine - l.beam[1]) / r_max(l.beam[0] - l.beam[1], R(1e-7)), R(0), R(1));
    return t * t * t * (R(10) + t * (R(-15) + R(6) * t));
}
template <class R> static V3<R> emitter_radiance(const Light<R>& l, V3<R> direction) {
    return l.color * beam_profile(l, direction);
}
// cone_segment (lights.wgsl:23-68); an empty interval is (1, 0)
template <class R>
static void cone_segment(V3<R> ro, V3<R> rd, R end, V3<R> apex, V3<R> axis, R cosine, R* lo, R* hi) {
    R ix = 0, iy = end;
    const V3<R> delta = ro - apex;
    const R axial = delta.dot(axis), slope = rd.dot(axis);
    auto empty = [&]() { *lo = 1; *hi = 0; };
    if (r_abs(slope) < R(1e-8)) {
        if (axial < R(0)) return empty();
    } else {
        const R crossing = -axial / slope;
        if (slope > R(0)) ix = r_max(ix, crossing);
        else iy = r_min(iy, crossing);
    }
    if (iy <= ix) return empty();
    const R c2 = cosine * cosine;
    const R s2 = (R(1) - cosine) * (R(1) + cosine);
    const V3<R> radial = delta - axis * axial;
    const V3<R> radial_slope = rd - axis * slope;
    const R a = s2 * slope * slope - c2 * radial_slope.dot(radial_slope);
    const R b = R(2) * (s2 * axial * slope - c2 * radial.dot(radial_slope));
    const R c = s2 * axial * axial - c2 * radial.dot(radial);
    if (r_abs(a) < R(1e-12)) {
        if (r_abs(b) < R(1e-12)) {
            if (c < R(0)) return empty();
        } else if (b > R(0)) {
            ix = r_max(ix, -c / b);
        } else {
            iy = r_min(iy, -c / b);
        }
        *lo = ix; *hi = iy;
        return;
    }
    const R discriminant = b * b - R(4) * a * c;
    if (discriminant <= R(0)) {
        const R middle = (ix + iy) * R(0.5);
        if ((a * middle + b) * middle + c < R(0)) return empty();
        *lo = ix; *hi = iy;
        return;
    }
    const R root = r_sqrt(discriminant);
    const R q = R(-0.5) * (b + (b >= R(0) ? root : -root));
    const R r0 = q / a, r1 = c / q;
    const R low = r_min(r0, r1), high = r_max(r0, r1);
    if (a < R(0)) { *lo = r_max(ix, low); *hi = r_min(iy, high); return; }
    if (r_min(iy, low) > ix) { *lo = ix; *hi = r_min(iy, low); return; }
    *lo = r_max(ix, high);
    *hi = iy;
}
// projector_bound_apex (lights.wgsl:72-75)
template <class R> static V3<R> projector_bound_apex(const Light<R>& l) {
    const R radius = R(0.5) * (l.b + l.c).length();
    return l.a - area_normal(l) * (radius / l.beam[2]);
}
// emitter_area (lights.wgsl:77-85)
template <class R> static R emitter_area(const Light<R>& l) {
    if (l.kind == SF_LIGHT_TUBE) return R(2) * R(PI_W) * l.radius * (l.length + R(2) * l.radius);
    return l.b.cross(l.c).length();
}
// emitter_normal (lights.wgsl:87-94)
template <class R> static V3<R> emitter_normal(const Light<R>& l, V3<R> point) {
    if (l.kind != SF_LIGHT_TUBE) return area_normal(l);
    const V3<R> axis = l.b - l.a;
    const R t = r_clamp((point - l.a).dot(axis) / axis.dot(axis), R(0), R(1));
    return safe_normalize(point - l.a - axis * t);
}
template <class R> static R area_intersection(V3<R> ro, V3<R> rd, const Light<R>& l) {
    V3<R> n = area_normal(l);
    R den = n.dot(rd);
    if (r_abs(den) < R(1e-7)) return R(1e30);
    R t = (l.a - ro).dot(n) / den;
    if (t <= R(1e-6)) return R(1e30);
    V3<R> q = ro + rd * t - l.a;
    R x = q.dot(l.b) / l.b.dot(l.b);
    R y = q.dot(l.c) / l.c.dot(l.c);
    if (r_abs(x) > R(0.5) || r_abs(y) > R(0.5)) return R(1e30);
    return t;
}
// tube_intersection (lights.wgsl:97-129)
template <class R> static R tube_intersection(V3<R> ro, V3<R> rd, const Light<R>& l) {
    const R r = l.radius, len = l.length;
    const V3<R> axis = (l.b - l.a) / len;
    const V3<R> oa = ro - l.a;
    const R axial_ray = axis.dot(rd), axial_origin = axis.dot(oa);
    const V3<R> side = axis.cross(rd);
    const R a = side.dot(side);
    R nearest = R(1e30);
    if (a > R(1e-10)) {
        const R perpendicular = oa.dot(side) / r_sqrt(a);
        const R h = r * r - perpendicular * perpendicular;
        if (h < R(0)) return nearest;
        const R middle = -(rd.dot(oa) - axial_origin * axial_ray) / a;
        const R root = r_sqrt(r_max(R(0), h) / a);
        for (int i = 0; i < 2; ++i) {
            const R t = middle + (i == 1 ? root : -root);
            const R y = axial_origin + t * axial_ray;
            if (t > R(1e-6) && y >= R(0) && y <= len) nearest = r_min(nearest, t);
        }
    } else {
        const V3<R> radial = oa - axis * axial_origin;
        if (radial.dot(radial) > r * r) return nearest;
    }
    for (int cap = 0; cap < 2; ++cap) {
        const V3<R> oc = ro - (cap == 1 ? l.b : l.a);
        const R projection = oc.dot(rd);
        const V3<R> closest = oc - rd * projection;
        const R h = r * r - closest.dot(closest);
        if (h < R(0)) continue;
        const R sh = r_sqrt(h);
        for (int i = 0; i < 2; ++i) {
            const R t = -projection + (i == 1 ? sh : -sh);
            const R y = (ro + rd * t - l.a).dot(axis);
            const bool on_cap = cap == 1 ? y >= len : y <= R(0);
            if (t > R(1e-6) && on_cap) nearest = r_min(nearest, t);
        }
    }
    return nearest;
}
template <class R> static R emitter_intersection(V3<R> ro, V3<R> rd, const Light<R>& l) {
    return l.kind == SF_LIGHT_TUBE ? tube_intersection(ro, rd, l) : area_intersection(ro, rd, l);
}
template <class R> static void tangent_frame(V3<R> n, V3<R>* t, V3<R>* bt);
// sample_emitter_point (lights.wgsl:143-160)
template <class R> static void sample_emitter_point(const Light<R>& l, R u, R v, R w, V3<R>* position, V3<R>* normal) {
    if (l.kind != SF_LIGHT_TUBE) {
        *position = l.a + l.b * (u - R(0.5)) + l.c * (v - R(0.5));
        *normal = area_normal(l);
        return;
    }
    const V3<R> axis = (l.b - l.a) / l.length;
    V3<R> t, bt;
    tangent_frame(axis, &t, &bt);
    const R phi = R(2) * R(PI_W) * w;
    const V3<R> radial = t * r_cos(phi) + bt * r_sin(phi);
    const R cylinder_fraction = l.length / (l.length + R(2) * l.radius);
    if (u < cylinder_fraction) {
        *position = (l.a * (R(1) - v) + l.b * v) + radial * l.radius;
        *normal = radial;
        return;
    }
    const bool top = (u - cylinder_fraction) / (R(1) - cylinder_fraction) >= R(0.5);
    const V3<R> n = radial * r_sqrt(r_max(R(0), R(1) - v * v)) + axis * (v * (top ? R(1) : R(-1)));
    *position = (top ? l.b : l.a) + n * l.radius;
    *normal = n;
}
// area_weight (lights.wgsl:285-302)
template <class R> static R area_weight(V3<R> p, V3<R> n, const Light<R>& l) {
    const bool tube = l.kind == SF_LIGHT_TUBE;
    R area = emitter_area(l);
    const V3<R> center = tube ? (l.a + l.b) * R(0.5) : l.a;
    V3<R> to_light = center - p;
    R dist2 = r_max(to_light.dot(to_light), R(1e-6));
    V3<R> dir = to_light / r_sqrt(dist2);
    R facing = tube ? R(0.25) : r_max(area_normal(l).dot(-dir), R(0));
    if (l.projector) {
        const V3<R> delta = p - projector_bound_apex(l);
        const R axial = delta.dot(area_normal(l));
        if (axial < R(0) || axial * axial < l.beam[1] * l.beam[1] * delta.dot(delta)) return 0;
        facing = facing * r_max(R(0.025), beam_profile(l, -dir));
    }
    return luminance(l.color) * area * facing * r_max(n.dot(dir), R(0.15)) / dist2;
}
template <class R> static R area_total_weight(const Scene<R>& sc, V3<R> p, V3<R> n) {
    R total = 0;
    for (uint32_t i = 0; i < sc.light_count; ++i)
        if (is_emitter(sc.lights[i])) total += area_weight(p, n, sc.lights[i]);
    return total;
}
template <class R> static R area_direction_pdf(const Light<R>& l, R dist2, R cos_l) {
    return dist2 / r_max(emitter_area(l) * cos_l, R(1e-20));
}
template <class R> static R mis_power(R a, R b) {
    R scale = r_max(a, b);
    if (scale <= R(0)) return 0;
    R pa = a / scale, pb = b / scale;
    return pa * pa / (pa * pa + pb * pb);
}
template <class R> static V3<R> area_emission(const Scene<R>& sc, V3<R> ro, V3<R> rd, R distance, R prev_pdf,
                                              bool use_mis, V3<R> prev_normal, R prev_total) {
    V3<R> L(0, 0, 0);
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        const Light<R>& l = sc.lights[i];
        if (!is_emitter(l)) continue;
        R cos_l = emitter_normal(l, ro + rd * distance).dot(-rd);
        if (cos_l <= R(0)) continue;
        R t = emitter_intersection(ro, rd, l);
        if (r_abs(t - distance) > r_max(R(1e-6), distance * R(1e-6))) continue;
        R w = 1;
        if (use_mis) {
            R pl = area_direction_pdf(l, distance * distance, cos_l);
            R selection = 0;
            if (prev_total > R(0)) selection = area_weight(ro, prev_normal, l) / prev_total;
            pl = pl * selection;
            w = mis_power(prev_pdf, pl);
        }
        L = L + emitter_radiance(l, -rd) * w;
    }
    return L;
}

// BRDF (pathtrace.wgsl:195-249, :394-463).
template <class R> struct Surface { V3<R> n, diffuse, f0; R alpha; V3<R> emission; R diffuse_sigma = 0; };
template <class R> static void tangent_frame(V3<R> n, V3<R>* t, V3<R>* bt) {
    R s = n.z >= R(0) ? R(1) : R(-1);
    R a = R(-1) / (s + n.z);
    R b = n.x * n.y * a;
    *t = V3<R>(R(1) + s * n.x * n.x * a, s * b, -s * n.x);
    *bt = V3<R>(b, s + n.y * n.y * a, -n.y);
}
template <class R> static V3<R> frame_mul(V3<R> t, V3<R> bt, V3<R> n, V3<R> v) { return t * v.x + bt * v.y + n * v.z; }
template <class R> static V3<R> cosine_sample(V3<R> n, R r1, R r2) {
    R phi = R(2) * R(PI_W) * r1;
    R r = r_sqrt(r2);
    V3<R> t, bt;
    tangent_frame(n, &t, &bt);
    return frame_mul(t, bt, n, V3<R>(r * r_cos(phi), r * r_sin(phi), r_sqrt(r_max(R(0), R(1) - r2))));
}
template <class R> static R ggx_d(R nh, R a2) { R d = nh * nh * (a2 - R(1)) + R(1); return a2 / (R(PI_W) * d * d); }
template <class R> static R smith_g1(R nv, R a2) { return R(2) * nv / (nv + r_sqrt(a2 + (R(1) - a2) * nv * nv)); }
template <class R> static V3<R> fresnel(V3<R> f0, R vh) { return f0 + (V3<R>::splat(1) - f0) * r_pow(R(1) - vh, R(5)); }
template <class R> static V3<R> sample_ggx_h(V3<R> n, V3<R> v, R alpha, R r1, R r2) {
    V3<R> t, bt;
    tangent_frame(n, &t, &bt);
    V3<R> lv(t.dot(v), bt.dot(v), n.dot(v));
    V3<R> vh = safe_normalize(V3<R>(alpha * lv.x, alpha * lv.y, r_max(lv.z, R(1e-5))));
    R lensq = vh.x * vh.x + vh.y * vh.y;
    V3<R> t1(1, 0, 0);
    if (lensq > R(0)) t1 = V3<R>(-vh.y, vh.x, 0) / r_sqrt(lensq);
    V3<R> t2 = vh.cross(t1);
    R r = r_sqrt(r1);
    R phi = R(2) * R(PI_W) * r2;
    R x = r * r_cos(phi);
    R blend = R(0.5) * (R(1) + vh.z);
    R y = mixs(r_sqrt(r_max(R(0), R(1) - x * x)), r * r_sin(phi), blend);
    V3<R> nh = t1 * x + t2 * y + vh * r_sqrt(r_max(R(0), R(1) - x * x - y * y));
    return frame_mul(t, bt, n, safe_normalize(V3<R>(alpha * nh.x, alpha * nh.y, r_max(nh.z, R(0)))));
}
template <class R> static V3<R> brdf_eval(const Surface<R>& s, V3<R> v, V3<R> l) {
    R nl = s.n.dot(l), nv = s.n.dot(v);
    if (nl <= R(0) || nv <= R(0)) return V3<R>(0, 0, 0);
    V3<R> h = normalize(v + l);
    R nh = r_max(s.n.dot(h), R(0));
    R vh = r_max(v.dot(h), R(0));
    R a2 = s.alpha * s.alpha;
    V3<R> f = fresnel(s.f0, vh);
    V3<R> spec = f * (ggx_d(nh, a2) * smith_g1(nv, a2) * smith_g1(nl, a2)) / r_max(R(4) * nv * nl, R(1e-4));
    R diffuse_factor = 1;
    if (s.diffuse_sigma > R(0)) {  // Oren-Nayar rough diffuse (pathtrace.wgsl:408-419)
        R sigma2 = s.diffuse_sigma * s.diffuse_sigma;
        R a = R(1) - sigma2 / (R(2) * (sigma2 + R(0.33)));
        R b = R(0.45) * sigma2 / (sigma2 + R(0.09));
        R sin_l = r_sqrt(r_max(R(0), R(1) - nl * nl));
        R sin_v = r_sqrt(r_max(R(0), R(1) - nv * nv));
        R cos_phi = r_max(R(0), (l - s.n * nl).dot(v - s.n * nv) / r_max(sin_l * sin_v, R(1e-8)));
        diffuse_factor = a + b * cos_phi * sin_l * sin_v / r_max(r_max(nl, nv), R(1e-5));
    }
    return s.diffuse * (V3<R>::splat(1) - f) * diffuse_factor / R(PI_W) + spec;
}
template <class R> static R spec_probability(const Surface<R>& s, R nv) {
    V3<R> f = fresnel(s.f0, nv);
    return r_clamp(luminance(f) / r_max(luminance(f) + luminance(s.diffuse), R(1e-4)), R(0.05), R(0.95));
}
template <class R> static R bsdf_pdf(const Surface<R>& s, V3<R> v, V3<R> l, R p_spec) {
    R nl = s.n.dot(l);
    if (nl <= R(0)) return 0;
    V3<R> hh = normalize(v + l);
    R nh = r_max(s.n.dot(hh), R(0));
    R a2 = s.alpha * s.alpha;
    R nv = r_max(s.n.dot(v), R(1e-4));
    R pdf_spec = ggx_d(nh, a2) * smith_g1(nv, a2) / (R(4) * nv);
    return p_spec * pdf_spec + (R(1) - p_spec) * nl / R(PI_W);
}

// make_surface (pathtrace.wgsl:271-386) without texture, detail and phenomena.
// palette_sample (common.wgsl:331-362).
template <class R> static V3<R> ramp_sample(const Coloring<R>& c, R value) {
    const uint32_t n = c.n;
    if (n == 0) return V3<R>(1, 1, 1);
    if (n == 1) return c.stops[0];
    auto mix = [&](uint32_t a, uint32_t b, R amount) {
        R f = r_clamp(amount, R(0), R(1));
        if (c.smooth) f = f * f * (R(3) - R(2) * f);
        return c.stops[a] * (R(1) - f) + c.stops[b] * f;
    };
    R t = value * c.frequency + c.phase;
    if (c.cyclic) t = t - std::floor(t);
    else t = r_clamp(t, R(0), R(1));
    if (c.gamma != R(1)) t = std::pow(t, c.gamma);
    if (!c.positioned && !c.cyclic) {
        R x = t * R(float(n - 1));
        uint32_t i = std::min<uint32_t>(uint32_t(std::floor(x)), n - 2);
        return mix(i, i + 1, x - R(float(i)));
    }
    R first = c.pos[0], last = c.pos[n - 1];
    if (c.cyclic && (t < first || t >= last)) {
        R x = t < first ? t + R(1) : t;
        return mix(n - 1, 0, (x - last) / r_max(R(1) + first - last, R(1e-8)));
    }
    if (t <= first) return c.stops[0];
    if (t >= last) return c.stops[n - 1];
    for (uint32_t i = 0; i + 1 < n; ++i)
        if (t < c.pos[i + 1]) return mix(i, i + 1, (t - c.pos[i]) / (c.pos[i + 1] - c.pos[i]));
    return c.stops[n - 1];
}

// ---------------------------------------------------------------- surface detail
// finish_detail.wgsl (:1-160): value noise with analytic gradients, footprint-filtered.
template <class R> static R smoothstep_r(R e0, R e1, R x) {
    R t = r_clamp((x - e0) / (e1 - e0), R(0), R(1));
    return t * t * (R(3) - R(2) * t);
}
template <class R> static R fract_r(R x) { return x - r_floor(x); }
template <class R> static R sign_r(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
template <class R> struct V4 { V3<R> g; R w; };
template <class R> static V4<R> v4add(V4<R> a, V4<R> b) { return {a.g + b.g, a.w + b.w}; }
template <class R> static V4<R> v4mul(V4<R> a, R s) { return {a.g * s, a.w * s}; }
static float finish_hash(int32_t cx, int32_t cy, int32_t cz, uint32_t seed) {  // :3-7
    uint32_t h = pcg(uint32_t(cx) ^ pcg(uint32_t(cy) + 0x9e3779b9u) ^ pcg(uint32_t(cz) + seed));
    return float(h >> 8u) / 16777216.0f;
}
static int32_t floor_i(double x) {  // WGSL vec3i(floor(p)): saturating conversion
    if (!(x == x)) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return -2147483647 - 1;
    return int32_t(x);
}
template <class R> static V4<R> finish_noise(V3<R> p, uint32_t seed) {  // :8-21
    V3<R> fl(r_floor(p.x), r_floor(p.y), r_floor(p.z));
    int32_t x = floor_i(double(fl.x)), y = floor_i(double(fl.y)), z = floor_i(double(fl.z));
    V3<R> f = p - fl;
    V3<R> t = f * f * (V3<R>::splat(3) - f * R(2));
    V3<R> dt = f * (V3<R>::splat(1) - f) * R(6);
    R a0 = R(finish_hash(x, y, z, seed)), a1 = R(finish_hash(x + 1, y, z, seed));
    R b0 = R(finish_hash(x, y + 1, z, seed)), b1 = R(finish_hash(x + 1, y + 1, z, seed));
    R c0 = R(finish_hash(x, y, z + 1, seed)), c1 = R(finish_hash(x + 1, y, z + 1, seed));
    R d0 = R(finish_hash(x, y + 1, z + 1, seed)), d1 = R(finish_hash(x + 1, y + 1, z + 1, seed));
    R a = mixs(a0, a1, t.x), b = mixs(b0, b1, t.x), c = mixs(c0, c1, t.x), d = mixs(d0, d1, t.x);
    R e = mixs(a, b, t.y), g = mixs(c, d, t.y);
    R dx = mixs(mixs(a1 - a0, b1 - b0, t.y), mixs(c1 - c0, d1 - d0, t.y), t.z);
    return {V3<R>(dx, mixs(b - a, d - c, t.z), g - e) * dt, mixs(e, g, t.z)};
}
template <class R> static V4<R> finish_fbm(V3<R> p, R width, uint32_t seed) {  // :22-33
    R frequency = 1, weight = R(0.5);
    V4<R> result{V3<R>(0, 0, 0), 0};
    for (uint32_t i = 0; i < 3u; ++i) {
        R visible = R(1) - smoothstep_r(R(0.35), R(0.85), width * frequency);
        if (visible > R(0)) {
            V4<R> n = finish_noise(p * frequency, seed + i * 97u);
            result = v4add(result, v4mul(V4<R>{n.g * frequency * visible, mixs(R(0.5), n.w, visible)}, weight));
        } else {
            result.w += weight * R(0.5);
        }
        frequency *= R(2.13);
        weight *= R(0.5);
    }
    return v4mul(result, R(1) / R(0.875));
}
template <class R> static R finish_smooth_derivative(R a, R b, R x) {
    R t = r_clamp((x - a) / (b - a), R(0), R(1));
    return R(6) * t * (R(1) - t) / (b - a);
}
template <class R> static V2<R> rot2(V2<R> v, R a) {
    R s = r_sin(a), c = r_cos(a);
    return V2<R>(c * v.x - s * v.y, s * v.x + c * v.y);
}
// finish_eval (:37-154); the coastal rock's wet band needs an ocean (not on this path).
template <class R> static V4<R> finish_eval(const Detail<R>& f, V3<R> p, R footprint, R wind) {
    const R scale = f.scale;
    const V3<R> q = p * scale;
    const R width = footprint * scale;
    const uint32_t seed = f.seed, kind = f.kind;
    const R PI = R(PI_W);
    if (kind == 12u) {
        V4<R> basin = finish_fbm(q * V3<R>(R(0.31), R(0.31), R(0.22)), width * R(0.31), seed + 911u);
        R wet = smoothstep_r(R(0.47), R(0.59), basin.w);
        V4<R> grit = finish_fbm(q * R(16), width * R(16), seed + 113u);
        R visible = R(1) - smoothstep_r(R(0.15), R(0.6), width * R(3));
        R phase = q.dot(V3<R>(R(2.8), R(0), R(4.1)));
        V3<R> ripple = V3<R>(R(2.8), R(0), R(4.1)) * r_cos(phase) * R(0.018) * visible;
        return {mixv(grit.g * R(16), ripple, wet) * scale, wet};
    }
    if (kind == 10u || kind == 11u) {
        V4<R> stains = finish_fbm(q * R(0.14), width * R(0.14), seed + 17u);
        V4<R> aggregate = finish_fbm(q * R(7), width * R(7), seed + 113u);
        V4<R> pore = finish_noise(q * R(23), seed + 307u);
        R visible = R(1) - smoothstep_r(R(0.25), R(0.75), width * R(23));
        R pit = R(1) - smoothstep_r(R(0.24), R(0.43), pore.w);
        V3<R> pit_gradient = pore.g * (-finish_smooth_derivative(R(0.24), R(0.43), pore.w) * R(23)) * visible;
        R phase = fract_r(q.y / R(1.25) + R(0.5)) - R(0.5);
        R board_visible = R(1) - smoothstep_r(R(0.03), R(0.15), width);
        R joint = (R(1) - smoothstep_r(R(0.006), R(0.027), r_abs(phase))) * board_visible;
        R joint_gradient = -finish_smooth_derivative(R(0.006), R(0.027), r_abs(phase)) * sign_r(phase) / R(1.25) *
                           board_visible;
        R height = R(0.18) * stains.w + R(0.65) * aggregate.w - R(0.14) * mixs(R(0.2), pit, visible) - R(0.09) * joint;
        V3<R> gradient = (stains.g * (R(0.18) * R(0.14)) + aggregate.g * (R(0.65) * R(7)) - pit_gradient * R(0.14) -
                          V3<R>(0, R(0.09) * joint_gradient, 0)) * scale;
        if (kind == 11u) {
            V3<R> axes(R(1.9), R(0.055), R(1.9));
            V4<R> rain = finish_fbm(q * axes, width * R(1.9), seed + 601u);
            R deposit = smoothstep_r(R(0.33), R(0.68), rain.w);
            V3<R> rain_gradient = rain.g * axes * scale * finish_smooth_derivative(R(0.33), R(0.68), rain.w);
            return {gradient + rain_gradient * R(0.12), r_clamp(R(0.72) * deposit + R(0.28) * stains.w, R(0), R(1))};
        }
        return {gradient, r_clamp(height + R(0.12), R(0), R(1))};
    }
    if (kind == 9u) {
        V4<R> wa = finish_fbm(q * R(0.17), width * R(0.17), seed + 17u);
        V4<R> wb = finish_fbm(q * R(0.17), width * R(0.17), seed + 53u);
        V3<R> warped = q + V3<R>(wa.w - R(0.5), R(0), wb.w - R(0.5)) * R(2.8);
        V4<R> cloud = finish_fbm(warped * R(0.16), width * R(0.48), seed + 211u);
        V3<R> axes(R(0.65), R(0.18), R(0.09));
        V4<R> streak = finish_fbm(warped * axes, width * R(1.95), seed + 397u);
        R density = R(0.78) * cloud.w + R(0.22) * streak.w;
        V3<R> g = cloud.g * (R(0.78) * R(0.16)) + axes * streak.g * R(0.22);
        V3<R> density_gradient = (g + (wa.g * g.x + wb.g * g.z) * (R(2.8) * R(0.17))) * scale;
        R deposit = smoothstep_r(R(0.36), R(0.64), density);
        V3<R> deposit_gradient = density_gradient * finish_smooth_derivative(R(0.36), R(0.64), density);
        V4<R> grain = finish_fbm(p * R(48), footprint * R(48), seed + 739u);
        R powder = R(0.85) + R(0.15) * grain.w;
        return {deposit_gradient * powder + grain.g * (deposit * R(0.15) * R(48)), deposit * powder};
    }
    if (kind == 8u) {
        V2<R> xz = rot2(V2<R>(p.x, p.z), wind) * scale;
        V4<R> warp = finish_noise(V3<R>(xz.x * R(0.045), R(0), xz.y * R(0.045)), seed);
        R phase = R(2) * PI * (xz.x + R(1.7) * warp.w + R(0.12) * r_sin(xz.y * R(0.22)));
        R w3 = width * R(3);
        R visible = r_exp(-(w3 * w3));
        R ripple = R(0.5) + R(0.36) * r_sin(phase) + R(0.10) * r_sin(R(2) * phase);
        R amp = R(2) * PI * (R(0.36) * r_cos(phase) + R(0.20) * r_cos(R(2) * phase));
        V2<R> gradient = V2<R>(R(1) + R(0.0765) * warp.g.x, R(0.0264) * r_cos(xz.y * R(0.22)) + R(0.0765) * warp.g.z) *
                         (amp * scale * visible);
        V4<R> grain = finish_fbm(p * R(90), footprint * R(90), seed + 139u);
        V2<R> grad = rot2(gradient, -wind);
        return {V3<R>(grad.x, R(0), grad.y) + grain.g * R(2.5), R(0.70) * mixs(R(0.5), ripple, visible) + R(0.30) * grain.w};
    }
    if (kind == 6u) {
        R tx = fract_r(q.x + R(0.5)) - R(0.5), ty = fract_r(q.z + R(0.5)) - R(0.5);
        R r = r_max(r_sqrt(tx * tx + ty * ty), R(1e-5));
        R angle = r_atan2(ty, tx);
        R flower = r - R(0.25) - R(0.07) * r_cos(angle * R(8));
        R ring = r - R(0.45);
        R ax = -ty / (r * r), ay = tx / (r * r);
        R sf = sign_r(flower), k8 = R(0.56) * r_sin(angle * R(8));
        R gx = sf * (tx / r + k8 * ax), gy = sf * (ty / r + k8 * ay);
        R distance = r_abs(flower);
        if (r_abs(ring) < distance) {
            distance = r_abs(ring);
            gx = sign_r(ring) * tx / r;
            gy = sign_r(ring) * ty / r;
        }
        R visible = R(1) - smoothstep_r(R(0.10), R(0.40), width);
        R carving = R(1) - smoothstep_r(R(0.012), R(0.045), distance);
        R k = -finish_smooth_derivative(R(0.012), R(0.045), distance) * visible * scale;
        return {V3<R>(gx * k, R(0), gy * k), mixs(R(0.2), carving, visible)};
    }
    if (kind == 3u) {
        V3<R> axes(R(18), R(0.45), R(3));
        V4<R> n = finish_fbm(q * axes, width * R(18), seed);
        return {n.g * axes * scale, n.w};
    }
    V4<R> n = finish_fbm(q, width, seed);
    V4<R> result = n;
    if (kind == 1u) {
        V3<R> axis(R(0.16), R(0.11), R(0.08));
        R phase = (q.dot(axis) + n.w * R(2.8)) * PI * R(2);
        R wave = r_sin(phase);
        R veins = R(1) - smoothstep_r(R(0.035), R(0.19), r_abs(wave));
        V3<R> gradient = (axis + n.g * R(2.8)) *
                         (-finish_smooth_derivative(R(0.035), R(0.19), r_abs(wave)) * sign_r(wave) * r_cos(phase) * PI * R(2));
        R visible = R(1) - smoothstep_r(R(0.18), R(0.45), width);
        V4<R> mixed = v4add(v4mul(n, R(0.65)), v4mul(V4<R>{gradient, veins}, R(0.35)));
        result = {mixv(n.g, mixed.g, visible), mixs(n.w, mixed.w, visible)};
    } else if (kind == 2u) {
        result = {n.g * finish_smooth_derivative(R(0.35), R(0.67), n.w), smoothstep_r(R(0.35), R(0.67), n.w)};
    } else if (kind == 4u || kind == 7u) {
        V4<R> grain = finish_fbm(q * R(3.7), width * R(3.7), seed + 53u);
        result = v4add(v4mul(n, R(0.8)), v4mul(V4<R>{grain.g * R(3.7), grain.w}, R(0.2)));
    } else if (kind == 5u) {
        R a = q.x + R(0.75) * n.w;
        R b = q.z * R(1.37) + q.x * R(0.4);
        R visible = R(1) - smoothstep_r(R(0.35), R(1), width);
        V3<R> gradient = ((V3<R>(1, 0, 0) + n.g * R(0.75)) * (R(0.32) * r_cos(a)) +
                          V3<R>(R(0.4), R(0), R(1.37)) * (R(0.18) * r_cos(b))) * visible;
        result = {gradient, R(0.5) + (R(0.32) * r_sin(a) + R(0.18) * r_sin(b)) * visible};
    }
    return {result.g * scale, result.w};
}
template <class R> static V3<R> finish_normal(R bump, V3<R> n, V3<R> gradient) {  // :155-159
    V3<R> slope = gradient - n * gradient.dot(n);
    R limit = R(0.75) / r_max(slope.length(), R(1e-5));
    return safe_normalize(n - slope * r_clamp(bump, -limit, limit));
}
// OrbitColoring::value (material.rs:39-55).
template <class R> static R orbit_mix(const R* w, const R* extra, const R* traps, R iter_frac, R normal_term) {
    R v = w[0] * traps[0] + w[1] * traps[1] + w[2] * traps[2] + w[3] * traps[3] + extra[0] * iter_frac +
          extra[1] * normal_term;
    if (extra[2] > R(0)) v = sign_r(v) * r_log(R(1) + extra[2] * r_abs(v)) / r_log(R(1) + extra[2]);
    return v;
}
// glam Quat::from_euler(XYZ) * p (common.wgsl:263-271): Z, then Y, then X.
template <class R> static V3<R> rotate_xyz(V3<R> p, const R* a) {
    V3<R> q = p;
    q = V3<R>(r_cos(a[2]) * q.x - r_sin(a[2]) * q.y, r_sin(a[2]) * q.x + r_cos(a[2]) * q.y, q.z);
    q = V3<R>(r_cos(a[1]) * q.x + r_sin(a[1]) * q.z, q.y, -r_sin(a[1]) * q.x + r_cos(a[1]) * q.z);
    q = V3<R>(q.x, r_cos(a[0]) * q.y - r_sin(a[0]) * q.z, r_sin(a[0]) * q.y + r_cos(a[0]) * q.z);
    return q;
}
template <class R> static R modf_euclid_r(R x, R m) { return x - m * r_floor(x / m); }
// pattern_value (pattern.wgsl:2-49) of the scene's texture.
template <class R> static R texture_value(const Texture<R>& T, V3<R> p) {
    V3<R> off(T.mapping[0], T.mapping[1], T.mapping[2]);
    const R scale = T.mapping[3];
    V3<R> q = rotate_xyz(p * scale, T.rotation) + off;
    R fan_angle = 0, fan_radius = 0;
    if (T.fan[3] > R(0)) {
        q = rotate_xyz(p, T.rotation) + off;
        R row = r_floor(q.z / T.fan[1]);
        R x = modf_euclid_r(q.x + modf_euclid_r(row, R(2)) * T.fan[0] * R(0.5), T.fan[0]) - T.fan[0] * R(0.5);
        R z = modf_euclid_r(q.z, T.fan[1]) + R(0.03);
        fan_angle = r_atan2(x, z);
        fan_radius = r_sqrt(x * x + z * z);
        q = V3<R>(fan_angle * T.fan[2] / R(PI_W), q.y, fan_radius) * scale;
    }
    const bool orbit = T.channel == 7u;
    const R budget = r_max(R(float(T.budget)), R(1));
    R total = 0, weights = 0, weight = 1;
    for (uint32_t o = 0; o < T.octaves; ++o) {
        Sample<R> smp = evaluate<R>(*T.graph, q);
        R value;
        if (orbit) value = orbit_mix(T.weights, T.extra, smp.traps, R(float(smp.iterations)) / budget, R(0.5));
        else if (T.channel < 4u) value = smp.traps[T.channel];
        else if (T.channel == 4u) value = R(float(smp.iterations)) / budget;
        else value = R(0.5) + R(0.5) * smp.distance / (R(1) + r_abs(smp.distance));
        if (!(value >= -R(3.4028235e38) && value <= R(3.4028235e38))) value = R(0.5);
        total += (orbit ? value : r_clamp(value, R(0), R(1))) * weight;
        weights += weight;
        q = q * R(2) + V3<R>(R(0.73), R(1.17), R(0.91));
        weight *= R(0.5);
    }
    R fractal = total / r_max(weights, R(1e-6));
    R value = fractal;
    if (T.fan[3] > R(0)) {
        R spoke = r_pow(R(1) - r_abs(r_sin(fan_angle * T.fan[2] + R(0.16) * (fractal - R(0.5)))), R(4));
        R arc = r_pow(R(1) - r_abs(r_sin(fan_radius * scale * R(PI_W) + R(0.35) * fractal)), R(6));
        value = R(0.16) + R(0.28) * fractal + R(0.42) * spoke + R(0.22) * arc;
    }
    R result = (value - R(0.5)) * T.rotation[3] + R(0.5);
    return orbit ? result : r_clamp(result, R(0), R(1));
}
template <class R> static R texture_mask(const Texture<R>& T, const R* traps) {  // texture.wgsl:17-21
    if (T.mask[3] == R(0)) return 1;
    return R(1) - smoothstep_r(T.mask[2] * R(0.5), T.mask[2], r_abs(traps[uint32_t(T.mask[0]) & 3u] - T.mask[1]));
}
template <class R> static R texture_filtered_value(const Texture<R>& T, V3<R> p, R footprint) {  // :27-31
    R fade = smoothstep_r(R(0.25), R(0.75), footprint * T.mapping[3]);
    if (fade >= R(1)) return R(0.5);
    return mixs(texture_value(T, p), R(0.5), fade);
}
template <class R> static V3<R> texture_parallax(const Texture<R>& T, V3<R> p, V3<R> n, V3<R> v, R footprint) {  // :35-55
    R depth = T.parallax[0] / T.mapping[3];
    if (depth <= R(0) || depth < footprint * R(0.25)) return p;
    R nv = r_max(n.dot(v), R(0.15));
    V3<R> direction = (v - n * n.dot(v)) / nv + n;
    uint32_t layers = uint32_t(mixs(R(4), T.parallax[1], R(1) - r_clamp(nv, R(0), R(1))));
    uint32_t count = std::max(layers, 4u);
    R step = R(1) / R(float(count));
    R previous = texture_value(T, p) - R(1);
    R layer = 0;
    for (uint32_t i = 0; i < count; ++i) {
        layer += step;
        V3<R> q = p - direction * depth * layer;
        R crossing = layer + texture_value(T, q) - R(1);
        if (crossing >= R(0)) {
            R fraction = r_clamp(-previous / r_max(crossing - previous, R(1e-6)), R(0), R(1));
            return p - direction * depth * (layer - step + step * fraction);
        }
        previous = crossing;
    }
    return p - direction * depth;
}
template <class R> static V3<R> texture_normal(const Texture<R>& T, V3<R> p, V3<R> n, R footprint) {  // :57-72
    R fade = smoothstep_r(R(0.25), R(0.75), footprint * T.mapping[3]);
    if (fade >= R(1)) return n;
    R h = r_max(footprint, R(0.005) / T.mapping[3]);
    V3<R> a(1, -1, -1), b(-1, -1, 1), c(-1, 1, -1), d(1, 1, 1);
    V3<R> gradient = (a * texture_value(T, p + a * h) + b * texture_value(T, p + b * h) + c * texture_value(T, p + c * h) +
                      d * texture_value(T, p + d * h)) / (R(4) * h);
    V3<R> tangent = (gradient - n * n.dot(gradient)) * T.effects[2] * (R(1) - fade) / T.mapping[3];
    tangent = tangent / r_max(R(1), tangent.length());
    return safe_normalize(n - tangent);
}

// make_surface (pathtrace.wgsl:271-386) without the nature phenomena: colouring ramp or
// orbit mix, finish, variation, the finish's detail, the texture on untagged surfaces.
template <class R>
static Surface<R> make_surface(const Scene<R>& sc, V3<R> p, V3<R> n, V3<R> v, const Sample<R>& smp, R footprint) {
    V3<R> albedo = sc.material.albedo;
    bool assigned = smp.material > 0 && smp.material <= sc.finish_count;
    if (!assigned && sc.coloring.n) {  // pathtrace.wgsl:275-288
        const uint32_t slot = sc.coloring.slot;
        const R iter_frac = R(float(smp.iterations)) / r_max(R(float(sc.iteration_product)), R(1));
        if (slot == 6)
            albedo = albedo * ramp_sample(sc.coloring, orbit_mix(sc.col_weights, sc.col_extra, smp.traps, iter_frac,
                                                                 n.y * R(0.5) + R(0.5)));
        else if (slot < 4) albedo = albedo * ramp_sample(sc.coloring, smp.traps[slot]);
        else if (slot == 5) albedo = albedo * ramp_sample(sc.coloring, n.y * R(0.5) + R(0.5));
        else if (slot == 4) albedo = albedo * ramp_sample(sc.coloring, iter_frac);
    }
    R rough = sc.material.roughness, metallic = sc.material.metallic, spec = sc.material.specular;
    V3<R> emission(0, 0, 0);
    if (assigned) {
        const Mat<R>& f = sc.finishes[smp.material - 1];
        albedo = f.albedo;
        rough = f.roughness;
        metallic = f.metallic;
        spec = f.specular;
        emission = f.emission;
    }
    if (!assigned && sc.variation_enabled) {
        R value;
        uint32_t slot = sc.variation_slot;
        if (slot < 4) value = smp.traps[slot];
        else if (slot == 5) value = n.y * R(0.5) + R(0.5);
        else value = R(smp.iterations) / r_max(R(sc.iteration_product), R(1));
        R t = r_clamp(value, R(0), R(1));
        rough = sc.var_rough[0] + (sc.var_rough[1] - sc.var_rough[0]) * t;
        metallic = sc.var_metal[0] + (sc.var_metal[1] - sc.var_metal[0]) * t;
    }
    V3<R> shading_n = n;
    bool rough_diffuse = false;
    if (assigned && sc.details[smp.material - 1].kind != 0u) {  // pathtrace.wgsl:303-340
        const Detail<R>& f = sc.details[smp.material - 1];
        V4<R> detail = finish_eval(f, p, footprint, sc.dune_wind);
        if (f.kind == 9u) detail = v4mul(detail, smoothstep_r(R(0.10), R(0.80), n.y));
        if (f.kind == 12u) detail.w *= smoothstep_r(R(0.45), R(0.95), n.y);
        R value = detail.w;
        R amount = f.strength * value;
        albedo = mixv(albedo, f.tint, amount);
        if (f.kind == 9u) {
            rough += r_max(f.rough_delta, R(0)) * amount;
            metallic *= R(1) - amount;
            spec = mixs(spec, R(0.025), amount);
        } else if (f.kind == 12u) {
            rough = mixs(rough, r_clamp(rough + f.rough_delta, R(0.025), R(1)), amount);
            spec = mixs(spec, R(0.0204), amount);
            metallic *= R(1) - amount;
        } else {
            rough += f.rough_delta * (R(2) * value - R(1));
        }
        if (f.kind == 2u) metallic *= R(1) - R(0.75) * amount;
        if (r_abs(f.bump) > R(0)) shading_n = finish_normal(f.bump, n, detail.g);
        rough_diffuse = f.kind >= 10u;
    }
    const Texture<R>& T = sc.tex;
    if (T.graph) {  // pathtrace.wgsl:345-355
        R amount = texture_mask(T, smp.traps);
        if (!assigned && T.effects[3] > R(0) && amount > R(0)) {
            V3<R> tex_p = texture_parallax(T, p, n, v, footprint);
            R value = texture_filtered_value(T, tex_p, footprint);
            albedo = albedo * mixv(V3<R>::splat(1), ramp_sample(T.ramp, value), T.effects[0] * amount);
            rough = mixs(rough, value, T.effects[1] * amount);
            if (T.effects[2] > R(0)) shading_n = safe_normalize(mixv(n, texture_normal(T, tex_p, n, footprint), amount));
        }
    }
    rough = r_clamp(rough, R(0.02), R(1));
    Surface<R> s;
    s.n = shading_n;
    s.diffuse_sigma = rough_diffuse ? rough * R(0.45) : R(0);
    s.diffuse = albedo * (R(1) - metallic);
    s.f0 = mixv(V3<R>::splat(spec), albedo, metallic);
    s.alpha = rough * rough;
    s.emission = emission;
    return s;
}

// ---------------------------------------------------------------- panoramas
// EnvironmentMap::from_rgb (environment.rs:271-366), restated in double precision.
static std::map<uint64_t, Panorama>& panoramas() {
    static std::map<uint64_t, Panorama> m;
    return m;
}
void panorama_register(uint64_t key, const Panorama& p) { panoramas()[key] = p; }
const Panorama* panorama_find(uint64_t key) {
    auto it = panoramas().find(key);
    return it == panoramas().end() ? nullptr : &it->second;
}
static double pano_cell_area(uint32_t w, uint32_t h, uint32_t row) {
    const double pi = 3.14159265358979323846;
    const double top = pi * row / h, bottom = pi * (row + 1) / h;
    return 2.0 * pi / w * 2.0 * std::sin((top + bottom) * 0.5) * std::sin((bottom - top) * 0.5);
}
bool panorama_tables(const float* rgb, uint32_t width, uint32_t height, Panorama& out) {
    if (!rgb || !width || !height || uint64_t(width) * height > 8192ull * 4096ull) return false;
    for (size_t i = 0; i < size_t(width) * height * 3; ++i)
        if (!std::isfinite(rgb[i])) return false;
    const double pi = 3.14159265358979323846;
    const double scale = std::max({double(width) / 2048.0, double(height) / 1024.0, 1.0});
    const uint32_t ow = uint32_t(std::max(std::floor(width / scale), 1.0));
    const uint32_t oh = uint32_t(std::max(std::floor(height / scale), 1.0));
    out.w = ow;
    out.h = oh;
    out.texels.assign(size_t(ow) * oh * 4, 0.0f);
    for (uint32_t oy = 0; oy < oh; ++oy) {
        const double top = double(oy) * height / oh, bottom = double(oy + 1) * height / oh;
        for (uint32_t ox = 0; ox < ow; ++ox) {
            const double left = double(ox) * width / ow, right = double(ox + 1) * width / ow;
            double sum[3] = {0, 0, 0}, total = 0;
            for (uint32_t iy = uint32_t(std::floor(top)); iy < std::min<uint32_t>(uint32_t(std::ceil(bottom)), height); ++iy) {
                const double lat = std::cos(pi * std::max(top, double(iy)) / height) -
                                   std::cos(pi * std::min(bottom, double(iy + 1)) / height);
                for (uint32_t ix = uint32_t(std::floor(left)); ix < std::min<uint32_t>(uint32_t(std::ceil(right)), width); ++ix) {
                    const double wgt = lat * (std::min(right, double(ix + 1)) - std::max(left, double(ix)));
                    for (int c = 0; c < 3; ++c) sum[c] += double(std::max(rgb[(size_t(iy) * width + ix) * 3 + c], 0.0f)) * wgt;
                    total += wgt;
                }
            }
            for (int c = 0; c < 3; ++c) out.texels[(size_t(oy) * ow + ox) * 4 + c] = float(sum[c] / total);
        }
    }
    const size_t n = size_t(ow) * oh;
    out.uniform = true;
    for (size_t i = 1; i < n && out.uniform; ++i)
        for (int c = 0; c < 3; ++c) out.uniform = out.uniform && out.texels[i * 4 + c] == out.texels[c];
    if (out.uniform) { out.texels[(n - 1) * 4 + 3] = 1.0f; return true; }
    auto lum = [&](size_t i) {
        return double(out.texels[i * 4]) * 0.2126 + double(out.texels[i * 4 + 1]) * 0.7152 + double(out.texels[i * 4 + 2]) * 0.0722;
    };
    std::vector<double> w(n);
    double total = 0;
    const int dd[3] = {-1, 0, 1};
    const double ww[3] = {0.125, 0.75, 0.125};
    for (uint32_t y = 0; y < oh; ++y)
        for (uint32_t x = 0; x < ow; ++x) {
            double acc = 0;
            for (int j = 0; j < 3; ++j) {
                const int row = std::min(std::max(int(y) + dd[j], 0), int(oh) - 1);
                for (int k = 0; k < 3; ++k) {
                    const int col = ((int(x) + dd[k]) % int(ow) + int(ow)) % int(ow);
                    acc += lum(size_t(row) * ow + col) * ww[k] * ww[j];
                }
            }
            w[size_t(y) * ow + x] = acc * pano_cell_area(ow, oh, y);
            total += w[size_t(y) * ow + x];
        }
    double cum = 0;
    for (size_t i = 0; i < n; ++i) {
        cum += total > 0 ? w[i] / total : pano_cell_area(ow, oh, uint32_t(i / ow)) / (4.0 * pi);
        out.texels[i * 4 + 3] = float(std::min(cum, 1.0));
    }
    out.texels[(n - 1) * 4 + 3] = 1.0f;
    return true;
}
// environment.wgsl:7-107.
template <class R> static V3<R> hdri_local(const Light<R>& l, V3<R> d) {
    return V3<R>(l.a.x * d.x + l.a.y * d.z, d.y, -l.a.y * d.x + l.a.x * d.z);
}
template <class R> static V3<R> hdri_world(const Light<R>& l, V3<R> d) {
    return V3<R>(l.a.x * d.x - l.a.y * d.z, d.y, l.a.y * d.x + l.a.x * d.z);
}
template <class R> static void hdri_uv(const Light<R>& l, V3<R> dir, R* u, R* v) {
    V3<R> q = hdri_local(l, dir);
    R x = r_atan2(q.z, q.x) / (R(2) * R(PI_W)) + R(1);
    *u = x - std::floor(x);
    *v = std::acos(r_clamp(q.y, R(-1), R(1))) / R(PI_W);
}
template <class R> static R hdri_cell_area(const Light<R>& l, uint32_t row) {
    R step = R(PI_W) / R(float(l.pano->h));
    return (R(2) * R(PI_W) / R(float(l.pano->w))) * R(2) * r_sin((R(float(row)) + R(0.5)) * step) * r_sin(step * R(0.5));
}
template <class R> static V3<R> hdri_texel(const Light<R>& l, int x, int y) {
    const int w = int(l.pano->w);
    const uint32_t col = uint32_t(((x % w) + w) % w), row = uint32_t(std::min(std::max(y, 0), int(l.pano->h) - 1));
    const float* t = &l.pano->texels[(size_t(row) * l.pano->w + col) * 4];
    return V3<R>(R(t[0]), R(t[1]), R(t[2]));
}
template <class R> static V3<R> hdri_lookup(const Light<R>& l, V3<R> dir) {
    if (!l.pano) return V3<R>(0, 0, 0);
    R u, v;
    hdri_uv(l, dir, &u, &v);
    R px = u * R(float(l.pano->w)) - R(0.5), py = v * R(float(l.pano->h)) - R(0.5);
    R bx = std::floor(px), by = std::floor(py);
    R fx = px - bx, fy = py - by;
    int x = int(bx), y = int(by);
    V3<R> top = mixv(hdri_texel(l, x, y), hdri_texel(l, x + 1, y), fx);
    V3<R> bottom = mixv(hdri_texel(l, x, y + 1), hdri_texel(l, x + 1, y + 1), fx);
    return mixv(top, bottom, fy) * l.color.x;
}
template <class R> static R hdri_pdf(const Light<R>& l, V3<R> dir) {
    const R mix = R(0.0625);
    if (!l.pano || l.a.z > R(0)) return R(1) / (R(4) * R(PI_W));
    R u, v;
    hdri_uv(l, dir, &u, &v);
    const uint32_t col = std::min(uint32_t(u * R(float(l.pano->w))), l.pano->w - 1);
    const uint32_t row = std::min(uint32_t(v * R(float(l.pano->h))), l.pano->h - 1);
    const size_t index = size_t(row) * l.pano->w + col;
    const R before = index > 0 ? R(l.pano->texels[(index - 1) * 4 + 3]) : R(0);
    const R mass = r_max(R(l.pano->texels[index * 4 + 3]) - before, R(0));
    return (R(1) - mix) * mass / hdri_cell_area(l, row) + mix / (R(4) * R(PI_W));
}
template <class R> static V3<R> hdri_sample(const Light<R>& l, R r0, R r1, R r2) {
    const R mix = R(0.0625);
    R phi = R(2) * R(PI_W) * r1;
    R cos_theta = R(1) - R(2) * r2;
    R sin_squared = r_max(R(0), R(1) - cos_theta * cos_theta);
    if (l.pano && l.a.z <= R(0) && r0 >= mix) {
        const R cdf_sample = (r0 - mix) / (R(1) - mix);
        uint32_t lo = 0, hi = l.pano->w * l.pano->h;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2u;
            if (R(l.pano->texels[size_t(mid) * 4 + 3]) <= cdf_sample) lo = mid + 1u;
            else hi = mid;
        }
        const uint32_t index = std::min(lo, l.pano->w * l.pano->h - 1u);
        const uint32_t col = index % l.pano->w, row = index / l.pano->w;
        phi = R(2) * R(PI_W) * (R(float(col)) + r1) / R(float(l.pano->w));
        const R top = R(PI_W) * R(float(row)) / R(float(l.pano->h));
        const R bottom = R(PI_W) * R(float(row + 1)) / R(float(l.pano->h));
        const R band = R(2) * r_sin((top + bottom) * R(0.5)) * r_sin((bottom - top) * R(0.5));
        const R cap = R(2) * r_sin(top * R(0.5)) * r_sin(top * R(0.5)) + r2 * band;
        const R lower_cap = R(2) * r_cos(bottom * R(0.5)) * r_cos(bottom * R(0.5)) + (R(1) - r2) * band;
        if (row < l.pano->h / 2u) { cos_theta = R(1) - cap; sin_squared = cap * (R(2) - cap); }
        else { cos_theta = lower_cap - R(1); sin_squared = lower_cap * (R(2) - lower_cap); }
    }
    const R sin_theta = r_sqrt(r_max(R(0), sin_squared));
    return hdri_world(l, V3<R>(sin_theta * r_cos(phi), cos_theta, sin_theta * r_sin(phi)));
}
template <class R> static V3<R> hdri_emission(const Scene<R>& sc, V3<R> dir, R previous_pdf, bool use_mis) {
    V3<R> L(0, 0, 0);
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        const Light<R>& l = sc.lights[i];
        if (l.kind != SF_LIGHT_HDRI) continue;
        R w = use_mis ? mis_power(previous_pdf, hdri_pdf(l, dir)) : R(1);
        L = L + hdri_lookup(l, dir) * w;
    }
    return L;
}

// Sky lights (pathtrace.wgsl:149-215, :432-468).
template <class R> static V3<R> environment_value(const Light<R>& l, V3<R> dir) {
    if (dir.y >= R(0)) return mixv(l.b, l.a, r_sqrt(dir.y));
    return mixv(l.b, l.c, r_sqrt(-dir.y));
}
template <class R> static R environment_probability(const Light<R>& l, R area_total) {
    if (l.energy <= R(0)) return 0;
    const R e = R(4) * R(PI_W) * l.energy;
    return r_clamp(e / (e + area_total), R(0.05), R(1));
}
template <class R>
static V3<R> environment_emission(const Scene<R>& sc, V3<R> dir, R pdf, bool use_mis, V3<R> n, bool from_volume,
                                  R area_total) {
    V3<R> L(0, 0, 0);
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        const Light<R>& l = sc.lights[i];
        if (l.kind != SF_LIGHT_ENVIRONMENT) continue;
        R w = 1;
        if (use_mis) {
            const R proposal = from_volume ? R(1) / (R(4) * R(PI_W)) : r_max(n.dot(dir), R(0)) / R(PI_W);
            w = mis_power(pdf, environment_probability(l, area_total) * proposal);
        }
        L = L + environment_value(l, dir) * w;
    }
    return L;
}
template <class R> static R sun_pdf(R cos_max) { return R(1) / (R(2) * R(PI_W) * r_max(R(1) - cos_max, R(1e-7))); }
template <class R> static V3<R> sun_radiance(const Scene<R>& sc, V3<R> dir, R pdf_bsdf, bool use_mis) {
    V3<R> L(0, 0, 0);
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        const Light<R>& l = sc.lights[i];
        if (l.kind != SF_LIGHT_SUN || dir.dot(l.a) < l.cos_max) continue;
        R pl = sun_pdf(l.cos_max);
        R w = use_mis ? mis_power(pdf_bsdf, pl) : R(1);
        L = L + l.color * (pl * w);
    }
    return L;
}
template <class R> static V3<R> cone_sample(V3<R> dir, R cos_max, R r1, R r2) {
    R cos_t = R(1) - r1 * (R(1) - cos_max);
    R sin_t = r_sqrt(r_max(R(0), R(1) - cos_t * cos_t));
    R phi = R(2) * R(PI_W) * r2;
    V3<R> t, bt;
    tangent_frame(dir, &t, &bt);
    return t * (sin_t * r_cos(phi)) + bt * (sin_t * r_sin(phi)) + dir * cos_t;
}

// ---------------------------------------------------------------- height fog
// fog_sigma .. fog_free_flight (pathtrace.wgsl:562-615).
template <class R> static R fog_sigma(const Scene<R>& sc, V3<R> p) {
    return sc.fog[0] * r_exp(r_min(R(0), -(p.y - sc.fog[1]) * sc.fog[2]));
}
template <class R> static R fog_segment_tau(const Scene<R>& sc, V3<R> ro, V3<R> rd, R begin, R end) {
    const R distance = r_max(end - begin, R(0));
    if (distance == R(0)) return 0;
    const R sigma = fog_sigma(sc, ro + rd * begin);
    const R mid_height = (ro + rd * ((begin + end) * R(0.5))).y;
    if (mid_height <= sc.fog[1] || sc.fog[2] == R(0)) return sc.fog[0] * distance;
    const R k = rd.y * sc.fog[2];
    const R x = k * distance;
    if (r_abs(x) < R(0.001)) return sigma * distance * (R(1) - x * R(0.5) + x * x / R(6));
    return r_max(R(0), (sigma - fog_sigma(sc, ro + rd * end)) / k);
}
template <class R> static R fog_split(const Scene<R>& sc, V3<R> ro, V3<R> rd, R distance) {
    if (r_abs(rd.y) < R(1e-8)) return distance;
    return r_clamp((sc.fog[1] - ro.y) / rd.y, R(0), distance);
}
template <class R> static R fog_optical_depth(const Scene<R>& sc, V3<R> ro, V3<R> rd, R distance) {
    const R split = fog_split(sc, ro, rd, distance);
    return fog_segment_tau(sc, ro, rd, R(0), split) + fog_segment_tau(sc, ro, rd, split, distance);
}
template <class R> static R fog_transmittance(const Scene<R>& sc, V3<R> ro, V3<R> rd, R distance) {
    return r_exp(-fog_optical_depth(sc, ro, rd, distance));
}
template <class R> static R fog_invert_segment(const Scene<R>& sc, V3<R> ro, V3<R> rd, R begin, R end, R tau) {
    const R sigma = fog_sigma(sc, ro + rd * begin);
    const R k = rd.y * sc.fog[2];
    if ((ro + rd * ((begin + end) * R(0.5))).y <= sc.fog[1] || r_abs(k * (end - begin)) < R(0.0001))
        return r_min(end, begin + tau / r_max(sigma, R(1e-30)));
    if (sigma > R(1e-20)) return r_clamp(begin - r_log(r_max(R(1e-7), R(1) - tau * k / sigma)) / k, begin, end);
    const R remaining = r_max(R(0), fog_segment_tau(sc, ro, rd, begin, end) - tau);
    const R end_sigma = fog_sigma(sc, ro + rd * end);
    return r_clamp(end + r_log(r_max(R(1e-7), R(1) + remaining * k / r_max(end_sigma, R(1e-30)))) / (-k), begin, end);
}
template <class R> static R fog_free_flight(const Scene<R>& sc, V3<R> ro, V3<R> rd, R t_end, uint32_t* rng) {
    if (sc.fog[0] <= R(0)) return t_end;
    const R tau = -r_log(r_max(R(1) - rnd<R>(rng), R(1e-7)));
    const R split = fog_split(sc, ro, rd, t_end);
    const R first = fog_segment_tau(sc, ro, rd, R(0), split);
    const R total = first + fog_segment_tau(sc, ro, rd, split, t_end);
    if (tau >= total) return t_end;
    if (tau < first) return fog_invert_segment(sc, ro, rd, R(0), split, tau);
    return fog_invert_segment(sc, ro, rd, split, t_end, tau - first);
}
// hg_phase, hg_sample (pathtrace.wgsl:717-731).
template <class R> static R hg_phase(R cos_theta, R g) {
    const R d = R(1) + g * g - R(2) * g * cos_theta;
    return (R(1) - g * g) / (R(4) * R(PI_W) * d * r_sqrt(d));
}
template <class R> static V3<R> hg_sample(V3<R> dir, R g, R r1, R r2) {
    R cos_t = R(1) - R(2) * r1;
    if (r_abs(g) > R(1e-3)) {
        const R sq = (R(1) - g * g) / (R(1) - g + R(2) * g * r1);
        cos_t = (R(1) + g * g - sq * sq) / (R(2) * g);
    }
    const R sin_t = r_sqrt(r_max(R(0), R(1) - cos_t * cos_t));
    const R phi = R(2) * R(PI_W) * r2;
    V3<R> t, bt;
    tangent_frame(dir, &t, &bt);
    return t * (sin_t * r_cos(phi)) + bt * (sin_t * r_sin(phi)) + dir * cos_t;
}
// volume_coordinate (pathtrace.wgsl:43-58), computed in f32 as the shader does.
static float volume_coordinate(uint32_t sample_index, uint32_t dimension, uint32_t stream) {
    static const uint32_t bases[6] = {2, 3, 5, 7, 11, 13};
    const uint32_t base = bases[dimension];
    uint32_t index = sample_index + 1u;
    float inverse = 1.0f / float(base);
    float value = 0.0f;
    while (index != 0u) {
        value += float(index % base) * inverse;
        index /= base;
        inverse /= float(base);
    }
    const float shift = float(pcg(stream ^ (dimension * 0x9e3779b9u)) >> 8u) / 16777216.0f;
    const float v = value + shift;
    return v - std::floor(v);
}
// fog_segment_weight (pathtrace.wgsl:621-633) and volume_light_probability
// (lights.wgsl:319-323).
template <class R> static R fog_segment_weight(V3<R> ro, V3<R> rd, R end, const Light<R>& l) {
    const V3<R> center = l.kind == SF_LIGHT_TUBE ? (l.a + l.b) * R(0.5) : l.a;
    R lo = 0, hi = end;
    if (l.projector) {
        cone_segment(ro, rd, end, projector_bound_apex(l), area_normal(l), l.beam[1], &lo, &hi);
        if (hi <= lo) return 0;
    }
    const R along = r_clamp((center - ro).dot(rd), lo, hi);
    const V3<R> delta = center - (ro + rd * along);
    const R area = emitter_area(l);
    return r_max(r_max(l.color.x, l.color.y), l.color.z) * area / (delta.dot(delta) + area);
}
template <class R> static R volume_light_probability(R weight, R total) {
    if (total <= R(0)) return 0;
    return r_min(R(1), R(3) * weight / total);
}

// trace_geometry_lights (lights.wgsl:183-209) around march_segment.
template <class R>
static Hit<R> trace_scene(const Graph& g, const Scene<R>& sc, V3<R> ro, V3<R> rd, R pixel_cone, R t_end, uint64_t* evals) {
    R nearest = t_end;
    uint32_t light_index = 0xffffffffu;
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        if (!is_emitter(sc.lights[i])) continue;
        R t = emitter_intersection(ro, rd, sc.lights[i]);
        if (t < nearest) { nearest = t; light_index = i; }
    }
    // the reference's cone-relative test, or a fixed epsilon when the render states one
    Hit<R> h = march_segment(g, ro, rd, sc.step_scale, pixel_cone * sc.pixel_tolerance, nearest, sc.max_steps,
                             sc.hit_eps > R(0), sc.hit_eps, evals);
    if (!h.hit && !h.exhausted && light_index != 0xffffffffu) {
        h.hit = true;
        h.t = nearest;
        h.light_index = light_index;
    }
    return h;
}

// fog_segment_direct (pathtrace.wgsl:635-715) for rectangles: every area light's
// independent roulette, a point on the segment by one-sample MIS of equiangular and
// optical-depth sampling, a visibility test from there to a point on the light.
// Returns the segment's in-scattered radiance (times the fog colour).
template <class R, class Visible>
static V3<R> fog_segment_direct(const Scene<R>& sc, V3<R> ro, V3<R> rd, R end, uint32_t* rng, uint32_t point_index,
                                uint32_t point_stream, bool primary, Visible&& visible) {
    V3<R> result(0, 0, 0);
    if (end <= R(0) || r_max(r_max(sc.fog_color.x, sc.fog_color.y), sc.fog_color.z) <= R(0)) return result;
    const R tau_end = fog_optical_depth(sc, ro, rd, end);
    if (tau_end <= R(0)) return result;
    R total = 0;
    for (uint32_t i = 0; i < sc.light_count; ++i)
        if (is_emitter(sc.lights[i])) total += fog_segment_weight(ro, rd, end, sc.lights[i]);
    const R g = sc.fog[3];
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        const Light<R>& l = sc.lights[i];
        if (!is_emitter(l)) continue;
        const R probability = volume_light_probability(fog_segment_weight(ro, rd, end, l), total);
        const uint32_t stream = pcg(point_stream ^ (i * 0x85ebca6bu));
        R selection = rnd<R>(rng);
        if (primary) selection = R(volume_coordinate(point_index, 5, stream));
        if (probability <= R(0) || selection >= probability) continue;
        // sample_emitter draws two numbers for a rectangle, three for a tube
        R u1 = rnd<R>(rng);
        R u2 = rnd<R>(rng);
        R u3 = l.kind == SF_LIGHT_TUBE ? rnd<R>(rng) : R(0);
        if (primary) {
            u1 = R(volume_coordinate(point_index, 0, stream));
            u2 = R(volume_coordinate(point_index, 1, stream));
            u3 = R(volume_coordinate(point_index, 2, stream));
        }
        V3<R> q, qn;
        sample_emitter_point(l, u1, u2, u3, &q, &qn);
        R lo = 0, hi = end;
        if (l.projector) {
            cone_segment(ro, rd, end, q, area_normal(l), l.beam[1], &lo, &hi);
            if (hi <= lo) continue;
        }
        const R tau_begin = fog_optical_depth(sc, ro, rd, lo);
        const R tau_finish = fog_optical_depth(sc, ro, rd, hi);
        const R tau_span = r_max(R(0), tau_finish - tau_begin);
        if (tau_span <= R(0)) continue;
        R conditional_mass = R(1) - r_exp(-tau_span);
        if (tau_span < R(0.001)) conditional_mass = tau_span * (R(1) - tau_span * R(0.5) + tau_span * tau_span / R(6));
        const R interval_mass = r_exp(-tau_begin) * conditional_mass;
        if (interval_mass < R(1e-30)) continue;
        const V3<R> delta = q - ro;
        const R projection = delta.dot(rd);
        const R perpendicular = (delta - rd * projection).length();
        const R theta_a = r_atan2(lo - projection, r_max(perpendicular, R(1e-6)));
        const R theta_b = r_atan2(hi - projection, r_max(perpendicular, R(1e-6)));
        const R span = theta_b - theta_a;
        const bool regular = perpendicular > R(1e-4) && span > R(1e-5);
        R xi = rnd<R>(rng);
        R technique = rnd<R>(rng);
        if (primary) {
            xi = R(volume_coordinate(point_index, 3, stream));
            technique = R(volume_coordinate(point_index, 4, stream));
        }
        R t = lo * (R(1) - xi) + hi * xi;  // mix(lo, hi, xi)
        if (technique < R(0.5)) {
            if (regular)
                t = r_clamp(projection + perpendicular * r_tan(theta_a * (R(1) - xi) + theta_b * xi), lo, hi);
        } else {
            const R tau = tau_begin - r_log(r_max(R(1) - xi * conditional_mass, R(1e-7)));
            const R split = fog_split(sc, ro, rd, hi);
            const R first = fog_segment_tau(sc, ro, rd, R(0), split);
            t = tau < first ? fog_invert_segment(sc, ro, rd, R(0), split, tau)
                            : fog_invert_segment(sc, ro, rd, split, hi, tau - first);
        }
        const V3<R> p = ro + rd * t;
        const R transmittance = r_exp(-fog_optical_depth(sc, ro, rd, t));
        const R sigma = fog_sigma(sc, p);
        R angular_pdf = R(1) / (hi - lo);
        if (regular)
            angular_pdf = perpendicular / (span * (perpendicular * perpendicular + (t - projection) * (t - projection)));
        const R distance_pdf = R(0.5) * (angular_pdf + sigma * transmittance / interval_mass);
        const V3<R> to_light = q - p;
        const R distance2 = to_light.dot(to_light);
        if (distance2 < R(1e-8)) continue;
        const R distance = r_sqrt(distance2);
        const V3<R> wi = to_light / distance;
        const R cosine = qn.dot(-wi);
        if (cosine <= R(0)) continue;
        const R vw = visible(p, wi, r_max(R(0), distance - r_max(R(1e-5), distance * R(1e-6))));
        if (!(vw > R(0))) continue;
        const R tr = vw * transmittance * r_exp(-fog_optical_depth(sc, p, wi, distance));
        result = result + emitter_radiance(l, -wi) * (sigma * tr * hg_phase(rd.dot(wi), g) /
                                     (probability * distance_pdf * area_direction_pdf(l, distance2, cosine)));
    }
    return result * sc.fog_color;
}
// fog_direct_light (pathtrace.wgsl:733-772): a scattering point's next events for the
// sky lights, phase function in place of the BRDF.
template <class R, class Visible>
static V3<R> fog_direct_light(const Scene<R>& sc, V3<R> p, V3<R> rd, R area_total, bool last, uint32_t* rng,
                              Visible&& visible) {
    const R g = sc.fog[3];
    const R extent = r_max(R(200), sc.far);
    V3<R> L(0, 0, 0);
    for (uint32_t i = 0; i < sc.light_count; ++i) {
        const Light<R>& l = sc.lights[i];
        if (l.kind == SF_LIGHT_ENVIRONMENT) {
            if (l.peak <= R(0)) continue;
            const R probability = environment_probability(l, area_total);
            if (rnd<R>(rng) >= probability) continue;
            const R z = R(1) - R(2) * rnd<R>(rng);
            const R phi = R(2) * R(PI_W) * rnd<R>(rng);
            const R radius = r_sqrt(r_max(R(0), R(1) - z * z));
            const V3<R> dir(radius * r_cos(phi), z, radius * r_sin(phi));
            const R vw = visible(p, dir, extent);
            if (!(vw > R(0))) continue;
            const R tr = vw * fog_transmittance(sc, p, dir, extent);
            const R ph = hg_phase(rd.dot(dir), g);
            const R pl = probability / (R(4) * R(PI_W));
            L = L + environment_value(l, dir) * ph * tr * (last ? R(1) : mis_power(pl, ph)) / pl;
        } else if (l.kind == SF_LIGHT_HDRI) {
            if (l.color.x <= R(0)) continue;
            const R r0 = rnd<R>(rng);
            const R r1 = rnd<R>(rng);
            const R r2 = rnd<R>(rng);
            const V3<R> dir = hdri_sample(l, r0, r1, r2);
            const R vw = visible(p, dir, extent);
            if (!(vw > R(0))) continue;
            const R tr = vw * fog_transmittance(sc, p, dir, extent);
            const R ph = hg_phase(rd.dot(dir), g);
            const R pl = hdri_pdf(l, dir);
            L = L + hdri_lookup(l, dir) * ph * tr * (last ? R(1) : mis_power(pl, ph)) / pl;
        } else if (l.kind == SF_LIGHT_SUN) {
            const R r1 = rnd<R>(rng);
            const R r2 = rnd<R>(rng);
            const V3<R> dir = cone_sample(l.a, l.cos_max, r1, r2);
            const R vw = visible(p, dir, extent);
            if (!(vw > R(0))) continue;
            const R tr = vw * fog_transmittance(sc, p, dir, extent);
            const R ph = hg_phase(rd.dot(dir), g);
            const R pl = sun_pdf(l.cos_max);
            L = L + l.color * ph * tr * (last ? R(1) : mis_power(pl, ph));
        }
    }
    return L;
}

// ---------------------------------------------------------------- optics (optics.wgsl)
template <class R> static const Optics<R>& material_optics(const Scene<R>& sc, uint32_t index) {  // :1-3
    return sc.optics[index <= sc.finish_count ? index : 0u];
}
template <class R> static bool optics_on(const Optics<R>& o) { return o.absorption[3] > R(0); }
// optical_refine_hit (:7-23): Newton steps along the ray on the exact field.
template <class R> static R optical_refine(const Graph& g, V3<R> ro, V3<R> rd, R t, uint64_t* evals) {
    const R eps = r_max(R(1e-5), r_min(R(1e-3), t * R(1e-5)));
    for (uint32_t i = 0; i < 8u; ++i) {
        V3<R> p = ro + rd * t;
        R d = evaluate<R>(g, p).distance;
        *evals += 1;
        if (r_abs(d) < R(1e-5)) break;
        R derivative = (evaluate<R>(g, p + rd * eps).distance - evaluate<R>(g, p - rd * eps).distance) / (R(2) * eps);
        *evals += 2;
        if (r_abs(derivative) < R(1e-5)) break;
        t = r_max(R(0), t - r_clamp(d / derivative, R(-0.5), R(0.5)));
    }
    return t;
}
// ocean_fresnel (ocean.wgsl:151-159).
template <class R> static R dielectric_fresnel(R cosine, R eta) {
    R ci = r_clamp(r_abs(cosine), R(0), R(1));
    R st2 = eta * eta * (R(1) - ci * ci);
    if (st2 >= R(1)) return 1;
    R ct = r_sqrt(r_max(R(0), R(1) - st2));
    R rs = (eta * ci - ct) / r_max(eta * ci + ct, R(1e-6));
    R rp = (ci - eta * ct) / r_max(ci + eta * ct, R(1e-6));
    return R(0.5) * (rs * rs + rp * rp);
}
template <class R> static V3<R> refract_w(V3<R> i, V3<R> n, R eta) {  // WGSL refract
    R ni = n.dot(i);
    R k = R(1) - eta * eta * (R(1) - ni * ni);
    if (k < R(0)) return V3<R>(0, 0, 0);
    return i * eta - n * (eta * ni + r_sqrt(k));
}
template <class R> static V3<R> reflect_w(V3<R> i, V3<R> n) { return i - n * (R(2) * n.dot(i)); }
template <class R> static V3<R> exp_v(V3<R> a) { return V3<R>(r_exp(a.x), r_exp(a.y), r_exp(a.z)); }
template <class R> struct OpticalBounce { V3<R> direction, weight; bool transmitted, valid; };
// optical_bounce (:30-64) without dispersion or thin-film coating.
template <class R>
static OpticalBounce<R> optical_bounce(const Optics<R>& o, V3<R> n, V3<R> rd, R alpha, bool entering, uint32_t* rng) {
    const R index = o.surface[2];
    const bool thin = o.surface[3] > R(0);
    const V3<R> tint = exp_v(V3<R>(-o.absorption[0], -o.absorption[1], -o.absorption[2]) * o.absorption[3]);
    if (index <= R(1.0001)) return {rd, thin ? tint : V3<R>::splat(1), true, true};
    const R eta = (entering || thin) ? R(1) / index : index;
    const R r1 = rnd<R>(rng);
    const R r2 = rnd<R>(rng);
    const V3<R> h = sample_ggx_h(n, -rd, alpha, r1, r2);
    R f = dielectric_fresnel(r_max(R(0), (-rd).dot(h)), eta);
    if (thin) f = R(2) * f / (R(1) + f);
    V3<R> color = V3<R>::splat(f);
    R probability = f;
    const V3<R> transmitted = refract_w(rd, h, eta);
    if (!thin && transmitted.dot(transmitted) < R(0.5)) {
        color = V3<R>::splat(1);
        probability = 1;
    }
    const R a2 = alpha * alpha;
    if (rnd<R>(rng) < probability) {
        V3<R> direction = reflect_w(rd, h);
        R cosine = n.dot(direction);
        return {direction, color / r_max(probability, R(1e-20)) * smith_g1(r_max(cosine, R(1e-6)), a2), false,
                cosine > R(0)};
    }
    V3<R> direction = thin ? rd : transmitted;
    R cosine = -n.dot(direction);
    V3<R> weight = thin ? tint : V3<R>::splat(smith_g1(r_max(cosine, R(1e-6)), a2) * eta * eta);
    weight = weight * (V3<R>::splat(1) - color) / r_max(R(1) - probability, R(1e-20));
    return {direction, weight, true, cosine > R(0) && direction.dot(direction) > R(0.5)};
}

// radiance (pathtrace.wgsl:802-1201) with the height fog, finish details, textures and optics, and with ocean,
// portals, nebulae, guiding and the nature phenomena disabled (those branches are identities when off),
// camera_ray (:781-800) and the per-sample film terms of main (:1203-1276).
template <class R> PixelResult radiance(const Graph& g, const Scene<R>& sc, uint32_t px, uint32_t py, uint32_t sample) {
    PixelResult res{};
    uint32_t rng = rng_init(px, py, sample, sc.seed);
    R pixel_cone = sc.cam.tan_half * R(2) / R(float(sc.width));
    // camera_ray
    R jx = rnd<R>(&rng);
    R jy = rnd<R>(&rng);
    R ndcx = ((R(float(px)) + jx) / R(float(sc.width))) * R(2) - R(1);
    R ndcy = ((R(float(py)) + jy) / R(float(sc.height))) * R(2) - R(1);
    V3<R> dir = normalize(sc.cam.forward + sc.cam.right * (ndcx * sc.cam.tan_half) +
                          sc.cam.up * (-ndcy * sc.cam.tan_half / sc.cam.aspect));
    V3<R> origin = sc.cam.origin;
    if (sc.cam.lens_radius > R(0)) {
        V3<R> focus = origin + dir * (sc.cam.focus_distance / r_max(dir.dot(sc.cam.forward), R(1e-4)));
        R r = sc.cam.lens_radius * r_sqrt(rnd<R>(&rng));
        R phi = R(2) * R(PI_W) * rnd<R>(&rng);
        origin = origin + sc.cam.right * (r * r_cos(phi)) + sc.cam.up * (r * r_sin(phi));
        dir = normalize(focus - origin);
    }
    V3<R> ro = origin, rd = dir;
    V3<R> throughput(1, 1, 1), L(0, 0, 0);
    V3<R> primary_volume(0, 0, 0);  // the camera segment's in-scattered light (pathtrace.wgsl:821-822)
    bool volume_path = false;        // the camera segment scattered in the fog
    R prev_pdf = 0, prev_area_total = 0;
    bool prev_from_bsdf = false;
    V3<R> prev_normal(0, 0, 0);
    bool prev_from_volume = false;  // prev_volume_nee is the same flag without ocean and nebulae
    const uint32_t point_stream = pcg(pcg(px ^ sc.seed) ^ pcg(py ^ 0x27d4eb2du));
    // the transported texture footprint (pathtrace.wgsl:811-814) and the optics state
    R tex_width = 0, tex_spread = pixel_cone * R(0.5);
    bool solid_medium = false;
    uint32_t medium_slot = 0, null_surfaces = 0;
    const bool in_fog = sc.fog[0] > R(0);
    const bool optics = sc.has_optics;
    if (optics) {  // the medium the camera ray starts in (:833-840)
        const Sample<R> init = evaluate<R>(g, ro);
        res.de_evals++;
        const Optics<R>& o = material_optics(sc, init.material);
        solid_medium = init.distance < R(0) && optics_on(o) && o.surface[1] > R(0) && o.surface[3] == R(0);
        medium_slot = init.material;
    }
    // scene_visibility_weight (lights.wgsl:260-283): with optics, surfaces of dielectric
    // materials pass the segment weighted by 1 - opacity, up to 32 segments
    auto visible_from = [&](V3<R> o, V3<R> dir, R t_end) -> R {
        if (!optics) {
            Hit<R> sh = trace_scene(g, sc, o, dir, pixel_cone, t_end, &res.de_evals);
            res.segments++;
            return (!sh.hit && !sh.exhausted) ? R(1) : R(0);
        }
        V3<R> origin = o;
        R remaining = t_end, visibility = 1;
        for (uint32_t i = 0; i < 32u; ++i) {
            Hit<R> sh = trace_scene(g, sc, origin, dir, pixel_cone, remaining, &res.de_evals);
            res.segments++;
            if (sh.hit && sh.light_index == 0xffffffffu && optics_on(material_optics(sc, sh.sample.material))) {
                sh.t = optical_refine(g, origin, dir, sh.t, &res.de_evals);
                sh.sample = evaluate<R>(g, origin + dir * sh.t);
                res.de_evals++;
            }
            if (sh.exhausted) return 0;
            if (!sh.hit) return visibility;
            if (sh.light_index != 0xffffffffu) return 0;
            const Optics<R>& oo = material_optics(sc, sh.sample.material);
            if (!optics_on(oo)) return 0;
            visibility *= R(1) - oo.surface[0];
            if (visibility < R(1e-6)) return 0;
            const R distance = sh.t + R(1e-4);
            origin = origin + dir * distance;
            remaining -= distance;
            if (remaining <= R(0)) return visibility;
        }
        return 0;
    };
    R first_depth = -1;
    R aux[4] = {0, 0, 0, -1};
    R extent = r_max(R(200), sc.far);
    for (uint32_t bounce = 0; bounce <= sc.max_bounces;) {
        Hit<R> h = trace_scene(g, sc, ro, rd, pixel_cone, extent, &res.de_evals);
        res.segments++;
        bool refined = false;  // a hit on a dielectric material: optical_refine_hit (optics.wgsl:7-23)
        if (optics && h.hit && h.light_index == 0xffffffffu && optics_on(material_optics(sc, h.sample.material))) {
            h.t = optical_refine(g, ro, rd, h.t, &res.de_evals);
            h.sample = evaluate<R>(g, ro + rd * h.t);
            res.de_evals++;
            refined = true;
        }
        if (optics && solid_medium) {  // inside a dielectric solid (pathtrace.wgsl:857-875)
            const Optics<R>& medium = material_optics(sc, medium_slot);
            R distance = h.t;
            if (medium.subsurface[3] > R(0))
                distance = r_min(h.t, -r_log(r_max(R(1e-7), R(1) - rnd<R>(&rng))) / medium.subsurface[3]);
            throughput = throughput * exp_v(V3<R>(-medium.absorption[0], -medium.absorption[1], -medium.absorption[2]) *
                                            distance);
            if (distance < h.t) {
                if (bounce == sc.max_bounces) break;
                throughput = throughput * V3<R>(medium.subsurface[0], medium.subsurface[1], medium.subsurface[2]);
                const R r1 = rnd<R>(&rng);
                const R r2 = rnd<R>(&rng);
                ro = ro + rd * distance;
                rd = hg_sample(rd, R(0), r1, r2);
                prev_from_bsdf = false;
                prev_from_volume = false;
                prev_pdf = 0;
                tex_spread = r_max(tex_spread, R(0.25));
                bounce++;
                continue;
            }
        }
        V3<R> gn(0, 0, 0);
        if (h.hit) {
            if (h.light_index != 0xffffffffu) gn = emitter_normal(sc.lights[h.light_index], ro + rd * h.t);
            else {
                const bool optical = refined && optics_on(material_optics(sc, h.sample.material));
                gn = normal_tetra(g, ro + rd * h.t,
                                  optical ? R(1e-4) : r_max(h.t * pixel_cone * R(0.5), R(1e-4)) * sc.pixel_tolerance);
                res.de_evals += 4;
            }
            if (bounce == 0) { first_depth = h.t; aux[0] = gn.x; aux[1] = gn.y; aux[2] = gn.z; aux[3] = R(h.steps); }
        }
        if (in_fog && !solid_medium) {  // pathtrace.wgsl:980-1011
            const R t_end = h.hit ? h.t : extent;
            const V3<R> direct_volume = throughput * fog_segment_direct(sc, ro, rd, t_end, &rng, sample, point_stream,
                                                                        bounce == 0 && null_surfaces == 0, visible_from);
            L = L + direct_volume;
            if (bounce == 0) primary_volume = primary_volume + direct_volume;
            const R t_s = fog_free_flight(sc, ro, rd, t_end, &rng);
            if (t_s < t_end) {
                if (bounce == 0) volume_path = true;
                tex_width += t_s * tex_spread;
                tex_spread = r_max(tex_spread, R(0.25));
                if (bounce == 0 && !h.hit) first_depth = t_s;
                const V3<R> p_s = ro + rd * t_s;
                const R volume_area_total = area_total_weight(sc, p_s, V3<R>(0, 0, 0));
                const bool last = bounce == sc.max_bounces;
                L = L + throughput * sc.fog_color *
                            fog_direct_light(sc, p_s, rd, volume_area_total, last, &rng, visible_from);
                throughput = throughput * sc.fog_color;
                if (last) break;
                const R r1 = rnd<R>(&rng);
                const R r2 = rnd<R>(&rng);
                const V3<R> nd = hg_sample(rd, sc.fog[3], r1, r2);
                prev_pdf = hg_phase(rd.dot(nd), sc.fog[3]);
                prev_from_bsdf = true;
                prev_from_volume = true;
                prev_normal = V3<R>(0, 0, 0);
                prev_area_total = volume_area_total;
                ro = p_s;
                rd = nd;
                bounce++;
                continue;
            }
        }
        if (!h.hit) {  // the sky, the panoramas, the suns (pathtrace.wgsl:1026-1040)
            if (!h.exhausted) {
                L = L + throughput * environment_emission(sc, rd, prev_pdf, prev_from_bsdf, prev_normal,
                                                          prev_from_volume, prev_area_total);
                L = L + throughput * hdri_emission(sc, rd, prev_pdf, prev_from_bsdf);
                L = L + throughput * sun_radiance(sc, rd, prev_pdf, prev_from_bsdf);
            }
            break;
        }
        V3<R> p = ro + rd * h.t;
        if (h.light_index != 0xffffffffu) {
            if (bounce == 0) {
                first_depth = h.t;
                V3<R> en = emitter_normal(sc.lights[h.light_index], ro + rd * h.t);
                aux[0] = en.x; aux[1] = en.y; aux[2] = en.z; aux[3] = R(h.steps);
            }
            // after a fog scattering point its segment estimate already holds the emitters
            if (!prev_from_volume)
                L = L + throughput * area_emission(sc, ro, rd, h.t, prev_pdf, prev_from_bsdf, prev_normal,
                                                   prev_area_total);
            break;
        }
        V3<R> n = gn;
        const Optics<R>& hit_optics = material_optics(sc, h.sample.material);
        const bool optical = optics && optics_on(hit_optics);
        const bool entering = rd.dot(gn) < R(0);
        if (optical && !entering) n = -n;
        if (optical && hit_optics.surface[0] < R(1) && rnd<R>(&rng) >= hit_optics.surface[0]) {
            // a coverage null event (pathtrace.wgsl:1058-1065): the same bounce continues past it
            null_surfaces++;
            if (null_surfaces > 32u) break;
            ro = p + rd * r_max(h.t * pixel_cone * R(0.15) * sc.pixel_tolerance, R(1e-4));
            if (bounce == 0) { first_depth = -1; aux[0] = aux[1] = aux[2] = 0; aux[3] = -1; }
            continue;
        }
        if (bounce == 0) {
            first_depth = h.t;
            aux[0] = n.x; aux[1] = n.y; aux[2] = n.z; aux[3] = R(h.steps);
            R x = r_clamp(R(float(h.steps)) / R(96), R(0), R(1));
            throughput = throughput * (R(1) - sc.cavity * (x * x * (R(3) - R(2) * x)));
        }
        V3<R> v = -rd;
        tex_width += h.t * tex_spread;
        Surface<R> s = make_surface(sc, p, n, v, h.sample, r_max(tex_width, R(1e-4)));
        L = L + throughput * s.emission;
        R offset = r_max(h.t * pixel_cone * R(2), R(1e-3)) * sc.pixel_tolerance;
        if (optical && hit_optics.surface[1] > R(0) && rnd<R>(&rng) < hit_optics.surface[1]) {
            // the dielectric lobe (pathtrace.wgsl:1088-1107)
            if (bounce == sc.max_bounces) break;
            const OpticalBounce<R> b = optical_bounce(hit_optics, n, rd, s.alpha, entering, &rng);
            if (!b.valid) break;
            throughput = throughput * b.weight;
            const R bias = r_max(R(1e-4), r_min(offset, R(0.001)));
            ro = p + b.direction * bias;
            rd = b.direction;
            if (b.transmitted && hit_optics.surface[3] == R(0)) {
                solid_medium = entering;
                medium_slot = h.sample.material;
            }
            prev_from_bsdf = false;
            prev_from_volume = false;
            prev_pdf = 0;
            tex_spread = r_max(tex_spread, s.alpha * R(0.1));
            bounce++;
            continue;
        }
        V3<R> p_off = p + n * offset;
        R nv = r_max(s.n.dot(v), R(1e-4));
        R p_spec = spec_probability(s, nv);
        R area_total = area_total_weight(sc, p_off, s.n);
        bool last = bounce == sc.max_bounces;
        // direct_light (pathtrace.wgsl:471-558): the area light selected by weight,
        // then every light in scene order; each clear shadow segment adds its radiance.
        {
            uint32_t selected = 0xffffffffu;
            R selected_weight = 0;
            if (area_total > R(0)) {
                R threshold = rnd<R>(&rng) * area_total;
                R sum = 0;
                for (uint32_t i = 0; i < sc.light_count; ++i) {
                    if (!is_emitter(sc.lights[i])) continue;
                    R w = area_weight(p_off, s.n, sc.lights[i]);
                    sum += w;
                    if (w > R(0)) {
                        selected = i;
                        selected_weight = w;
                        if (threshold < sum) break;
                    }
                }
            }
            auto visible = [&](V3<R> dir, R t_end) { return visible_from(p_off, dir, t_end); };
            // direct_light's fog transmittance toward each light (pathtrace.wgsl:501-549)
            auto fog_tr = [&](V3<R> dir, R dist) {
                return (in_fog && !solid_medium) ? fog_transmittance(sc, p_off, dir, dist) : R(1);
            };
            for (uint32_t i = 0; i < sc.light_count; ++i) {
                const Light<R>& l = sc.lights[i];
                if (l.kind == SF_LIGHT_ENVIRONMENT) {
                    if (l.peak <= R(0)) continue;
                    R probability = environment_probability(l, area_total);
                    if (rnd<R>(&rng) >= probability) continue;
                    R r1 = rnd<R>(&rng);
                    R r2 = rnd<R>(&rng);
                    V3<R> ldir = cosine_sample(s.n, r1, r2);
                    R nl = r_max(s.n.dot(ldir), R(0));
                    if (n.dot(ldir) <= R(0) || nl <= R(0)) continue;
                    const R vw = visible(ldir, extent);
                    if (!(vw > R(0))) continue;
                    R pl = probability * nl / R(PI_W);
                    R pb = last ? R(0) : bsdf_pdf(s, v, ldir, p_spec);
                    R w = last ? R(1) : mis_power(pl, pb);
                    L = L + throughput * (brdf_eval(s, v, ldir) * nl * environment_value(l, ldir) *
                                          (vw * fog_tr(ldir, extent)) * w / pl);
                } else if (l.kind == SF_LIGHT_HDRI) {
                    if (l.color.x <= R(0)) continue;
                    R r0 = rnd<R>(&rng);
                    R r1 = rnd<R>(&rng);
                    R r2 = rnd<R>(&rng);
                    V3<R> ldir = hdri_sample(l, r0, r1, r2);
                    R nl = s.n.dot(ldir);
                    if (nl <= R(0) || n.dot(ldir) <= R(0)) continue;
                    const R vw = visible(ldir, extent);
                    if (!(vw > R(0))) continue;
                    R pl = hdri_pdf(l, ldir);
                    R pb = last ? R(0) : bsdf_pdf(s, v, ldir, p_spec);
                    R w = last ? R(1) : mis_power(pl, pb);
                    L = L + throughput * (brdf_eval(s, v, ldir) * nl * hdri_lookup(l, ldir) *
                                          (vw * fog_tr(ldir, extent)) * w / pl);
                } else if (l.kind == SF_LIGHT_SUN) {
                    R r1 = rnd<R>(&rng);
                    R r2 = rnd<R>(&rng);
                    V3<R> ldir = cone_sample(l.a, l.cos_max, r1, r2);
                    R nl = s.n.dot(ldir);
                    if (nl <= R(0) || n.dot(ldir) <= R(0)) continue;
                    const R vw = visible(ldir, extent);
                    if (!(vw > R(0))) continue;
                    R pl = sun_pdf(l.cos_max);
                    R pb = last ? R(0) : bsdf_pdf(s, v, ldir, p_spec);
                    R w = last ? R(1) : mis_power(pl, pb);
                    L = L + throughput * (brdf_eval(s, v, ldir) * nl * l.color * w * (vw * fog_tr(ldir, extent)));
                } else if (i == selected) {
                    // sample_emitter: two numbers for a rectangle, three for a tube
                    R u1 = rnd<R>(&rng);
                    R u2 = rnd<R>(&rng);
                    R u3 = l.kind == SF_LIGHT_TUBE ? rnd<R>(&rng) : R(0);
                    V3<R> q, ln;
                    sample_emitter_point(l, u1, u2, u3, &q, &ln);
                    V3<R> to_q = q - p_off;
                    R dist2 = to_q.dot(to_q);
                    if (dist2 < R(1e-8)) continue;
                    R dist = r_sqrt(dist2);
                    V3<R> ldir = to_q / dist;
                    R nl = s.n.dot(ldir);
                    R cos_l = ln.dot(-ldir);
                    if (nl <= R(0) || cos_l <= R(0) || n.dot(ldir) <= R(0)) continue;
                    R endpoint = r_max(R(0), dist - r_max(R(1e-5), dist * R(1e-6)));
                    const R vw = visible(ldir, endpoint);
                    if (!(vw > R(0))) continue;
                    R pl = (selected_weight / area_total) * area_direction_pdf(l, dist2, cos_l);
                    R pb = last ? R(0) : bsdf_pdf(s, v, ldir, p_spec);
                    R w = last ? R(1) : mis_power(pl, pb);
                    L = L + throughput * (brdf_eval(s, v, ldir) * nl * emitter_radiance(l, -ldir) * (vw * fog_tr(ldir, dist)) *
                                          w / pl);
                }
            }
        }
        if (last) break;
        R r0 = rnd<R>(&rng), r1 = rnd<R>(&rng), r2 = rnd<R>(&rng);
        V3<R> ldir;
        if (r0 < p_spec) {
            V3<R> hh = sample_ggx_h(s.n, v, s.alpha, r1, r2);
            V3<R> i = -v;
            ldir = i - hh * (R(2) * hh.dot(i));
        } else ldir = cosine_sample(s.n, r1, r2);
        R nl = s.n.dot(ldir);
        if (nl <= R(0) || n.dot(ldir) <= R(0)) break;
        R pdf = bsdf_pdf(s, v, ldir, p_spec);
        if (pdf <= R(1e-6)) break;
        throughput = throughput * (brdf_eval(s, v, ldir) * nl / pdf);
        prev_pdf = pdf;
        prev_from_bsdf = true;
        prev_from_volume = false;
        prev_normal = s.n;
        prev_area_total = area_total;
        if (bounce >= 2) {
            R q = r_clamp(r_max(throughput.x, r_max(throughput.y, throughput.z)), R(0.05), R(0.95));
            if (rnd<R>(&rng) > q) break;
            throughput = throughput / q;
        }
        ro = p_off;
        rd = ldir;
        tex_spread = r_max(tex_spread, s.alpha * R(0.25));
        bounce++;
    }
    bool ok = L.x == L.x && L.y == L.y && L.z == L.z && r_abs(L.x) < R(1e30) && r_abs(L.y) < R(1e30) &&
              r_abs(L.z) < R(1e30);
    res.L[0] = ok ? double(L.x) : 0.0;
    res.L[1] = ok ? double(L.y) : 0.0;
    res.L[2] = ok ? double(L.z) : 0.0;
    const V3<R> volume = volume_path ? L : primary_volume;  // pathtrace.wgsl:1198
    res.V[0] = ok ? double(volume.x) : 0.0;
    res.V[1] = ok ? double(volume.y) : 0.0;
    res.V[2] = ok ? double(volume.z) : 0.0;
    res.depth = double(first_depth);
    for (int i = 0; i < 4; ++i) res.aux[i] = double(aux[i]);
    return res;
}

// ---------------------------------------------------------------- planar
// PlanarFractal::sample (crates/syfrack-core/src/scene/planar.rs:77-194).
template <class R> Sample<R> planar_sample(const PlanarParams& f, V2<R> input) {
    auto cmul = [](V2<R> a, V2<R> b) { return V2<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
    auto cpow = [&](V2<R> z, uint32_t n) { V2<R> r(1, 0); for (uint32_t i = 0; i < n; ++i) r = cmul(r, z); return r; };
    auto cdiv = [&](V2<R> a, V2<R> b) { return cmul(a, V2<R>(b.x, -b.y)) / r_max(b.length_squared(), R(1e-24)); };
    R a = to_radians(R(f.angle));
    R sn = r_sin(a), cs = r_cos(a);
    V2<R> point = V2<R>(cs * input.x - sn * input.y, sn * input.x + cs * input.y) / R(f.zoom);
    if (R(f.inversion) != R(0)) point = point * (R(f.inversion) / r_max(point.length_squared(), R(1e-8)));
    point = point + V2<R>(R(f.center[0]), R(f.center[1]));
    bool parameter_plane = f.family == 1 || f.family == 2;
    bool root = f.family == 3 || f.family == 4;
    V2<R> c = parameter_plane ? point : V2<R>(R(f.julia[0]), R(f.julia[1]));
    V2<R> z = parameter_plane ? V2<R>(0, 0) : point;
    V2<R> previous(0, 0);
    R tw = to_radians(R(f.twist));
    V2<R> rotation(r_cos(tw), r_sin(tw));
    V2<R> lambda = rotation * R(f.relaxation);
    R ring = R(1e20), stripe = 0, previous_error = 1;
    uint32_t count = 0, measured = 0;
    R smooth = R(float(f.iterations));
    bool escaped = false;
    const R bail = R(f.bailout), stripes = R(f.stripes);
    for (uint32_t it = 0; it < f.iterations; ++it) {
        R radius = z.length();
        if (radius > bail) { escaped = true; break; }
        ring = r_min(ring, r_abs(radius - R(f.trap_radius)));
        R angle = radius == R(0) ? R(0) : r_atan2(z.y, z.x);
        stripe += R(0.5) + R(0.5) * r_sin(stripes * angle);
        measured += 1;
        if (root) {
            V2<R> residual = cpow(z, f.power) - V2<R>(1, 0);
            if (f.family == 3 && residual.length_squared() < R(1e-12)) {
                R error = r_max(residual.length(), R(1e-20));
                R fraction = r_clamp(r_log(R(1e-6) / previous_error) / r_log(error / previous_error), R(0), R(1));
                smooth = count == 0 ? R(0) : R(float(count)) - R(1) + fraction;
                break;
            }
            previous_error = r_max(residual.length(), R(1e-20));
            V2<R> old = z;
            V2<R> derivative = cpow(z, f.power - 1) * R(float(f.power));
            z = z - cmul(lambda, cdiv(residual, derivative));
            if (f.family == 4) {
                z = z + c;
                if ((z - old).length_squared() < R(1e-12)) { count += 1; smooth = R(float(count)); break; }
            }
        } else {
            V2<R> base = f.family == 2 ? V2<R>(r_abs(z.x), r_abs(z.y)) : z;
            V2<R> next = cmul(rotation, cpow(base, f.power)) + c;
            if (f.family == 5) next = next + previous * R(f.memory);
            previous = z;
            z = next;
        }
        count += 1;
    }
    R radius = r_min(z.length(), R(1e20));
    escaped = escaped || radius > bail;
    R lnp = r_log(R(float(f.power)));
    if (escaped && !root) smooth = R(float(count)) + R(1) - r_log(r_log(r_max(radius, R(1.0001)))) / lnp;
    else if (escaped) smooth = R(float(count));
    const R TAU = R(6.28318530717958647692);
    R final_angle = radius == R(0) ? R(0.5) : r_atan2(z.y, z.x) / TAU + R(0.5);
    R bands = stripe / R(float(std::max<uint32_t>(measured, 1)));
    if (escaped && !root && measured > 0) {
        R angle = radius == R(0) ? R(0) : r_atan2(z.y, z.x);
        R last = R(0.5) + R(0.5) * r_sin(stripes * angle);
        R full = (stripe + last) / R(float(measured + 1));
        R t = r_clamp(R(1) + (r_log(r_log(bail)) - r_log(r_log(r_max(radius, R(1.0001))))) / lnp, R(0), R(1));
        bands += (full - bands) * t;
    }
    Sample<R> out;
    out.material = 0;
    out.distance = radius / (R(1) + radius);
    out.iterations = count;
    out.traps[0] = r_clamp(smooth / R(float(f.iterations)), R(0), R(1));
    out.traps[1] = ring / (R(1) + ring);
    out.traps[2] = bands;
    out.traps[3] = final_angle;
    return out;
}

// explicit instantiations
template Sample<float> evaluate<float>(const Graph&, V3<float>, bool);
template Sample<double> evaluate<double>(const Graph&, V3<double>, bool);
template Sample<float> evaluate_union_search<float>(const Graph&, V3<float>, uint32_t*);
template Sample<double> evaluate_union_search<double>(const Graph&, V3<double>, uint32_t*);
template <class R> R texture_value_at(const Scene<R>& sc, V3<R> p) { return texture_value(sc.tex, p); }
template float texture_value_at<float>(const Scene<float>&, V3<float>);
template double texture_value_at<double>(const Scene<double>&, V3<double>);
template Scene<float> make_scene<float>(const Graph&, const sf_scene_desc&, const sf_render_config&);
template Scene<double> make_scene<double>(const Graph&, const sf_scene_desc&, const sf_render_config&);
template PixelResult radiance<float>(const Graph&, const Scene<float>&, uint32_t, uint32_t, uint32_t);
template PixelResult radiance<double>(const Graph&, const Scene<double>&, uint32_t, uint32_t, uint32_t);
template Hit<float> march_segment<float>(const Graph&, V3<float>, V3<float>, float, float, float, uint32_t, bool, float, uint64_t*);
template Hit<double> march_segment<double>(const Graph&, V3<double>, V3<double>, double, double, double, uint32_t, bool, double, uint64_t*);
template V3<float> normal_tetra<float>(const Graph&, V3<float>, float);
template V3<double> normal_tetra<double>(const Graph&, V3<double>, double);
template V3<float> normal_central<float>(const Graph&, V3<float>, float);
template V3<double> normal_central<double>(const Graph&, V3<double>, double);
template Sample<float> planar_sample<float>(const PlanarParams&, V2<float>);
template Sample<double> planar_sample<double>(const PlanarParams&, V2<double>);

}  // namespace orc
