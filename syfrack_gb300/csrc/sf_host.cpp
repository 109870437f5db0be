// Host side of the C ABI (include/syfrack_gpu.h): graph validation and
// lowering, device context with HBM admission, DE probe, primary rays, render
// sessions with tile scheduling and checkpoints, escape time and deep zoom.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <cfloat>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include "../../include/syfrack_gpu.h"
#include "sf_host_internal.h"
#include "sf_kernels.cuh"
#include "sf_program.h"

namespace sfh {

thread_local std::string g_error;

sf_status fail(sf_status s, const std::string& msg) {
    g_error = msg;
    return s;
}
const std::string& last_error() { return g_error; }
sf_status cuda_fail(cudaError_t e, const char* what) {
    g_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SF_ERR_OOM : SF_ERR_CUDA;
}

constexpr uint32_t MAX_DEPTH = 3;          // graph/mod.rs:41
constexpr uint32_t MAX_PLACEMENTS = 16384; // graph/mod.rs:18
constexpr uint32_t MAX_INSTANCE_PRODUCT = 65536;  // graph/mod.rs:20
// 1.1: sf_film_planes.color; 1.2: sf_render_config.hit_epsilon; 1.3: finish details, orbit
// colouring, optics and textures in sf_scene_desc
constexpr uint32_t ABI_VERSION = (1u << 16) | 6u;

// ------------------------------------------------------------------ graph preparation

bool is_point_kind(uint32_t k) {
    switch (k) {
    case SF_NODE_TRANSLATE: case SF_NODE_ROTATE: case SF_NODE_SCALE: case SF_NODE_SCALE_AXES:
    case SF_NODE_MIRROR: case SF_NODE_BOX_FOLD: case SF_NODE_BOX_FOLD_AXES: case SF_NODE_SPHERE_INVERSION:
    case SF_NODE_SPHERE_FOLD: case SF_NODE_ABS: case SF_NODE_MENGER_FOLD: case SF_NODE_KALEIDO:
    case SF_NODE_POWER: case SF_NODE_ADD_ORIGIN: case SF_NODE_ADD_SEED: case SF_NODE_ADD_CONSTANT:
    case SF_NODE_TWIST: case SF_NODE_BEND: case SF_NODE_TILE: case SF_NODE_REPEAT_FINITE:
    case SF_NODE_ITERATE: case SF_NODE_TRAP:
        return true;
    default: return false;
    }
}
bool is_fence_kind(uint32_t k) { return k >= SF_NODE_SPHERE && k <= SF_NODE_BULB_FENCE; }
bool is_combine_kind(uint32_t k) { return k >= SF_NODE_UNION && k <= SF_NODE_SMOOTH_INTERSECTION; }
// Port types (NodeKind::inputs/outputs, graph/mod.rs:366-396): 0 point, 1 distance.
std::vector<int> in_ports(uint32_t k) {
    if (k == SF_NODE_INPUT) return {};
    if (k == SF_NODE_OUTPUT || k == SF_NODE_MATERIAL_TAG || k == SF_NODE_INSTANCES) return {1};
    if (k == SF_NODE_BOUNDED) return {0, 1};
    if (is_combine_kind(k)) return {1, 1};
    return {0};
}
std::vector<int> out_ports(uint32_t k) {
    if (k == SF_NODE_OUTPUT) return {};
    if (k == SF_NODE_MATERIAL_TAG || k == SF_NODE_BOUNDED || k == SF_NODE_INSTANCES || is_fence_kind(k) ||
        is_combine_kind(k))
        return {1};
    return {0};
}

std::vector<uint32_t> active_nodes(const HostGraph& g) {
    const sf_node* out = nullptr;
    for (auto& n : g.nodes)
        if (n.kind == SF_NODE_OUTPUT) { out = &n; break; }
    if (!out) return {};
    std::set<uint32_t> seen;
    std::vector<uint32_t> stack{out->id};
    while (!stack.empty()) {
        uint32_t id = stack.back();
        stack.pop_back();
        if (!seen.insert(id).second) continue;
        for (auto& l : g.links)
            if (l.to_node == id) stack.push_back(l.from_node);
    }
    return std::vector<uint32_t>(seen.begin(), seen.end());
}

// validate_structure (validate.rs:146-330) for the checks the device path relies on.
std::string validate(const HostGraph& g) {
    std::set<uint32_t> ids;
    int inputs = 0, outputs = 0;
    for (auto& n : g.nodes) {
        if (n.kind >= SF_NODE_KIND_COUNT) return "unknown node kind on node " + std::to_string(n.id);
        if (!ids.insert(n.id).second) return "duplicate node id " + std::to_string(n.id);
        inputs += n.kind == SF_NODE_INPUT;
        outputs += n.kind == SF_NODE_OUTPUT;
        if (n.kind == SF_NODE_SCALE && std::fabs(n.f[0]) < 1e-3f) return "Scale factor cannot be zero";
        if (n.kind == SF_NODE_ITERATE && size_t(n.body_offset) + n.body_len > g.body.size())
            return "Iterate body out of range on node " + std::to_string(n.id);
        if (n.kind == SF_NODE_INSTANCES) {
            // validate.rs:198-207 and the placement bounds of graph/mod.rs:557-584
            const std::string at = " on node " + std::to_string(n.id);
            if (n.u[1] == 0 || n.u[1] > MAX_PLACEMENTS) return "Instances: between 1 and 16384 placements" + at;
            if (size_t(n.u[0]) + n.u[1] > g.placements.size()) return "Instances placements out of range" + at;
            if (!(n.f[3] >= 0.001f && n.f[3] <= 10.0f)) return "Instances margin out of [0.001, 10]" + at;
            for (uint32_t i = 0; i < n.u[1]; ++i) {
                const sf_placement& pl = g.placements[n.u[0] + i];
                for (int k = 0; k < 3; ++k) {
                    if (!(std::fabs(pl.position[k]) <= 1000.0f)) return "placement position out of [-1000, 1000]" + at;
                    if (!(std::fabs(pl.angles[k]) <= 180.0f)) return "placement angle out of [-180, 180]" + at;
                    if (!(pl.scale[k] >= 0.05f && pl.scale[k] <= 20.0f)) return "placement scale out of [0.05, 20]" + at;
                }
            }
        }
    }
    if (inputs != 1) return "the graph must have exactly one Input";
    if (outputs != 1) return "the graph must have exactly one Output";
    std::map<uint32_t, uint32_t> member;
    for (auto& n : g.nodes)
        for (uint32_t b : g.body_of(n)) {
            if (member.count(b)) return "node " + std::to_string(b) + " is in two Iterate bodies";
            member[b] = n.id;
            const sf_node* bn = g.node(b);
            if (!bn) return "Iterate body cites unknown node " + std::to_string(b);
            if (!is_point_kind(bn->kind)) return "Iterate body node " + std::to_string(b) + " is not Point -> Point";
            for (auto& l : g.links)
                if (l.from_node == b || l.to_node == b)
                    return "Iterate body node " + std::to_string(b) + " cannot be wired";
        }
    std::set<std::pair<uint32_t, uint32_t>> wired;
    for (auto& l : g.links) {
        const sf_node* from = g.node(l.from_node);
        const sf_node* to = g.node(l.to_node);
        if (!from) return "link from unknown node " + std::to_string(l.from_node);
        if (!to) return "link to unknown node " + std::to_string(l.to_node);
        auto op = out_ports(from->kind);
        auto ip = in_ports(to->kind);
        if (l.from_port >= op.size()) return "missing output port on node " + std::to_string(from->id);
        if (l.to_port >= ip.size()) return "missing input port on node " + std::to_string(to->id);
        if (op[l.from_port] != ip[l.to_port]) return "port type mismatch into node " + std::to_string(to->id);
        if (!wired.insert({l.to_node, l.to_port}).second)
            return "two wires into one input of node " + std::to_string(to->id);
    }
    // iterate nesting depth (validate.rs:87-110)
    std::function<uint32_t(uint32_t, std::vector<uint32_t>&)> depth = [&](uint32_t id, std::vector<uint32_t>& seen) -> uint32_t {
        if (std::find(seen.begin(), seen.end(), id) != seen.end()) return 99;
        seen.push_back(id);
        const sf_node* n = g.node(id);
        uint32_t d = 0;
        if (n && n->kind == SF_NODE_ITERATE) {
            uint32_t m = 0;
            for (uint32_t b : g.body_of(*n)) m = std::max(m, depth(b, seen));
            d = 1 + m;
        }
        seen.pop_back();
        return d;
    };
    for (auto& n : g.nodes) {
        std::vector<uint32_t> seen;
        if (depth(n.id, seen) > MAX_DEPTH) return "Iterate nesting deeper than 3";
    }
    return "";
}

bool topo_order(const HostGraph& g, std::vector<uint32_t>& order) {
    auto act = active_nodes(g);
    std::set<uint32_t> active(act.begin(), act.end());
    std::set<uint32_t> owned;
    for (auto& n : g.nodes)
        for (uint32_t b : g.body_of(n)) owned.insert(b);
    std::map<uint32_t, size_t> indeg;
    for (uint32_t id : active)
        if (!owned.count(id)) indeg[id] = 0;
    for (auto& l : g.links)
        if (indeg.count(l.to_node) && active.count(l.from_node)) indeg[l.to_node] += 1;
    std::vector<uint32_t> ready;
    for (auto& kv : indeg)
        if (kv.second == 0) ready.push_back(kv.first);
    auto desc = [](uint32_t a, uint32_t b) { return a > b; };
    std::sort(ready.begin(), ready.end(), desc);
    order.clear();
    while (!ready.empty()) {
        uint32_t id = ready.back();
        ready.pop_back();
        order.push_back(id);
        for (auto& l : g.links) {
            if (l.from_node != id) continue;
            auto it = indeg.find(l.to_node);
            if (it != indeg.end() && --it->second == 0) ready.push_back(l.to_node);
        }
        std::sort(ready.begin(), ready.end(), desc);
    }
    return order.size() == indeg.size();
}

uint32_t iter_product(const HostGraph& g, uint32_t id, std::vector<uint32_t>& seen) {
    if (std::find(seen.begin(), seen.end(), id) != seen.end()) return 0xffffffffu;
    seen.push_back(id);
    uint32_t p = 1;
    const sf_node* n = g.node(id);
    if (n && n->kind == SF_NODE_ITERATE) {
        uint32_t m = 0;
        bool any = false;
        for (uint32_t b : g.body_of(*n)) { m = std::max(m, iter_product(g, b, seen)); any = true; }
        uint64_t r = uint64_t(n->u[0]) * (any ? m : 1);
        p = r > 0xffffffffull ? 0xffffffffu : uint32_t(r);
    }
    seen.pop_back();
    return p;
}

void trap_walk(const HostGraph& g, uint32_t id, uint32_t depth, float* scales) {
    if (depth > MAX_DEPTH + 1) return;
    const sf_node* n = g.node(id);
    if (!n || !n->enabled) return;
    if (n->kind == SF_NODE_TRAP) scales[std::min<uint32_t>(n->u[0], 3)] = n->f[0];
    else if (n->kind == SF_NODE_ITERATE)
        for (uint32_t b : g.body_of(*n)) trap_walk(g, b, depth + 1, scales);
}

void lip_visit(const HostGraph& g, uint32_t id, float radius, uint32_t depth, float* l) {
    if (depth > MAX_DEPTH + 1) return;
    const sf_node* n = g.node(id);
    if (!n || !n->enabled) return;
    if (n->kind == SF_NODE_TWIST || n->kind == SF_NODE_BEND) {
        float x = n->f[0] * radius;
        *l *= sqrtf(1.0f + x * x);
    }
    for (uint32_t b : g.body_of(*n)) lip_visit(g, b, radius, depth + 1, l);
}

// ------------------------------------------------------------------ instances
// Rotation of glam's Quat::from_euler(EulerRot::XYZ, a, b, c) = Qx(a) Qy(b) Qz(c),
// kept as a unit quaternion (x, y, z, w) and applied with glam's mul_vec3 formula.
struct Quat4 { float x, y, z, w; };
Quat4 quat_mul(const Quat4& a, const Quat4& b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
Quat4 quat_euler_xyz(const float deg[3]) {
    const float k = 3.14159265358979323846f / 180.0f;
    const float a = deg[0] * k, b = deg[1] * k, c = deg[2] * k;
    Quat4 qx{std::sin(a * 0.5f), 0.f, 0.f, std::cos(a * 0.5f)};
    Quat4 qy{0.f, std::sin(b * 0.5f), 0.f, std::cos(b * 0.5f)};
    Quat4 qz{0.f, 0.f, std::sin(c * 0.5f), std::cos(c * 0.5f)};
    return quat_mul(quat_mul(qx, qy), qz);
}
void quat_rotate(const Quat4& q, const float v[3], float out[3]) {
    const float b2 = q.x * q.x + q.y * q.y + q.z * q.z;
    const float vb = v[0] * q.x + v[1] * q.y + v[2] * q.z;
    const float cr[3] = {q.y * v[2] - q.z * v[1], q.z * v[0] - q.x * v[2], q.x * v[1] - q.y * v[0]};
    const float bq[3] = {q.x, q.y, q.z};
    for (int i = 0; i < 3; ++i) out[i] = v[i] * (q.w * q.w - b2) + bq[i] * (vb * 2.0f) + cr[i] * (q.w * 2.0f);
}

// The copies' fence hierarchy (bvh.rs:26-102): leaves bound each rotated, scaled
// fence box (padded for roundoff); interior nodes split at the median of the
// longest axis, ties by placement index; preorder layout with escape indices.
struct InstNode { float center[3], half[3]; uint32_t escape; int32_t placement; };
void inst_split(std::vector<InstNode>& leaves, size_t lo, size_t hi, std::vector<InstNode>& nodes) {
    float mn[3], mx[3];
    for (int k = 0; k < 3; ++k) { mn[k] = INFINITY; mx[k] = -INFINITY; }
    for (size_t i = lo; i < hi; ++i)
        for (int k = 0; k < 3; ++k) {
            mn[k] = std::min(mn[k], leaves[i].center[k] - leaves[i].half[k]);
            mx[k] = std::max(mx[k], leaves[i].center[k] + leaves[i].half[k]);
        }
    const size_t index = nodes.size();
    InstNode n{};
    for (int k = 0; k < 3; ++k) {
        n.center[k] = mn[k] * 0.5f + mx[k] * 0.5f;
        n.half[k] = std::max(mx[k] - n.center[k], n.center[k] - mn[k]) + 0.002f;
    }
    n.placement = -1;
    nodes.push_back(n);
    if (hi - lo == 1) {
        nodes[index].placement = leaves[lo].placement;
    } else {
        const float ex = mx[0] - mn[0], ey = mx[1] - mn[1], ez = mx[2] - mn[2];
        const int axis = (ex >= ey && ex >= ez) ? 0 : (ey >= ez ? 1 : 2);
        const size_t middle = lo + (hi - lo) / 2;
        std::nth_element(leaves.begin() + lo, leaves.begin() + middle, leaves.begin() + hi,
                         [axis](const InstNode& a, const InstNode& b) {
                             if (a.center[axis] != b.center[axis]) return a.center[axis] < b.center[axis];
                             return a.placement < b.placement;
                         });
        inst_split(leaves, lo, middle, nodes);
        inst_split(leaves, middle, hi, nodes);
    }
    nodes[index].escape = uint32_t(nodes.size());
}
// Appends one Instances node's device block: per placement the inverse affine rows
// (graph_wgsl.rs:140-152: row_i = (R e_i) / scale_i, w = -row_i . position), then the
// hierarchy nodes as 8 floats (centre, half, escape, placement or -1).
void pack_instances(const sf_placement* pl, uint32_t count, const float half[3], std::vector<float>& out) {
    std::vector<InstNode> leaves(count);
    for (uint32_t i = 0; i < count; ++i) {
        const Quat4 r = quat_euler_xyz(pl[i].angles);
        float ext[3] = {0.f, 0.f, 0.f};
        for (int a = 0; a < 3; ++a) {
            const float e[3] = {a == 0 ? 1.f : 0.f, a == 1 ? 1.f : 0.f, a == 2 ? 1.f : 0.f};
            float col[3];
            quat_rotate(r, e, col);
            const float h = half[a] * pl[i].scale[a];
            for (int k = 0; k < 3; ++k) ext[k] += std::fabs(col[k]) * h;
            float row[4];
            for (int k = 0; k < 3; ++k) row[k] = col[k] / pl[i].scale[a];
            row[3] = -(row[0] * pl[i].position[0] + row[1] * pl[i].position[1] + row[2] * pl[i].position[2]);
            out.insert(out.end(), row, row + 4);
        }
        InstNode& n = leaves[i];
        for (int k = 0; k < 3; ++k) {
            const float pad = (std::fabs(pl[i].position[k]) + ext[k]) * (16.0f * FLT_EPSILON) + 0.002f;
            n.center[k] = pl[i].position[k];
            n.half[k] = ext[k] + pad;
        }
        n.escape = 0;
        n.placement = int32_t(i);
    }
    std::vector<InstNode> nodes;
    nodes.reserve(2 * size_t(count) - 1);
    inst_split(leaves, 0, leaves.size(), nodes);
    for (const InstNode& n : nodes) {
        const float v[8] = {n.center[0], n.center[1], n.center[2], n.half[0], n.half[1], n.half[2],
                            float(n.escape), float(n.placement)};
        out.insert(out.end(), v, v + 8);
    }
}

// ------------------------------------------------------------------ lowering
float sqrt_threshold(float b);
// negative_bounds (graph_wgsl.rs:976-1006): a lower bound stays safe only through
// monotone combinations. A Bounded node reached through the second input of an
// enabled Subtraction (its sign flipped) is evaluated exactly everywhere.
void negative_bounds(const HostGraph& g, uint32_t id, bool negative, std::set<std::pair<uint32_t, bool>>& seen,
                     std::set<uint32_t>& unsafe, int guard = 0) {
    if (guard > 512 || !seen.insert({id, negative}).second) return;
    const sf_node* n = g.node(id);
    if (!n) return;
    if (negative && (n->kind == SF_NODE_BOUNDED || n->kind == SF_NODE_INSTANCES)) unsafe.insert(id);
    const uint32_t ports = uint32_t(in_ports(n->kind).size());
    for (uint32_t port = 0; port < ports; ++port) {
        const bool sign = negative ^ (n->enabled && n->kind == SF_NODE_SUBTRACTION && port == 1);
        uint32_t src = 0;
        if (g.input_of(id, port, &src)) negative_bounds(g, src, sign, seen, unsafe, guard + 1);
    }
}

struct Lowerer {
    const HostGraph& g;
    DeProgram& P;
    std::set<uint32_t> unsafe_bounds;
    std::vector<float>* inst = nullptr;
    std::string err;
    int stack_depth = 0, max_stack = 0;
    // Instances templates being lowered (at most SF_MAX_INST_DEPTH nested), and whether
    // the innermost runs exactly: the template of a copy search that may not skip is
    // the reference's `_exact` variant (graph_wgsl.rs:744-790), so no Bounded or
    // Instances node inside it skips either
    int template_depth = 0;
    bool template_exact = false;

    bool push(const DeOp& op) {
        if (P.n_ops >= SF_MAX_OPS) { err = "graph too large for the device program"; return false; }
        P.ops[P.n_ops++] = op;
        return true;
    }
    static DeOp mk(uint32_t code) { DeOp o; std::memset(&o, 0, sizeof o); o.code = code; return o; }

    bool point_op(uint32_t id) {
        const sf_node* n = g.node(id);
        if (!n || !n->enabled || !is_point_kind(n->kind)) return true;  // no-op (eval.rs:351-353, :555)
        if (n->kind == SF_NODE_ITERATE) {
            uint32_t begin = P.n_ops;
            DeOp b = mk(SF_OP_ITER_BEGIN);
            b.a = n->u[0];
            b.f[0] = n->f[0];
            b.f[1] = sqrt_threshold(n->f[0]);
            if (!push(b)) return false;
            for (uint32_t c : g.body_of(*n))
                if (!point_op(c)) return false;
            DeOp e = mk(SF_OP_ITER_END);
            e.a = begin;
            if (!push(e)) return false;
            P.ops[begin].b = P.n_ops - 1;
            return true;
        }
        DeOp o = mk(n->kind);
        std::memcpy(o.f, n->f, sizeof o.f);
        switch (n->kind) {
        case SF_NODE_POWER: {
            float pw = n->f[0];
            o.a = (pw >= 1.f && pw <= 16.f && pw == std::floor(pw)) ? uint32_t(pw) : 0u;
            break;
        }
        case SF_NODE_BOX_FOLD_AXES: case SF_NODE_ABS:
            o.a = (n->u[0] ? 1u : 0u) | (n->u[1] ? 2u : 0u) | (n->u[2] ? 4u : 0u);
            break;
        case SF_NODE_KALEIDO: o.a = n->u[0]; break;
        case SF_NODE_REPEAT_FINITE: o.a = n->u[0]; o.b = n->u[1]; o.c = n->u[2]; break;
        case SF_NODE_TRAP: o.a = std::min<uint32_t>(n->u[0], 3); o.b = n->u[1]; o.c = n->u[2]; break;
        default: break;
        }
        return push(o);
    }
    // The point state feeding a port: a chain of point ops from the Input.
    bool chain(bool has_src, uint32_t src, int guard = 0) {
        if (guard > 256) { err = "point chain too deep"; return false; }
        if (!has_src) return push(mk(SF_OP_BEGIN));
        const sf_node* n = g.node(src);
        if (!n) return push(mk(SF_OP_BEGIN));
        if (n->kind == SF_NODE_INPUT) return push(mk(SF_OP_BEGIN));
        if (!is_point_kind(n->kind)) { err = "distance value wired into a point port"; return false; }
        uint32_t up = 0;
        bool has = g.input_of(src, 0, &up);
        if (!chain(has, up, guard + 1)) return false;
        return point_op(src);
    }
    bool dist(bool has_src, uint32_t src, int guard = 0) {
        if (guard > 256) { err = "distance tree too deep"; return false; }
        if (!has_src || !g.node(src)) {
            stack_depth++;
            max_stack = std::max(max_stack, stack_depth);
            return push(mk(SF_OP_EMPTY));
        }
        const sf_node& n = *g.node(src);
        uint32_t a = 0, b = 0;
        bool ha = g.input_of(src, 0, &a), hb = g.input_of(src, 1, &b);
        if (is_fence_kind(n.kind)) {
            if (!chain(ha, a)) return false;
            DeOp o = mk(n.enabled ? n.kind : (uint32_t)SF_OP_FENCE_OFF);
            std::memcpy(o.f, n.f, sizeof o.f);
            if (n.kind == SF_NODE_ROCK) o.a = n.u[0];
            stack_depth++;
            max_stack = std::max(max_stack, stack_depth);
            return push(o);
        }
        if (n.kind == SF_NODE_MATERIAL_TAG) {
            if (!dist(ha, a, guard + 1)) return false;
            if (!n.enabled) return true;
            DeOp o = mk(SF_OP_TAG);
            o.a = n.u[0];
            return push(o);
        }
        if (n.kind == SF_NODE_BOUNDED) {
            if (n.enabled && !unsafe_bounds.count(src) && !template_exact) {
                // skippable bound (graph_wgsl.rs:800-814): bound first, detail only near it
                if (!chain(ha, a)) return false;
                const uint32_t at = P.n_ops;
                DeOp o = mk(SF_OP_BOUND_FAST);
                std::memcpy(o.f, n.f, sizeof o.f);
                if (!push(o)) return false;
                stack_depth++;
                max_stack = std::max(max_stack, stack_depth);
                if (!dist(hb, b, guard + 1)) return false;
                if (!push(mk(SF_OP_BOUND_END))) return false;
                stack_depth--;
                P.ops[at].b = P.n_ops - 1;
                P.fast_bounds++;
                return true;
            }
            if (!dist(hb, b, guard + 1)) return false;
            if (!n.enabled) return true;
            if (!chain(ha, a)) return false;
            DeOp o = mk(SF_OP_BOUND);
            std::memcpy(o.f, n.f, sizeof o.f);
            return push(o);
        }
        if (n.kind == SF_NODE_INSTANCES) {
            if (!n.enabled) return dist(ha, a, guard + 1);  // passes its template through (eval.rs:816)
            if (template_depth >= SF_MAX_INST_DEPTH) { err = "Instances nested deeper than 3 levels"; return false; }
            if (!ha) {  // no template: the copies are empty (eval.rs:752-755)
                stack_depth++;
                max_stack = std::max(max_stack, stack_depth);
                return push(mk(SF_OP_EMPTY));
            }
            const uint32_t at = P.n_ops;
            DeOp o = mk(SF_OP_INST_BEGIN);
            o.a = n.u[1];
            o.c = uint32_t(inst->size());
            std::memcpy(o.f, n.f, 4 * sizeof(float));
            const bool skippable = !unsafe_bounds.count(src) && !template_exact;
            o.f[4] = skippable ? 1.f : 0.f;
            pack_instances(g.placements.data() + n.u[0], n.u[1], n.f, *inst);
            if (!push(o)) return false;
            const bool outer_exact = template_exact;
            template_depth++;
            template_exact = !skippable;
            const bool ok = dist(ha, a, guard + 1);
            template_depth--;
            template_exact = outer_exact;
            if (!ok) return false;
            DeOp e = mk(SF_OP_INST_END);
            e.a = at;
            if (!push(e)) return false;
            P.ops[at].b = P.n_ops - 1;
            return true;
        }
        if (is_combine_kind(n.kind)) {
            if (!dist(ha, a, guard + 1)) return false;
            if (!n.enabled) return true;  // disabled: port 0 passes through (eval.rs:822)
            if (!dist(hb, b, guard + 1)) return false;
            DeOp o = mk(SF_OP_COMBINE);
            o.a = n.kind;
            o.f[0] = n.f[0];
            stack_depth--;
            return push(o);
        }
        err = "point value wired into a distance port";
        return false;
    }
    // The Output's input lowered as dist() lowers it, recording the op range of each
    // leaf below its enabled Unions (union_leaves, graph_wgsl.rs:18-26: depth-first,
    // first input first, a leaf reached twice kept once).
    struct Leaf {
        bool has;
        uint32_t id, begin, end;
    };
    std::vector<Leaf> leaves;
    bool union_tree(bool has_src, uint32_t src, int guard = 0) {
        if (guard > 256) { err = "distance tree too deep"; return false; }
        const sf_node* n = has_src ? g.node(src) : nullptr;
        if (n && n->enabled && n->kind == SF_NODE_UNION) {
            uint32_t a = 0, b = 0;
            const bool ha = g.input_of(src, 0, &a), hb = g.input_of(src, 1, &b);
            if (!union_tree(ha, a, guard + 1) || !union_tree(hb, b, guard + 1)) return false;
            DeOp o = mk(SF_OP_COMBINE);
            o.a = n->kind;
            o.f[0] = n->f[0];
            stack_depth--;
            return push(o);
        }
        const uint32_t begin = P.n_ops;
        if (!dist(has_src, src, guard)) return false;
        const bool known = n && std::any_of(leaves.begin(), leaves.end(),
                                            [&](const Leaf& l) { return l.has && l.id == src; });
        if (!known) leaves.push_back({n != nullptr, src, begin, P.n_ops});
        return true;
    }
};

// Largest float x with sqrtf(x) <= b. sqrtf is correctly rounded and monotonic,
// so |p| > b (the reference's `p.length() > bailout`) is exactly dot(p,p) > T.
float sqrt_threshold(float b) {
    if (!(b == b)) return b;                  // NaN: no comparison is ever true
    if (b < 0.f) return -1.0f;                // any x >= 0 exceeds it (sqrt(x) >= 0 > b)
    if (std::isinf(b)) return b;
    float t = b * b;
    if (std::isinf(t)) t = 3.4028235e38f;
    while (t > 0.f && sqrtf(t) > b) t = std::nextafter(t, 0.0f);
    for (;;) {
        float u = std::nextafter(t, INFINITY);
        if (std::isinf(u) || sqrtf(u) > b) break;
        t = u;
    }
    return t;
}

// Recognises the iterated forms of graphs/{mandelbulb,mandelbox,menger}.ron.
void detect_form(const HostGraph& g, DeProgram& P) {
    P.form = SF_FORM_GENERIC;
    const sf_node* out = nullptr;
    for (auto& n : g.nodes)
        if (n.kind == SF_NODE_OUTPUT) out = &n;
    uint32_t fid;
    if (!out || !g.input_of(out->id, 0, &fid)) return;
    const sf_node* fence = g.node(fid);
    uint32_t material = 0;
    if (fence && fence->kind == SF_NODE_MATERIAL_TAG) {
        if (!fence->enabled) return;
        material = fence->u[0];
        if (!g.input_of(fence->id, 0, &fid)) return;
        fence = g.node(fid);
    }
    if (!fence || !fence->enabled || !is_fence_kind(fence->kind)) return;
    uint32_t iid;
    if (!g.input_of(fence->id, 0, &iid)) return;
    const sf_node* it = g.node(iid);
    if (!it || !it->enabled || it->kind != SF_NODE_ITERATE) return;
    uint32_t src;
    if (!g.input_of(it->id, 0, &src)) return;
    const sf_node* in = g.node(src);
    if (!in || in->kind != SF_NODE_INPUT) return;
    std::vector<const sf_node*> body;
    for (uint32_t b : g.body_of(*it)) {
        const sf_node* bn = g.node(b);
        if (!bn || !bn->enabled) return;
        body.push_back(bn);
    }
    auto kinds = [&](std::initializer_list<uint32_t> want) {
        if (body.size() != want.size()) return false;
        size_t i = 0;
        for (uint32_t k : want)
            if (body[i++]->kind != k) return false;
        return true;
    };
    FormParams& f = P.fp;
    std::memset(&f, 0, sizeof f);
    f.iterations = it->u[0];
    f.bailout = it->f[0];
    f.bailout_t = sqrt_threshold(it->f[0]);
    f.material = material;
    auto set_trap = [&](const sf_node* t) {
        f.trap_slot = std::min<uint32_t>(t->u[0], 3);
        f.trap_measure = t->u[1];
        f.trap_mode = t->u[2];
        f.trap_squared = t->u[1] == SF_MEASURE_NORM && t->u[2] != SF_TRAP_MAXIMUM;
    };
    if (fence->kind == SF_NODE_BULB_FENCE && kinds({SF_NODE_TRAP, SF_NODE_POWER, SF_NODE_ADD_ORIGIN})) {
        set_trap(body[0]);
        f.power = body[1]->f[0];
        float pw = f.power;
        f.power_int = (pw >= 1.f && pw <= 16.f && pw == std::floor(pw)) ? uint32_t(pw) : 0u;
        P.form = SF_FORM_BULB;
    } else if (fence->kind == SF_NODE_NORM_FENCE &&
               kinds({SF_NODE_BOX_FOLD, SF_NODE_TRAP, SF_NODE_SPHERE_FOLD, SF_NODE_SCALE, SF_NODE_ADD_ORIGIN})) {
        f.limit = body[0]->f[0];
        set_trap(body[1]);
        float mr = body[2]->f[0], fr = body[2]->f[1];
        f.min_radius2 = mr * mr;
        f.fixed_radius2 = fr * fr;
        f.fold_k_min = f.fixed_radius2 / f.min_radius2;
        f.fold_clamped = f.fold_k_min >= 1.0f ? 1u : 0u;
        f.scale = body[3]->f[0];
        f.abs_scale = std::fabs(f.scale);
        f.fence[0] = fence->f[0];
        P.form = SF_FORM_BOX;
    } else if (fence->kind == SF_NODE_BOX && kinds({SF_NODE_MENGER_FOLD, SF_NODE_TRAP})) {
        f.scale = body[0]->f[0];
        f.offset[0] = body[0]->f[1];
        f.offset[1] = body[0]->f[2];
        f.offset[2] = body[0]->f[3];
        set_trap(body[1]);
        f.fence[0] = fence->f[0];
        f.fence[1] = fence->f[1];
        f.fence[2] = fence->f[2];
        P.form = SF_FORM_MENGER;
    }
}

}  // namespace sfh

// ------------------------------------------------------------------ context

namespace sfh {

sf_status ctx_alloc(sf_context* c, size_t bytes, void** p, bool trim) {
    *p = nullptr;
    if (bytes == 0) return SF_OK;
    std::unique_lock<std::mutex> lk(c->alloc_mu);
    for (size_t i = 0; i < c->cached.size(); ++i) {  // an idle arena of this exact size
        if (c->cached[i].second == bytes) {
            *p = c->cached[i].first;
            c->cached.erase(c->cached.begin() + long(i));
            return SF_OK;
        }
    }
    while (!c->cached.empty() && c->used + bytes > c->budget) {  // idle arenas give way first
        cudaFree(c->cached.front().first);
        c->used -= std::min<uint64_t>(c->used, c->cached.front().second);
        c->cached.erase(c->cached.begin());
    }
    if (trim && c->used + bytes > c->budget) {
        // The cached scratch of primary and escape-time calls gives way to an admission.
        // Its owner (stage_mu) may be in a readback: then wait for it, taking the locks in
        // the order the scratch's users take them (stage_mu, then alloc_mu), so that the
        // admission's outcome does not depend on timing. No caller that trims holds stage_mu.
        std::unique_lock<std::mutex> sl(c->stage_mu, std::try_to_lock);
        if (!sl.owns_lock()) {
            lk.unlock();
            sl.lock();
            lk.lock();
        }
        if (c->scratch && c->used + bytes > c->budget) {
            cudaFree(c->scratch);
            c->used -= c->scratch_bytes;
            c->scratch = nullptr;
            c->scratch_bytes = 0;
        }
    }
    if (c->used + bytes > c->budget)
        return fail(SF_ERR_BUDGET, "HBM admission budget exceeded: " + std::to_string(c->used + bytes) + " > " +
                                       std::to_string(c->budget) + " bytes");
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    c->used += bytes;
    return SF_OK;
}
void ctx_free(sf_context* c, void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(c->alloc_mu);
    cudaFree(p);
    c->used -= std::min<uint64_t>(c->used, bytes);
}
void ctx_free_cached(sf_context* c, void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(c->alloc_mu);
    c->cached.emplace_back(p, bytes);
    if (c->cached.size() > 4) {
        cudaFree(c->cached.front().first);
        c->used -= std::min<uint64_t>(c->used, c->cached.front().second);
        c->cached.erase(c->cached.begin());
    }
}

void ctx_retain(sf_context* c) {
    std::lock_guard<std::mutex> lk(c->mu);
    c->refs++;
}
void collect_timing(sf_context* c);
void ctx_release(sf_context* c) {
    {
        std::lock_guard<std::mutex> lk(c->mu);
        if (--c->refs > 0) return;
    }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    collect_timing(c);
    for (auto e : c->spare) cudaEventDestroy(e);
    ctx_free(c, c->d_stats, SF_STAT_COUNT * sizeof(unsigned long long) + 64 * sizeof(uint32_t));
    for (auto& b : c->cached) cudaFree(b.first);
    c->cached.clear();
    if (c->stage) cudaFreeHost(c->stage);
    ctx_free(c, c->scratch, c->scratch_bytes);
    cudaStreamDestroy(c->stream);
    delete c;
}

cudaEvent_t get_event(sf_context* c) {
    if (!c->spare.empty()) {
        cudaEvent_t e = c->spare.back();
        c->spare.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
void collect_timing(sf_context* c) {
    if (c->timed.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto& t : c->timed) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
            c->kernel_ms += ms;
            if (t.trace) c->trace_ms += ms;
        }
        c->spare.push_back(t.a);
        c->spare.push_back(t.b);
    }
    c->timed.clear();
}

sf_status wait_stream(cudaStream_t st, uint32_t timeout_ms) {
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) return SF_OK;
        if (e != cudaErrorNotReady) return cuda_fail(e, "stream");
        double el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms && el > timeout_ms) return fail(SF_ERR_TIMEOUT, "dispatch exceeded its time limit");
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

// Runs f(begin, end) over [0, n) on up to 8 host threads (one below 1 M items).
template <class F> void host_parallel(size_t n, F&& f) {
    const size_t parts = std::min<size_t>(8, std::max<size_t>(1, n >> 20));
    if (parts == 1) { f(size_t(0), n); return; }
    std::vector<std::thread> pool;
    for (size_t k = 0; k < parts; ++k) pool.emplace_back([&, k] { f(n * k / parts, n * (k + 1) / parts); });
    for (auto& t : pool) t.join();
}

// The context's pinned staging at `bytes` or more (stage_mu held).
cudaError_t ensure_stage(sf_context* c, size_t bytes) {
    if (c->stage_bytes >= bytes) return cudaSuccess;
    if (c->stage) cudaFreeHost(c->stage);
    c->stage = nullptr;
    c->stage_bytes = 0;
    cudaError_t e = cudaHostAlloc(&c->stage, bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) c->stage_bytes = bytes;
    return e;
}

// The context's device scratch at `bytes` or more (stage_mu held), within the budget.
sf_status ensure_scratch(sf_context* c, size_t bytes) {
    if (c->scratch_bytes >= bytes) return SF_OK;
    ctx_free(c, c->scratch, c->scratch_bytes);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    const sf_status s = ctx_alloc(c, bytes, &c->scratch, false);  // stage_mu is held: no trim
    if (s == SF_OK) c->scratch_bytes = bytes;
    return s;
}

std::string topology_of(const HostGraph& g) {
    // Everything but the float parameters (topology_key, graph/mod.rs:397-425).
    std::string s;
    char buf[96];
    for (auto& n : g.nodes) {
        float pw = n.kind == SF_NODE_POWER ? n.f[0] : 0.f;
        bool even68 = pw == 6.f || pw == 8.f;
        std::snprintf(buf, sizeof buf, "%u:%u:%u:%u:%u:%u:%u:%u;", n.id, n.kind, n.enabled, n.body_offset, n.body_len,
                      n.u[0], n.u[1], n.u[2]);
        s += buf;
        if (n.kind == SF_NODE_POWER && !even68) { std::snprintf(buf, sizeof buf, "p%g;", pw); s += buf; }
    }
    for (auto& l : g.links) {
        std::snprintf(buf, sizeof buf, "%u.%u>%u.%u;", l.from_node, l.from_port, l.to_node, l.to_port);
        s += buf;
    }
    for (uint32_t b : g.body) s += std::to_string(b) + ",";
    return s;
}

// Copies budget (validate.rs:340-372): along any path, at most 3 enabled Instances
// and at most 65,536 copies in product.
bool copies_budget(const HostGraph& g, uint32_t id, std::map<uint32_t, std::pair<uint32_t, uint64_t>>& memo,
                   std::pair<uint32_t, uint64_t>& out, int guard = 0) {
    auto it = memo.find(id);
    if (it != memo.end()) { out = it->second; return true; }
    if (guard > 512) return false;
    const sf_node* n = g.node(id);
    std::pair<uint32_t, uint64_t> b{0, 1};
    if (n) {
        const uint32_t ports = uint32_t(in_ports(n->kind).size());
        for (uint32_t port = 0; port < ports; ++port) {
            uint32_t src = 0;
            if (!g.input_of(id, port, &src)) continue;
            std::pair<uint32_t, uint64_t> c;
            if (!copies_budget(g, src, memo, c, guard + 1)) return false;
            b.first = std::max(b.first, c.first);
            b.second = std::max(b.second, c.second);
        }
        if (n->kind == SF_NODE_INSTANCES && n->enabled) {
            b.first += 1;
            b.second = std::min<uint64_t>(b.second * n->u[1], 0xffffffffull);
        }
    }
    memo[id] = b;
    out = b;
    return true;
}

sf_status build_graph(const sf_graph_desc* d, HostGraph& g, DeProgram& P, sf_graph_info& info,
                      std::vector<float>& inst) {
    if (!d || (!d->nodes && d->node_count)) return fail(SF_ERR_INVALID, "null graph descriptor");
    g.nodes.assign(d->nodes, d->nodes + d->node_count);
    g.links.assign(d->links ? d->links : nullptr, d->links ? d->links + d->link_count : nullptr);
    g.body.assign(d->body_ids ? d->body_ids : nullptr, d->body_ids ? d->body_ids + d->body_id_count : nullptr);
    g.placements.assign(d->placements ? d->placements : nullptr,
                        d->placements ? d->placements + d->placement_count : nullptr);
    g.safety = d->safety;
    g.hint = d->bounding_radius_hint;
    std::string e = validate(g);
    if (!e.empty()) return fail(SF_ERR_GRAPH, e);
    std::vector<uint32_t> order;
    if (!topo_order(g, order)) return fail(SF_ERR_GRAPH, "cycle in the graph");
    {
        std::map<uint32_t, std::pair<uint32_t, uint64_t>> memo;
        for (auto& n : g.nodes) {
            std::pair<uint32_t, uint64_t> b;
            if (!copies_budget(g, n.id, memo, b)) return fail(SF_ERR_GRAPH, "graph too deep");
            if (b.first > MAX_DEPTH || b.second > MAX_INSTANCE_PRODUCT)
                return fail(SF_ERR_GRAPH, "nested Instances: at most 3 levels and 65536 copies on node " +
                                              std::to_string(n.id));
        }
    }
    std::memset(&P, 0, sizeof P);
    inst.clear();
    for (int i = 0; i < 4; ++i) P.trap_scales[i] = 1.f;
    for (uint32_t id : order) trap_walk(g, id, 0, P.trap_scales);
    std::set<uint32_t> owned;
    for (auto& n : g.nodes)
        for (uint32_t b : g.body_of(n)) owned.insert(b);
    uint32_t best = 0;
    bool any = false;
    for (uint32_t id : active_nodes(g)) {
        if (owned.count(id)) continue;
        std::vector<uint32_t> seen;
        best = std::max(best, iter_product(g, id, seen));
        any = true;
    }
    P.iteration_product = any ? best : 1;
    float lip = 1.f;
    for (uint32_t id : active_nodes(g)) lip_visit(g, id, g.hint, 0, &lip);
    Lowerer L{g, P, {}, &inst};
    const sf_node* out = nullptr;
    for (auto& n : g.nodes)
        if (n.kind == SF_NODE_OUTPUT) out = &n;
    {
        std::set<std::pair<uint32_t, bool>> seen;
        negative_bounds(g, out->id, false, seen, L.unsafe_bounds);
    }
    uint32_t src = 0;
    bool has = g.input_of(out->id, 0, &src);
    if (!L.union_tree(has, src)) return fail(L.err.find("not supported") != std::string::npos ? SF_ERR_UNSUPPORTED : SF_ERR_GRAPH, L.err);
    if (L.max_stack > SF_MAX_DIST_STACK) return fail(SF_ERR_UNSUPPORTED, "distance tree wider than the device stack");
    P.max_stack = L.max_stack;
    // The branch-and-bound needs a skippable node anywhere in the graph (the `fast` set
    // of graph_wgsl.rs:1021-1033: enabled Bounded or Instances not reached negatively).
    // Past SF_MAX_UNION_LEAVES leaves the plain exact program runs: the same sample.
    const bool any_fast = std::any_of(g.nodes.begin(), g.nodes.end(), [&](const sf_node& n) {
        return n.enabled && (n.kind == SF_NODE_BOUNDED || n.kind == SF_NODE_INSTANCES) &&
               !L.unsafe_bounds.count(n.id);
    });
    if (any_fast && L.leaves.size() > 1 && L.leaves.size() <= SF_MAX_UNION_LEAVES) {
        P.union_leaves = uint32_t(L.leaves.size());
        for (size_t i = 0; i < L.leaves.size(); ++i) {
            P.leaf_begin[i] = uint8_t(L.leaves[i].begin);
            P.leaf_end[i] = uint8_t(L.leaves[i].end);
        }
    }
    P.inst_floats = uint32_t(inst.size());
    detect_form(g, P);
    std::memset(&info, 0, sizeof info);
    info.step_scale = g.safety / lip;
    info.lipschitz = lip;
    for (int i = 0; i < 4; ++i) info.trap_scales[i] = P.trap_scales[i];
    info.iteration_product = P.iteration_product;
    info.form = P.form;
    info.op_count = P.n_ops;
    info.bounding_radius_hint = g.hint;
    info.exact_union_leaves = P.form == SF_FORM_GENERIC ? P.union_leaves : 0;
    return SF_OK;
}

sf_status scene_check(const sf_scene_desc& d, uint32_t max_lights, bool inline_shadows) {
    if (d.finish_count > SF_MAX_FINISHES) return fail(SF_ERR_INVALID, "more than 8 finishes");
    if (!d.light_list && d.light_count > SF_MAX_LIGHTS)
        return fail(SF_ERR_INVALID, "more than 8 inline lights (light_list holds up to 96)");
    if (d.light_list && d.light_list_count > SF_MAX_SCENE_LIGHTS)
        return fail(SF_ERR_INVALID, "a scene may have at most 96 lights");  // Scene::validate (scene/mod.rs:512)
    const uint32_t n_lights = scene_light_count(d);
    if (n_lights > max_lights)
        return fail(SF_ERR_UNSUPPORTED, "more than 8 lights: batches, the server, previews and exports take 8, "
                                        "sessions up to 96");
    const sf_area_light* lights = scene_lights(d);
    for (uint32_t i = 0; i < n_lights; ++i) {
        const sf_area_light& l = lights[i];
        if (l.kind > SF_LIGHT_TUBE) return fail(SF_ERR_UNSUPPORTED, "light kind not built on the device");
        // Light::visit_params bounds (light.rs:162-226)
        if (l.kind == SF_LIGHT_PROJECTOR &&
            !(l.direction[0] >= 0.1f && l.direction[1] <= 89.0f && l.direction[0] <= l.direction[1] - 0.01f))
            return fail(SF_ERR_INVALID, "projector angles: inner in [0.1, outer - 0.01], outer at most 89 degrees");
        if (l.kind == SF_LIGHT_TUBE) {
            const float dx = l.edge_u[0] - l.center[0], dy = l.edge_u[1] - l.center[1], dz = l.edge_u[2] - l.center[2];
            if (!(l.edge_v[0] >= 0.001f && l.edge_v[0] <= 1000.0f))
                return fail(SF_ERR_INVALID, "tube radius must lie in [0.001, 1000]");
            if (!(dx * dx + dy * dy + dz * dz > 0.0f)) return fail(SF_ERR_INVALID, "a tube needs distinct ends");
        }
        if (l.kind == SF_LIGHT_HDRI && !l.environment)
            return fail(SF_ERR_INVALID, "an HDRI light needs a panorama (sf_environment_create)");
    }
    if (d.coloring.stop_count > SF_MAX_RAMP_STOPS) return fail(SF_ERR_INVALID, "more than 16 ramp stops");
    for (uint32_t i = 0; i < d.finish_count; ++i) {
        const sf_finish_detail& f = d.details[i];
        if (f.pattern > 12) return fail(SF_ERR_INVALID, "finish detail pattern out of range (0..12)");
        if (f.pattern && !(f.scale >= 0.01f && f.scale <= 200.0f))  // FinishDetail bounds (material.rs:226-231)
            return fail(SF_ERR_INVALID, "finish detail scale must lie in [0.01, 200]");
    }
    for (uint32_t i = 0; i <= SF_MAX_FINISHES; ++i) {
        const sf_optics& o = d.optics[i];
        if (!o.enabled) continue;
        // Optics bounds (optics.rs:40-72)
        if (!(o.ior >= 1.0f && o.ior <= 3.0f) || !(o.opacity >= 0.0f && o.opacity <= 1.0f) ||
            !(o.transmission >= 0.0f && o.transmission <= 1.0f) ||
            !(o.absorption_distance >= 0.001f && o.absorption_distance <= 1000.0f) ||
            !(o.subsurface_radius >= 0.001f && o.subsurface_radius <= 1000.0f) ||
            !(o.subsurface >= 0.0f && o.subsurface <= 1.0f))
            return fail(SF_ERR_INVALID, "optics parameter out of range");
    }
    const sf_texture& t = d.texture;
    if (t.graph) {
        // FractalTexture bounds (texture.rs:196-215)
        if (t.octaves < 1 || t.octaves > 4) return fail(SF_ERR_INVALID, "texture octaves must lie in 1..4");
        if (t.parallax_steps < 4 || t.parallax_steps > 32)
            return fail(SF_ERR_INVALID, "texture parallax steps must lie in 4..32");
        if (!(t.channel <= 4 || t.channel == 6 || t.channel == 7)) return fail(SF_ERR_INVALID, "texture channel");
        if (t.mask && t.mask_slot > 3) return fail(SF_ERR_INVALID, "texture mask slot must lie in 0..3");
        if (t.fan && !(t.fan_period[0] > 0.0f && t.fan_period[1] > 0.0f))
            return fail(SF_ERR_INVALID, "texture fan periods must be positive");
        if (!(t.scale > 0.0f)) return fail(SF_ERR_INVALID, "texture scale must be positive");
        if (t.ramp.stop_count == 0 || t.ramp.stop_count > SF_MAX_RAMP_STOPS)
            return fail(SF_ERR_INVALID, "the texture ramp needs 1..16 stops");
    }
    if (!(d.fog.density >= 0.0f) || !(std::fabs(d.fog.anisotropy) < 1.0f))
        return fail(SF_ERR_INVALID, "fog density must be >= 0 and anisotropy in (-1, 1)");
    if (!inline_shadows && shadow_slots_of(d) > 8)
        return fail(SF_ERR_UNSUPPORTED, "more than 8 shadow segments per bounce (sky lights, and emitters in fog): "
                                        "the wavefront stores them; the megakernel integrator traces them inline");
    return SF_OK;
}
// Shadow segments one bounce can issue: the surface's next events (the selected area
// light, every sky light) or a fog scattering point's (every sky light), plus, in fog,
// one per area light for the segment's line integral.
uint32_t shadow_slots_of(const sf_scene_desc& d) {
    uint32_t area = 0, sky = 0;
    const sf_area_light* lights = scene_lights(d);
    for (uint32_t i = 0; i < scene_light_count(d); ++i)
        (lights[i].kind == SF_LIGHT_AREA || lights[i].kind == SF_LIGHT_PROJECTOR || lights[i].kind == SF_LIGHT_TUBE
             ? area
             : sky)++;
    return 1 + sky + (d.fog.density > 0.0f ? area : 0);
}
void light_dev(const sf_area_light& l, DevLight& o) {
    std::memset(&o, 0, sizeof o);
    o.kind = l.kind;
    auto lum = [](const float* c) { return c[0] * 0.2126f + c[1] * 0.7152f + c[2] * 0.0722f; };
    if (l.kind == SF_LIGHT_SUN) {
        // GpuLight::from_light (uniforms.rs:656-668): normalised direction, cos of the half angle
        std::memcpy(o.a, l.direction, 12);
        std::memcpy(o.color, l.radiance, 12);
        o.cos_max = cosf((l.angular_size * 0.5f) * (3.14159265f / 180.0f));
        return;
    }
    if (l.kind == SF_LIGHT_HDRI) {
        // GpuLight::from_light (uniforms.rs:643-654): rotation as cos/sin, intensity
        const float r = l.rotation * (3.14159265f / 180.0f);
        o.a[0] = cosf(r);
        o.a[1] = sinf(r);
        o.color[0] = l.radiance[0];
        environment_dev(l.environment, o);
        return;
    }
    if (l.kind == SF_LIGHT_ENVIRONMENT) {
        std::memcpy(o.a, l.zenith, 12);
        std::memcpy(o.b, l.horizon, 12);
        std::memcpy(o.c, l.ground, 12);
        o.energy = std::max(std::max(lum(l.zenith), lum(l.horizon)), lum(l.ground));
        float peak = 0.0f;
        for (int k = 0; k < 3; ++k) peak = std::max({peak, l.zenith[k], l.horizon[k], l.ground[k]});
        o.peak = peak;
        return;
    }
    if (l.kind == SF_LIGHT_TUBE) {
        // GpuLight::from_light (uniforms.rs:717-729): start, end, radius, length
        std::memcpy(o.a, l.center, 12);
        std::memcpy(o.b, l.edge_u, 12);
        std::memcpy(o.color, l.radiance, 12);
        const float dx = l.edge_u[0] - l.center[0], dy = l.edge_u[1] - l.center[1], dz = l.edge_u[2] - l.center[2];
        o.radius = l.edge_v[0];
        o.length = sqrtf(dx * dx + dy * dy + dz * dz);
        o.area = 2.0f * 3.14159265f * o.radius * (o.length + 2.0f * o.radius);  // emitter_area, lights.wgsl:80-85
        o.n[1] = 1.0f;
        o.lum = lum(l.radiance);
        return;
    }
    // a projector is an area light with its beam (kind.y = 1, uniforms.rs:690-715)
    o.kind = SF_LIGHT_AREA;
    if (l.kind == SF_LIGHT_PROJECTOR) {
        const float deg = 3.14159265f / 180.0f;
        o.projector = 1;
        o.beam[0] = cosf(l.direction[0] * deg);
        o.beam[1] = cosf(l.direction[1] * deg);
        o.beam[2] = tanf(l.direction[1] * deg);
    }
    std::memcpy(o.a, l.center, 12);
    std::memcpy(o.b, l.edge_u, 12);
    std::memcpy(o.c, l.edge_v, 12);
    std::memcpy(o.color, l.radiance, 12);
    float cx = l.edge_u[1] * l.edge_v[2] - l.edge_u[2] * l.edge_v[1];
    float cy = l.edge_u[2] * l.edge_v[0] - l.edge_u[0] * l.edge_v[2];
    float cz = l.edge_u[0] * l.edge_v[1] - l.edge_u[1] * l.edge_v[0];
    float len = sqrtf(cx * cx + cy * cy + cz * cz);
    float rcp = 1.0f / len;
    if (!(len > 0.f) || !(rcp > 0.f) || !(rcp <= 3.4028235e38f)) { o.n[0] = 0; o.n[1] = 1; o.n[2] = 0; }
    else { o.n[0] = cx * rcp; o.n[1] = cy * rcp; o.n[2] = cz * rcp; }
    o.area = len;
    float bb = l.edge_u[0] * l.edge_u[0] + l.edge_u[1] * l.edge_u[1] + l.edge_u[2] * l.edge_u[2];
    float cc = l.edge_v[0] * l.edge_v[0] + l.edge_v[1] * l.edge_v[1] + l.edge_v[2] * l.edge_v[2];
    o.inv_bb = 1.0f / bb;
    o.inv_cc = 1.0f / cc;
    o.lum = lum(l.radiance);
}
void material_dev(const sf_material& m, DevMaterial& o) {
    std::memcpy(o.albedo, m.albedo, 12);
    o.roughness = m.roughness;
    o.metallic = m.metallic;
    o.specular = m.specular;
    std::memcpy(o.emission, m.emission, 12);
}
// GpuRamp::from_ramp (uniforms.rs) of a colouring or texture ramp.
static void ramp_dev(const sf_coloring& c, DevRamp& r) {
    r.n = std::min<uint32_t>(c.stop_count, SF_MAX_RAMP);
    r.cyclic = c.cyclic;
    r.smooth = c.smooth;
    r.positioned = c.positioned;
    r.map[0] = c.frequency;
    r.map[1] = c.phase;
    r.map[2] = c.gamma;
    std::memcpy(r.stops, c.stops, sizeof r.stops);
}
void scene_lights_dev(const sf_scene_desc& d, std::vector<DevLight>& more) {
    const uint32_t n = scene_light_count(d);
    more.assign(n > SF_SHARED_LIGHTS ? n - SF_SHARED_LIGHTS : 0, DevLight{});
    for (uint32_t i = SF_SHARED_LIGHTS; i < n; ++i) light_dev(scene_lights(d)[i], more[i - SF_SHARED_LIGHTS]);
}
// Uniforms::from_scene (uniforms.rs:748-830) for the DE path.
void scene_dev(const sf_scene_desc& d, const sf_render_config& c, const sf_graph_info& gi, DevScene& S) {
    std::memset(&S, 0, sizeof S);
    std::memcpy(S.origin, d.camera.origin, 12);
    std::memcpy(S.forward, d.camera.forward, 12);
    std::memcpy(S.right, d.camera.right, 12);
    std::memcpy(S.up, d.camera.up, 12);
    S.tan_half = d.camera.tan_half_fov;
    S.aspect = d.camera.aspect;
    S.lens_radius = d.camera.lens_radius;
    S.focus_distance = d.camera.focus_distance;
    S.width = c.width;
    S.height = c.height;
    S.max_bounces = c.max_bounces;
    S.max_steps = c.max_steps;
    S.seed = uint32_t(d.seed) ^ uint32_t(d.seed >> 32);
    S.light_count = scene_light_count(d);  // lights past SF_SHARED_LIGHTS: the light table
    S.finish_count = std::min<uint32_t>(d.finish_count, SF_MAX_FINISHES);
    S.variation_slot = d.variation_slot;
    S.variation_enabled = d.variation_enabled;
    S.var_rough[0] = d.variation_roughness[0];
    S.var_rough[1] = d.variation_roughness[1];
    S.var_metal[0] = d.variation_metallic[0];
    S.var_metal[1] = d.variation_metallic[1];
    S.cavity = d.cavity_darkness;
    S.pixel_tolerance = c.pixel_tolerance;
    S.step_scale = gi.step_scale;
    float ol = sqrtf(d.camera.origin[0] * d.camera.origin[0] + d.camera.origin[1] * d.camera.origin[1] +
                     d.camera.origin[2] * d.camera.origin[2]);
    float far = std::max(2.0f * gi.bounding_radius_hint + ol, 200.0f);  // uniforms.rs:781-782
    S.extent = std::max(200.0f, far);                                   // ray_extent, common.wgsl:206-208
    S.pixel_cone = d.camera.tan_half_fov * 2.0f / float(c.width);
    S.hit_eps = c.hit_epsilon;
    S.iteration_product = gi.iteration_product;
    material_dev(d.material, S.material);
    for (uint32_t i = 0; i < S.finish_count; ++i) material_dev(d.finishes[i], S.finishes[i]);
    for (uint32_t i = 0; i < std::min<uint32_t>(S.light_count, SF_SHARED_LIGHTS); ++i)
        light_dev(scene_lights(d)[i], S.lights[i]);
    S.shadow_slots = shadow_slots_of(d);
    // GpuAtmosphere (uniforms.rs:217-227): fog in a, its colour in b
    S.fog[0] = d.fog.density;
    S.fog[1] = d.fog.height;
    S.fog[2] = d.fog.falloff;
    S.fog[3] = d.fog.anisotropy;
    std::memcpy(S.fog_color, d.fog.color, 12);
    S.col_slot = d.coloring.slot;
    ramp_dev(d.coloring, S.col);
    std::memcpy(S.col_weights, d.coloring_orbit.traps, 16);
    S.col_extra[0] = d.coloring_orbit.iterations;
    S.col_extra[1] = d.coloring_orbit.normal;
    S.col_extra[2] = d.coloring_orbit.logarithmic;
    // finish details (GpuFinish.detail_*, uniforms.rs:797-815)
    S.dune_wind = d.dune_wind * (3.14159265f / 180.0f);
    for (uint32_t i = 0; i < S.finish_count; ++i) {
        const sf_finish_detail& f = d.details[i];
        DevDetail& o = S.details[i];
        o.kind = f.pattern;
        o.seed = f.seed;
        o.mapping[0] = f.scale;
        o.mapping[1] = f.strength;
        o.mapping[2] = f.bump;
        o.mapping[3] = f.roughness_delta;
        std::memcpy(o.tint, f.tint, 12);
        if (f.pattern) S.rich |= SF_RICH_DETAIL;
        if (f.pattern >= 10) S.rich |= SF_RICH_ROUGH_DIFFUSE;
    }
    // GpuOptics::from_optics (uniforms.rs:103-122); slots past the finish count stay opaque
    for (uint32_t i = 0; i <= S.finish_count; ++i) {
        const sf_optics& o = d.optics[i];
        if (!o.enabled) continue;
        DevOptics& g = S.optics[i];
        g.surface[0] = o.opacity;
        g.surface[1] = o.transmission;
        g.surface[2] = o.ior;
        g.surface[3] = o.thin_walled ? 1.0f : 0.0f;
        for (int k = 0; k < 3; ++k)
            g.absorption[k] = -logf(std::max(o.absorption_color[k], 0.0001f)) / o.absorption_distance;
        g.absorption[3] = o.absorption_distance;
        std::memcpy(g.subsurface, o.subsurface_color, 12);
        g.subsurface[3] = o.subsurface / o.subsurface_radius;
        S.rich |= SF_RICH_OPTICS;
    }
    // GpuTexture::from_texture (uniforms.rs:340-379)
    const sf_texture& t = d.texture;
    if (t.graph) {
        DevTexture& x = S.tex;
        x.channel = t.channel;
        x.octaves = t.octaves;
        x.budget = t.graph->info.iteration_product;  // FractalTexture::iteration_budget
        x.enabled = 1;
        std::memcpy(x.mapping, t.offset, 12);
        x.mapping[3] = t.scale;
        for (int k = 0; k < 3; ++k) x.rotation[k] = t.rotation[k] * (3.14159265f / 180.0f);
        x.rotation[3] = t.contrast;
        x.effects[0] = t.strength;
        x.effects[1] = t.roughness;
        x.effects[2] = t.bump;
        x.effects[3] = 1.0f;
        if (t.channel == 7) {
            std::memcpy(x.weights, t.orbit.traps, 16);
            x.extra[0] = t.orbit.iterations;
            x.extra[1] = t.orbit.normal;
            x.extra[2] = t.orbit.logarithmic;
        }
        x.parallax[0] = t.parallax;
        x.parallax[1] = float(t.parallax_steps);
        if (t.fan) {
            x.fan[0] = t.fan_period[0];
            x.fan[1] = t.fan_period[1];
            x.fan[2] = float(t.fan_rays);
            x.fan[3] = 1.0f;
        }
        if (t.mask) {
            x.mask[0] = float(t.mask_slot);
            x.mask[1] = t.mask_value;
            x.mask[2] = t.mask_width;
            x.mask[3] = 1.0f;
        }
        x.prog = reinterpret_cast<uint64_t>(t.graph->d_prog);
        ramp_dev(t.ramp, x.ramp);
        S.rich |= SF_RICH_TEXTURE;
    }
}

}  // namespace sfh

// Error reporting for the other translation units of the library.
sf_status sf_report_error(sf_status status, const std::string& message) { return sfh::fail(status, message); }

using namespace sfh;

// ------------------------------------------------------------------ ABI: basics
extern "C" const char* sf_status_string(sf_status s) {
    static const char* names[] = {"SF_OK", "SF_ERR_INVALID", "SF_ERR_GRAPH", "SF_ERR_UNSUPPORTED", "SF_ERR_CUDA",
                                  "SF_ERR_OOM", "SF_ERR_TIMEOUT", "SF_ERR_BUDGET", "SF_ERR_IO", "SF_ERR_CHECKPOINT",
                                  "SF_ERR_WAVEFRONT", "SF_ERR_NO_DEVICE", "SF_ERR_BUSY"};
    if (s < 0 || s > 12) return "SF_ERR_UNKNOWN";
    return names[s];
}
extern "C" const char* sf_last_error(void) { return g_error.c_str(); }
extern "C" uint32_t sf_abi_version(void) { return ABI_VERSION; }

extern "C" sf_status sf_context_create(int device, uint64_t budget, sf_context** out) {
    if (!out) return fail(SF_ERR_INVALID, "null output");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(SF_ERR_NO_DEVICE, "no CUDA device available");
    if (device < 0 || device >= count) return fail(SF_ERR_INVALID, "device index out of range");
    CU(cudaSetDevice(device));
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, device));
    auto* c = new sf_context();
    c->device = device;
    c->device_name = prop.name;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    c->sm_count = prop.multiProcessorCount;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    c->budget = budget ? budget : uint64_t(double(free_b) * 0.9);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }
    void* p = nullptr;
    sf_status s = ctx_alloc(c, SF_STAT_COUNT * sizeof(unsigned long long) + 64 * sizeof(uint32_t), &p);
    if (s != SF_OK) { cudaStreamDestroy(c->stream); delete c; return s; }
    c->d_stats = static_cast<unsigned long long*>(p);
    c->d_work = reinterpret_cast<uint32_t*>(c->d_stats + SF_STAT_COUNT);
    cudaMemsetAsync(p, 0, SF_STAT_COUNT * sizeof(unsigned long long) + 64 * sizeof(uint32_t), c->stream);
    *out = c;
    return SF_OK;
}
extern "C" sf_status sf_context_destroy(sf_context* c) {
    if (!c) return SF_OK;
    ctx_release(c);
    return SF_OK;
}
extern "C" sf_status sf_context_stream(sf_context* c, void** s) {
    if (!c || !s) return fail(SF_ERR_INVALID, "null argument");
    *s = c->stream;
    return SF_OK;
}
extern "C" sf_status sf_context_memory(sf_context* c, uint64_t* used, uint64_t* budget) {
    if (!c) return fail(SF_ERR_INVALID, "null context");
    if (used) *used = c->used;
    if (budget) *budget = c->budget;
    return SF_OK;
}
extern "C" sf_status sf_context_set_profiling(sf_context* c, int enable) {
    if (!c) return fail(SF_ERR_INVALID, "null context");
    if (enable < 0 || enable > 2) return fail(SF_ERR_INVALID, "profiling level must be 0, 1 or 2");
    collect_timing(c);
    c->profiling = enable != 0;
    c->lane_stats = enable == 2;
    return SF_OK;
}
extern "C" sf_status sf_context_reset_stats(sf_context* c) {
    if (!c) return fail(SF_ERR_INVALID, "null context");
    cudaSetDevice(c->device);
    collect_timing(c);
    c->kernel_ms = c->trace_ms = 0;
    c->launches = c->trace_launches = 0;
    CU(cudaMemsetAsync(c->d_stats, 0, SF_STAT_COUNT * sizeof(unsigned long long), c->stream));
    return SF_OK;
}
extern "C" sf_status sf_context_stats(sf_context* c, sf_stats* out) {
    if (!c || !out) return fail(SF_ERR_INVALID, "null argument");
    cudaSetDevice(c->device);
    collect_timing(c);
    unsigned long long h[SF_STAT_COUNT];
    CU(cudaMemcpyAsync(h, c->d_stats, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    std::memset(out, 0, sizeof *out);
    out->de_evals = h[SF_STAT_DE_EVALS];
    out->de_iterations = h[SF_STAT_DE_ITERS];
    out->segments = h[SF_STAT_SEGMENTS];
    out->shadow_segments = h[SF_STAT_SHADOW_SEGMENTS];
    out->steps = h[SF_STAT_STEPS];
    out->warp_de_calls = h[SF_STAT_WARP_DE_CALLS];
    out->iteration_slots = h[SF_STAT_ITER_SLOTS];
    out->warp_cycles = h[SF_STAT_WARP_CYCLES];
    out->tail_cycles = h[SF_STAT_TAIL_CYCLES];
    out->launches = c->launches;
    out->kernel_ms = c->kernel_ms;
    out->trace_ms = c->trace_ms;
    out->trace_launches = c->trace_launches;
    return SF_OK;
}
extern "C" sf_status sf_context_sync(sf_context* c, uint32_t timeout_ms) {
    if (!c) return fail(SF_ERR_INVALID, "null context");
    cudaSetDevice(c->device);
    return wait_stream(c->stream, timeout_ms);
}

// ------------------------------------------------------------------ ABI: graph
extern "C" sf_status sf_graph_validate(const sf_graph_desc* d, sf_graph_info* out) {
    HostGraph h;
    DeProgram P;
    sf_graph_info info;
    std::vector<float> inst;
    sf_status s = build_graph(d, h, P, info, inst);
    if (s == SF_OK && out) *out = info;
    return s;
}
extern "C" sf_status sf_graph_compile(sf_context* c, const sf_graph_desc* d, sf_graph** out) {
    if (!c || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    auto* g = new sf_graph();
    g->ctx = c;
    std::vector<float> inst;
    sf_status s = build_graph(d, g->host, g->prog, g->info, inst);
    if (s != SF_OK) { delete g; return s; }
    g->topology = topology_of(g->host);
    cudaSetDevice(c->device);
    void* p = nullptr;
    if (!inst.empty()) {
        g->inst_bytes = inst.size() * sizeof(float);
        s = ctx_alloc(c, g->inst_bytes, &p);
        if (s != SF_OK) { delete g; return s; }
        g->d_inst = static_cast<float*>(p);
        g->prog.inst_data = reinterpret_cast<uint64_t>(g->d_inst);
    }
    s = ctx_alloc(c, sizeof(DeProgram), &p);
    if (s != SF_OK) {
        if (g->d_inst) ctx_free(c, g->d_inst, g->inst_bytes);
        delete g;
        return s;
    }
    g->d_prog = static_cast<DeProgram*>(p);
    cudaError_t e = cudaSuccess;
    if (g->d_inst) e = cudaMemcpyAsync(g->d_inst, inst.data(), g->inst_bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->d_prog, &g->prog, sizeof(DeProgram), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        ctx_free(c, g->d_prog, sizeof(DeProgram));
        if (g->d_inst) ctx_free(c, g->d_inst, g->inst_bytes);
        delete g;
        return cuda_fail(e, "graph upload");
    }
    ctx_retain(c);
    *out = g;
    return SF_OK;
}
extern "C" sf_status sf_graph_info_get(const sf_graph* g, sf_graph_info* out) {
    if (!g || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = g->info;
    return SF_OK;
}
extern "C" sf_status sf_graph_update(sf_graph* g, const sf_graph_desc* d) {
    if (!g) return fail(SF_ERR_INVALID, "null graph");
    HostGraph h;
    DeProgram P;
    sf_graph_info info;
    std::vector<float> inst;
    sf_status s = build_graph(d, h, P, info, inst);
    if (s != SF_OK) return s;
    if (topology_of(h) != g->topology || inst.size() * sizeof(float) != g->inst_bytes)
        return fail(SF_ERR_GRAPH, "topology changed: compile a new graph");
    P.inst_data = reinterpret_cast<uint64_t>(g->d_inst);
    cudaSetDevice(g->ctx->device);
    CU(cudaDeviceSynchronize());  // no launch on any stream (previews, server slots) may read what is replaced
    if (g->d_inst) CU(cudaMemcpyAsync(g->d_inst, inst.data(), g->inst_bytes, cudaMemcpyHostToDevice, g->ctx->stream));
    CU(cudaMemcpyAsync(g->d_prog, &P, sizeof P, cudaMemcpyHostToDevice, g->ctx->stream));
    CU(cudaStreamSynchronize(g->ctx->stream));
    g->host = h;
    g->prog = P;
    g->info = info;
    return SF_OK;
}
namespace sfh {
void graph_retain(sf_graph* g) {
    std::lock_guard<std::mutex> lk(g->ctx->mu);
    g->refs++;
}
}  // namespace sfh
extern "C" sf_status sf_graph_destroy(sf_graph* g) {
    if (!g) return SF_OK;
    sf_context* c = g->ctx;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        if (--g->refs > 0) return SF_OK;
    }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    ctx_free(c, g->d_prog, sizeof(DeProgram));
    if (g->d_inst) ctx_free(c, g->d_inst, g->inst_bytes);
    delete g;
    ctx_release(c);
    return SF_OK;
}

// ------------------------------------------------------------------ ABI: DE probe
extern "C" sf_status sf_de_probe_device(sf_graph* g, const float* x, const float* y, const float* z, size_t n,
                                        float* dist, float* traps, uint32_t* iters, uint32_t* mats) {
    if (!g) return fail(SF_ERR_INVALID, "null graph");
    if (n && (!x || !y || !z || !dist || !traps || !iters || !mats)) return fail(SF_ERR_INVALID, "null buffer");
    sf_context* c = g->ctx;
    cudaSetDevice(c->device);
    LaunchTimer t(c, true);
    CU(sf_launch_de_probe(g->d_prog, x, y, z, n, dist, traps, iters, mats, c->stream));
    return SF_OK;
}

extern "C" sf_status sf_de_probe(sf_graph* g, const float* xyz, size_t n, sf_de_sample* out) {
    if (!g) return fail(SF_ERR_INVALID, "null graph");
    if (n == 0) return SF_OK;
    if (!xyz || !out) return fail(SF_ERR_INVALID, "null buffer");
    sf_context* c = g->ctx;
    cudaSetDevice(c->device);
    std::vector<float> soa(3 * n);
    for (size_t i = 0; i < n; ++i) {
        soa[i] = xyz[3 * i];
        soa[n + i] = xyz[3 * i + 1];
        soa[2 * n + i] = xyz[3 * i + 2];
    }
    size_t bytes = n * (3 + 1 + 4) * sizeof(float) + 2 * n * sizeof(uint32_t);
    void* buf = nullptr;
    sf_status s = ctx_alloc(c, bytes, &buf);
    if (s != SF_OK) return s;
    float* d_in = static_cast<float*>(buf);
    float* d_dist = d_in + 3 * n;
    float* d_traps = d_dist + n;
    uint32_t* d_iter = reinterpret_cast<uint32_t*>(d_traps + 4 * n);
    uint32_t* d_mat = d_iter + n;
    std::vector<float> h_dist(n), h_traps(4 * n);
    std::vector<uint32_t> h_iter(n), h_mat(n);
    cudaError_t e = cudaMemcpyAsync(d_in, soa.data(), 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        LaunchTimer t(c, true);
        e = sf_launch_de_probe(g->d_prog, d_in, d_in + n, d_in + 2 * n, n, d_dist, d_traps, d_iter, d_mat, c->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_dist.data(), d_dist, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_traps.data(), d_traps, 4 * n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_iter.data(), d_iter, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_mat.data(), d_mat, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, buf, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "sf_de_probe");
    for (size_t i = 0; i < n; ++i) {
        out[i].distance = h_dist[i];
        for (int k = 0; k < 4; ++k) out[i].traps[k] = h_traps[k * n + i];
        out[i].iterations = h_iter[i];
        out[i].material = h_mat[i];
    }
    return SF_OK;
}

// ------------------------------------------------------------------ ABI: primary rays
extern "C" sf_status sf_primary_trace(sf_graph* g, const sf_primary_desc* d, float* t_out, uint32_t* steps_out,
                                      float* normal_out) {
    if (!g || !d) return fail(SF_ERR_INVALID, "null argument");
    if (!d->width || !d->height) return fail(SF_ERR_INVALID, "empty image");
    if (!t_out || !steps_out || !normal_out) return fail(SF_ERR_INVALID, "null output");
    sf_context* c = g->ctx;
    cudaSetDevice(c->device);
    size_t n = size_t(d->width) * d->height;
    sf_scene_desc sd;
    std::memset(&sd, 0, sizeof sd);
    sd.camera = d->camera;
    sf_render_config rc;
    std::memset(&rc, 0, sizeof rc);
    rc.width = d->width;
    rc.height = d->height;
    rc.max_steps = d->max_steps;
    rc.pixel_tolerance = d->pixel_tolerance > 0 ? d->pixel_tolerance : 1.0f;
    DevScene S;
    scene_dev(sd, rc, g->info, S);
    const size_t bytes = sizeof(DevScene) + n * (1 + 1 + 3) * 4;
    // the context's scratch and pinned staging, kept between calls
    std::lock_guard<std::mutex> lk(c->stage_mu);
    if (const sf_status s = ensure_scratch(c, bytes); s != SF_OK) return s;
    void* buf = c->scratch;
    DevScene* dS = static_cast<DevScene*>(buf);
    float* dt = reinterpret_cast<float*>(reinterpret_cast<char*>(buf) + sizeof(DevScene));
    uint32_t* ds = reinterpret_cast<uint32_t*>(dt + n);
    float* dn = reinterpret_cast<float*>(ds + n);
    cudaError_t e = cudaMemcpyAsync(dS, &S, sizeof S, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_work, 0, 4, c->stream);
    if (e == cudaSuccess) {
        LaunchTimer t(c, true);
        e = sf_launch_primary(g->d_prog, dS, d->width, d->height, d->max_steps, d->rule, d->eps, d->t_far,
                              d->normal_mode, dt, ds, dn, c->d_work, c->d_stats, 1, c->stream);
    }
    // t, steps and normals are contiguous after the scene: one copy into the staging
    if (e == cudaSuccess) e = ensure_stage(c, n * 20);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->stage, dt, n * 20, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "sf_primary_trace");
    const char* st = static_cast<const char*>(c->stage);
    host_parallel(n, [&](size_t b, size_t end) {
        std::memcpy(t_out + b, st + b * 4, (end - b) * 4);
        std::memcpy(steps_out + b, st + n * 4 + b * 4, (end - b) * 4);
        std::memcpy(normal_out + 3 * b, st + n * 8 + b * 12, (end - b) * 12);
    });
    return SF_OK;
}

// ------------------------------------------------------------------ sessions

namespace sfh {


void tile_grid(sf_session* s) {
    s->tiles.clear();
    uint32_t ts = std::max<uint32_t>(s->tile_size, 8);  // MIN_TILE_SIZE, tiles.rs:1
    for (uint32_t y = 0; y < s->cfg.height; y += std::min(ts, s->cfg.height - y)) {
        uint32_t h = std::min(ts, s->cfg.height - y);
        for (uint32_t x = 0; x < s->cfg.width; x += std::min(ts, s->cfg.width - x)) {
            uint32_t w = std::min(ts, s->cfg.width - x);
            s->tiles.push_back({x, y, w, h, 0});
        }
    }
}

sf_status validate_config(const sf_render_config& c) {
    // RenderConfig::validate (renderer.rs:81-138)
    if (c.width < 1 || c.height < 1) return fail(SF_ERR_INVALID, "width and height must be at least 1");
    if (c.samples_per_pixel < 1) return fail(SF_ERR_INVALID, "samples_per_pixel must be at least 1");
    if (c.max_bounces > 32) return fail(SF_ERR_INVALID, "max_bounces must be at most 32");
    if (c.max_steps < 1) return fail(SF_ERR_INVALID, "max_steps must be at least 1");
    if (!(c.pixel_tolerance >= 0.125f && c.pixel_tolerance <= 1.0f))
        return fail(SF_ERR_INVALID, "pixel_tolerance must be between 0.125 and 1.0");
    if (!(c.hit_epsilon >= 0.0f && c.hit_epsilon <= 1.0f))
        return fail(SF_ERR_INVALID, "hit_epsilon must be between 0 (cone-relative test) and 1.0");
    if (c.integrator > SF_INTEGRATOR_WAVEFRONT) return fail(SF_ERR_INVALID, "unknown integrator");
    return SF_OK;
}

sf_status session_alloc(sf_session* s) {
    sf_context* c = s->ctx;
    const sf_render_config& cfg = s->cfg;
    uint32_t ts = std::max<uint32_t>(cfg.tile_size ? cfg.tile_size : 256, 8);
    s->tile_size = ts;
    uint32_t tw = std::min(ts, cfg.width), th = std::min(ts, cfg.height);
    uint32_t spd = std::max<uint32_t>(std::min(cfg.samples_per_dispatch ? cfg.samples_per_dispatch : 1,
                                               cfg.samples_per_pixel), 1);
    s->cfg.samples_per_dispatch = spd;
    uint64_t cap64 = uint64_t(tw) * th * spd;
    if (cap64 > 0x7fffffffull) return fail(SF_ERR_INVALID, "tile_size^2 * samples_per_dispatch too large");
    s->capacity = uint32_t(cap64);
    const size_t N = s->capacity;
    // a window session (a tiled export's) holds a tile-sized film; others the image
    const uint32_t fw = s->window ? tw : cfg.width, fh = s->window ? th : cfg.height;
    const size_t px = size_t(fw) * fh;
    const bool wf = cfg.integrator == SF_INTEGRATOR_WAVEFRONT;
    const uint32_t R = rounds_of(cfg, s->scene);
    // layout
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    size_t o_scene = take(sizeof(DevScene));
    std::vector<DevLight> more;  // lights past the staged ones: the light table, right after the scene
    scene_lights_dev(s->scene, more);
    size_t o_lights = more.empty() ? 0 : take(more.size() * sizeof(DevLight));
    if (!more.empty() && o_lights != o_scene + SF_LIGHT_TABLE_OFFSET) return fail(SF_ERR_INVALID, "light table layout");
    s->light_smem = uint32_t(more.size() * sizeof(DevLight));  // staged per block by the light-reading kernels
    size_t o_acc = take(px * 16), o_depth = take(px * 4), o_aux = take(px * 16);
    size_t o_Ls = take(N * 16);
    // fog scenes keep the film's volume layer split: a per-path volume row and three planes
    const bool split = has_fog(s->scene);
    size_t o_pv = split ? take(N * 16) : 0, o_vol = split ? take(px * 48) : 0;
    // scenes with finish details, a texture or optics keep a per-path footprint and medium row
    const bool rich = wf && rich_of(s->scene) != 0u;
    size_t o_ex = rich ? take(N * 16) : 0;
    size_t o_soa = 0, o_lists = 0, o_march = 0, o_resume = 0;
    const uint32_t K = shadow_slots_of(s->scene);  // shadow segments one bounce may issue
    s->shadow_slots = K;
    if (wf) {
        o_soa = take(wave_soa_bytes(N, K));
        o_lists = take(wave_lists_bytes(N, K));
        o_march = take(wave_march_bytes(N, K));
        o_resume = take(wave_resume_bytes(N, K));
    }
    size_t o_counts = take(size_t(R + 1) * 4 * 4);
    size_t o_qcounts = take(size_t(R) * 64 * 2 * 4);
    size_t o_status = take(16);
    s->mem_bytes = off;
    sf_status st = ctx_alloc(c, off, &s->mem);
    if (st != SF_OK) return st;
    char* base = static_cast<char*>(s->mem);
    s->d_scene = reinterpret_cast<DevScene*>(base + o_scene);
    s->film.accum = reinterpret_cast<float4*>(base + o_acc);
    s->film.depth = reinterpret_cast<float*>(base + o_depth);
    s->film.aux = reinterpret_cast<float4*>(base + o_aux);
    s->film.width = fw;
    s->film.height = fh;
    std::memset(&s->soa, 0, sizeof s->soa);
    s->soa.capacity = s->capacity;
    s->soa.shadow_slots = K;
    if (wf) {
        wave_bind(s->soa, base + o_soa, base + o_march, s->capacity, K);
        s->lists = reinterpret_cast<uint32_t*>(base + o_lists);
        s->resume = reinterpret_cast<uint32_t*>(base + o_resume);
    }
    s->soa.Ls = reinterpret_cast<float4*>(base + o_Ls);
    if (rich) s->soa.ex = reinterpret_cast<float4*>(base + o_ex);
    if (split) {
        s->soa.pv = reinterpret_cast<float4*>(base + o_pv);
        s->film.vol = reinterpret_cast<float4*>(base + o_vol);
        s->film.vmom = s->film.vol + px;
        s->film.surf = s->film.vmom + px;
    }
    s->counts = reinterpret_cast<uint32_t*>(base + o_counts);
    s->qcounts = reinterpret_cast<uint32_t*>(base + o_qcounts);
    s->status = reinterpret_cast<uint32_t*>(base + o_status);
    DevScene S;
    scene_dev(s->scene, cfg, s->graph->info, S);
    if (!more.empty()) {
        CU(cudaMemcpyAsync(base + o_lights, more.data(), more.size() * sizeof(DevLight), cudaMemcpyHostToDevice,
                           c->stream));
    }
    CU(cudaMemcpyAsync(s->d_scene, &S, sizeof S, cudaMemcpyHostToDevice, c->stream));
    // depth = -1 and aux = (0,0,0,-1) until sample 0 lands (RenderOutput conventions)
    CU(sf_launch_film_clear(s->film, c->stream));
    CU(cudaMemsetAsync(s->status, 0, 16, c->stream));
    tile_grid(s);
    return SF_OK;
}

}  // namespace sfh

extern "C" sf_status sf_session_create(sf_context* c, sf_graph* g, const sf_scene_desc* scene,
                                       const sf_render_config* cfg, sf_session** out) {
    if (!c || !g || !scene || !cfg || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    sf_status st = validate_config(*cfg);
    if (st != SF_OK) return st;
    if (const sf_status sc =
            scene_check(*scene, SF_MAX_SCENE_LIGHTS, cfg->integrator == SF_INTEGRATOR_MEGAKERNEL);
        sc != SF_OK)
        return sc;
    cudaSetDevice(c->device);
    auto* s = new sf_session();
    s->ctx = c;
    s->graph = g;
    s->scene = *scene;
    if (scene->light_list) {
        s->light_store.assign(scene->light_list, scene->light_list + scene->light_list_count);
        s->scene.light_list = s->light_store.data();
    }
    s->cfg = *cfg;
    st = session_alloc(s);
    if (st != SF_OK) {
        if (s->mem) ctx_free(c, s->mem, s->mem_bytes);
        delete s;
        return st;
    }
    ctx_retain(c);
    graph_retain(g);
    *out = s;
    return SF_OK;
}

namespace sfh {
sf_status check_launch(uint32_t min_blocks, uint32_t quantum, uint32_t regen, bool small_blocks) {
    // 2..4 blocks of 256 threads per SM; a single job may also take 6 or 7 of 128
    const bool ok = (min_blocks >= 2 && min_blocks <= 4) || (small_blocks && (min_blocks == 6 || min_blocks == 7));
    if (!ok) return fail(SF_ERR_INVALID, "trace launch: 2..4 resident blocks per SM (6 or 7 of 128 threads for a session)");
    if (quantum != 0 && quantum < 8) return fail(SF_ERR_INVALID, "step quantum below 8");
    if (regen < 1 || regen > 32) return fail(SF_ERR_INVALID, "regeneration threshold outside 1..32 lanes");
    return SF_OK;
}
}  // namespace sfh

extern "C" sf_status sf_session_set_launch(sf_session* s, uint32_t min_blocks_per_sm, uint32_t quantum,
                                           uint32_t regen) {
    if (!s) return fail(SF_ERR_INVALID, "null session");
    sf_status st = check_launch(min_blocks_per_sm, quantum, regen, true);
    if (st != SF_OK) return st;
    s->min_blocks = min_blocks_per_sm;
    s->quantum = quantum;
    s->regen = regen;
    return SF_OK;
}

extern "C" sf_status sf_session_dispatch(sf_session* s, sf_tile tile, uint32_t samples) {
    if (!s) return fail(SF_ERR_INVALID, "null session");
    if (tile.w == 0 || tile.h == 0 || samples == 0) return SF_OK;
    if (tile.x + tile.w > s->cfg.width || tile.y + tile.h > s->cfg.height)
        return fail(SF_ERR_INVALID, "tile outside the image");
    if (s->window && (tile.x < s->film.x0 || tile.y < s->film.y0 || tile.x + tile.w > s->film.x0 + s->film.width ||
                      tile.y + tile.h > s->film.y0 + s->film.height))
        return fail(SF_ERR_INVALID, "tile outside the window film");
    uint64_t paths = uint64_t(tile.w) * tile.h * samples;
    if (paths > s->capacity) return fail(SF_ERR_INVALID, "tile * samples exceeds the session capacity");
    sf_context* c = s->ctx;
    cudaSetDevice(c->device);
    DispatchGeom g{tile.x, tile.y, tile.w, tile.h, tile.done, samples, uint32_t(paths), s->light_smem};
    cudaStream_t st = c->stream;
    if (s->cfg.integrator == SF_INTEGRATOR_MEGAKERNEL) {
        {
            LaunchTimer t(c, true);
            CU(sf_launch_megakernel(s->graph->d_prog, s->d_scene, rich_of(s->scene), s->soa, g, s->film, c->d_stats,
                                    st));
        }
        LaunchTimer t2(c, false);
        CU(sf_launch_commit(s->soa, g, s->film, st));
        s->dispatches++;
        return SF_OK;
    }
    const uint32_t R = rounds_of(s->cfg, s->scene);
    const size_t N = s->capacity;
    // launches per round: the first, then one per step quantum a segment may still need
    const uint32_t Q = s->quantum ? std::min<uint32_t>((s->cfg.max_steps + s->quantum - 1) / s->quantum + 1, 64) : 1;
    CU(cudaMemsetAsync(s->counts, 0, size_t(R + 1) * 16, st));
    CU(cudaMemsetAsync(s->qcounts, 0, size_t(R) * 64 * 2 * 4, st));
    {
        LaunchTimer t(c, false);
        CU(sf_launch_generate(s->d_scene, s->soa, g, s->counts, st));
    }
    const uint32_t rich = rich_of(s->scene);
    // the optics trace kernel runs 6 blocks of 128 threads per SM
    const int blocks = int((rich & SF_RICH_OPTICS) ? 6u : s->min_blocks) * c->sm_count;
    const uint32_t K = s->shadow_slots;
    for (uint32_t r = 0; r < R; ++r) {
        RoundQueues q;
        wave_round_queues(q, s->lists, N, K, r, s->counts);
        for (uint32_t j = 0; j < Q; ++j) {
            TraceLaunch tl{};
            tl.q = q;
            uint32_t* qc = s->qcounts + (size_t(r) * 64 + j) * 2;
            tl.work_counter = qc;
            tl.resume = j == 0 ? nullptr : wave_resume(s->resume, N, K, j - 1);
            tl.resume_count = j == 0 ? nullptr : qc - 2 + 1;  // previous launch's resumed count
            tl.next_resume = wave_resume(s->resume, N, K, j);
            tl.next_resume_count = qc + 1;
            tl.quantum = j + 1 == Q ? 0u : s->quantum;  // the last launch runs segments to completion
            tl.regen = s->regen;
            tl.lane_stats = c->lane_stats ? 1u : 0u;
            tl.optics = (rich & SF_RICH_OPTICS) ? 1u : 0u;
            LaunchTimer t(c, true);
            CU(sf_launch_trace(s->graph->prog.form, s->graph->d_prog, s->d_scene, s->soa, tl, c->d_stats, blocks,
                               int(s->min_blocks), s->light_smem, st));
        }
        LaunchTimer t(c, false);
        CU(sf_launch_shade(s->d_scene, rich, s->soa, q, g, s->film, s->status, r + 1 == R ? 1 : 0, st));
    }
    LaunchTimer t(c, false);
    CU(sf_launch_commit(s->soa, g, s->film, st));
    s->dispatches++;
    return SF_OK;
}

extern "C" sf_status sf_session_sync(sf_session* s, uint32_t timeout_ms, uint32_t* status_word) {
    if (!s) return fail(SF_ERR_INVALID, "null session");
    sf_context* c = s->ctx;
    cudaSetDevice(c->device);
    sf_status st = wait_stream(c->stream, timeout_ms);
    if (st != SF_OK) return st;
    uint32_t w = 0;
    CU(cudaMemcpy(&w, s->status, 4, cudaMemcpyDeviceToHost));
    s->status_host |= w;
    if (status_word) *status_word = s->status_host;
    if (s->status_host) return fail(SF_ERR_WAVEFRONT, "wavefront invariant word " + std::to_string(s->status_host));
    return SF_OK;
}

extern "C" sf_status sf_session_step(sf_session* s, uint32_t budget_ms, int* done) {
    if (!s) return fail(SF_ERR_INVALID, "null session");
    auto t0 = std::chrono::steady_clock::now();
    const uint32_t target = s->cfg.samples_per_pixel;
    // Dispatches are queued on the session stream without waiting for each one; the
    // host waits when the queued work is predicted to reach the budget (from the
    // measured cost of earlier dispatches), then checks the budget on the wall clock.
    double queued_ms = 0.0;
    for (;;) {
        // TileGrid::next_pending (tiles.rs:52-59): least-advanced tile below target, lowest index.
        int best = -1;
        for (size_t i = 0; i < s->tiles.size(); ++i)
            if (s->tiles[i].done < target && (best < 0 || s->tiles[i].done < s->tiles[best].done)) best = int(i);
        if (best < 0) break;
        sf_tile& t = s->tiles[best];
        uint32_t n = std::min(s->cfg.samples_per_dispatch, target - t.done);
        sf_status st = sf_session_dispatch(s, t, n);
        if (st != SF_OK) return st;
        t.done += n;
        double per_path_ms = s->ms_per_path > 0 ? s->ms_per_path : 0.0;
        queued_ms += per_path_ms * double(t.w) * t.h * n;
        double el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (per_path_ms == 0.0 || !budget_ms || el + queued_ms >= budget_ms) {
            auto w0 = std::chrono::steady_clock::now();
            st = sf_session_sync(s, 10000, nullptr);  // DISPATCH_TIMEOUT, renderer.rs:236
            if (st != SF_OK) return st;
            double waited = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
            if (per_path_ms == 0.0) s->ms_per_path = (waited + 1e-3) / (double(t.w) * t.h * n);
            queued_ms = 0.0;
            el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (budget_ms && el >= budget_ms) break;
        }
    }
    sf_status st = sf_session_sync(s, 10000, nullptr);
    if (st != SF_OK) return st;
    bool complete = true;
    for (auto& t : s->tiles)
        if (t.done < target) complete = false;
    if (done) *done = complete ? 1 : 0;
    return SF_OK;
}

extern "C" sf_status sf_session_progress(sf_session* s, sf_progress* out) {
    if (!s || !out) return fail(SF_ERR_INVALID, "null argument");
    std::memset(out, 0, sizeof *out);
    out->tiles = uint32_t(s->tiles.size());
    out->dispatches = s->dispatches;
    out->target = s->cfg.samples_per_pixel;
    uint32_t mn = 0xffffffffu, mx = 0;
    for (auto& t : s->tiles) {
        mn = std::min(mn, t.done);
        mx = std::max(mx, t.done);
        out->pixel_samples_done += uint64_t(t.w) * t.h * t.done;
    }
    out->samples_min = s->tiles.empty() ? 0 : mn;
    out->samples_max = mx;
    out->pixel_samples_total = uint64_t(s->cfg.width) * s->cfg.height * s->cfg.samples_per_pixel;
    out->status_word = s->status_host;
    return SF_OK;
}

extern "C" sf_status sf_session_tiles(sf_session* s, sf_tile* tiles, uint32_t capacity, uint32_t* count) {
    if (!s || !count) return fail(SF_ERR_INVALID, "null argument");
    *count = uint32_t(s->tiles.size());
    if (tiles)
        for (uint32_t i = 0; i < std::min<uint32_t>(capacity, *count); ++i) tiles[i] = s->tiles[i];
    return SF_OK;
}

namespace sfh {
// Film readback through the context's pinned staging: the device planes arrive at
// full link speed, then the host threads copy them into the caller's (pageable)
// buffers and derive color = accum.rgb / max(count, 1) with alpha 1
// (RenderOutput.color). A film without the volume layer split (no fog) has a zero
// volume contribution: volume and moments are (0, 0, 0, samples) and surface = accum.
cudaError_t film_readback(sf_context* c, const FilmPlanes& f, const sf_film_planes& out, cudaStream_t st) {
    const size_t px = size_t(f.width) * f.height;
    const bool split = f.vol != nullptr;
    const bool need_acc = out.accum || out.color || (!split && (out.volume || out.moments || out.surface));
    const bool need_vol = split && (out.volume || out.moments || out.surface);
    const size_t bytes = (need_acc ? px * 16 : 0) + (out.depth ? px * 4 : 0) + (out.aux ? px * 16 : 0) +
                         (need_vol ? px * 48 : 0);
    if (!bytes) return cudaSuccess;
    std::lock_guard<std::mutex> lk(c->stage_mu);
    if (cudaError_t e = ensure_stage(c, bytes); e != cudaSuccess) return e;
    float* acc = static_cast<float*>(c->stage);
    float* depth = acc + (need_acc ? px * 4 : 0);
    float* aux = depth + (out.depth ? px : 0);
    float* vol = aux + (out.aux ? px * 4 : 0);  // volume | moments | surface (contiguous on the device)
    cudaError_t e = cudaSuccess;
    if (need_acc) e = cudaMemcpyAsync(acc, f.accum, px * 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && out.depth) e = cudaMemcpyAsync(depth, f.depth, px * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && out.aux) e = cudaMemcpyAsync(aux, f.aux, px * 16, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && need_vol) e = cudaMemcpyAsync(vol, f.vol, px * 48, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    host_parallel(px, [&](size_t b, size_t end) {
        const size_t n = end - b;
        if (out.accum) std::memcpy(out.accum + 4 * b, acc + 4 * b, n * 16);
        if (out.depth) std::memcpy(out.depth + b, depth + b, n * 4);
        if (out.aux) std::memcpy(out.aux + 4 * b, aux + 4 * b, n * 16);
        if (split) {
            if (out.volume) std::memcpy(out.volume + 4 * b, vol + 4 * b, n * 16);
            if (out.moments) std::memcpy(out.moments + 4 * b, vol + 4 * (px + b), n * 16);
            if (out.surface) std::memcpy(out.surface + 4 * b, vol + 4 * (2 * px + b), n * 16);
        } else if (out.surface) {
            std::memcpy(out.surface + 4 * b, acc + 4 * b, n * 16);
        }
        for (size_t i = b; i < end; ++i) {
            const float cnt = acc[4 * i + 3];
            if (out.color) {
                const float d = std::max(cnt, 1.0f);
                out.color[4 * i] = acc[4 * i] / d;
                out.color[4 * i + 1] = acc[4 * i + 1] / d;
                out.color[4 * i + 2] = acc[4 * i + 2] / d;
                out.color[4 * i + 3] = 1.0f;
            }
            if (split) continue;
            if (out.volume) { out.volume[4 * i] = out.volume[4 * i + 1] = out.volume[4 * i + 2] = 0.0f; out.volume[4 * i + 3] = cnt; }
            if (out.moments) { out.moments[4 * i] = out.moments[4 * i + 1] = out.moments[4 * i + 2] = 0.0f; out.moments[4 * i + 3] = cnt; }
        }
    });
    return cudaSuccess;
}
}  // namespace sfh

extern "C" sf_status sf_session_readback(sf_session* s, sf_film_planes* out) {
    if (!s || !out) return fail(SF_ERR_INVALID, "null argument");
    sf_context* c = s->ctx;
    cudaSetDevice(c->device);
    CU(film_readback(c, s->film, *out, c->stream));
    return SF_OK;
}

extern "C" sf_status sf_session_stats(sf_session* s, sf_stats* out) {
    if (!s) return fail(SF_ERR_INVALID, "null session");
    return sf_context_stats(s->ctx, out);
}

extern "C" sf_status sf_session_destroy(sf_session* s) {
    if (!s) return SF_OK;
    sf_context* c = s->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    ctx_free_cached(c, s->mem, s->mem_bytes);  // idle now: kept for the next session of its size
    sf_graph* g = s->graph;
    delete s;
    sf_graph_destroy(g);  // drops the session's reference
    ctx_release(c);
    return SF_OK;
}

// ------------------------------------------------------------------ checkpoints
namespace sfh {

uint64_t fnv1a(const void* data, size_t n, uint64_t h) {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}


const uint32_t CK_MAGIC = 0x4b434653u;  // "SFCK"
const uint32_t CK_VERSION = 4;  // 3: the scene carries its fog; 4: the config its hit epsilon

std::string producer_of(const sf_context* c) {
    return c->device_name + "|sm_" + std::to_string(c->cc_major) + std::to_string(c->cc_minor) + "|abi " +
           std::to_string(ABI_VERSION);
}

bool write_file(const std::string& path, const std::vector<uint8_t>& data) {
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) return false;
    f.write(reinterpret_cast<const char*>(data.data()), std::streamsize(data.size()));
    return bool(f);
}
bool read_file(const std::string& path, std::vector<uint8_t>& data) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    f.seekg(0, std::ios::end);
    std::streamoff n = f.tellg();
    if (n < 0) return false;
    f.seekg(0);
    data.resize(size_t(n));
    f.read(reinterpret_cast<char*>(data.data()), n);
    return bool(f) || f.eof();
}
void remove_tree(const std::string& dir) {
    for (const char* name : {"state.bin", "film.bin", "export.bin"}) unlink((dir + "/" + name).c_str());
    rmdir(dir.c_str());
}
// Writes the files into a sibling directory, then swaps it into place (session.rs:33-45).
sf_status install_checkpoint(const std::string& final_dir,
                             const std::vector<std::pair<std::string, const std::vector<uint8_t>*>>& files) {
    std::string tmp = final_dir + ".tmp-" + std::to_string(getpid()), old = final_dir + ".old";
    remove_tree(tmp);
    if (mkdir(tmp.c_str(), 0755) != 0) return fail(SF_ERR_IO, "cannot create " + tmp);
    for (auto& f : files)
        if (!write_file(tmp + "/" + f.first, *f.second)) {
            remove_tree(tmp);
            return fail(SF_ERR_IO, "cannot write checkpoint files");
        }
    struct stat st;
    bool existed = stat(final_dir.c_str(), &st) == 0;
    if (existed) {
        remove_tree(old);
        if (rename(final_dir.c_str(), old.c_str()) != 0) { remove_tree(tmp); return fail(SF_ERR_IO, "cannot move old checkpoint"); }
    }
    if (rename(tmp.c_str(), final_dir.c_str()) != 0) return fail(SF_ERR_IO, "cannot install checkpoint");
    if (existed) remove_tree(old);
    return SF_OK;
}

}  // namespace sfh

namespace sfh {
bool has_hdri(const sf_scene_desc& d) {
    for (uint32_t i = 0; i < scene_light_count(d); ++i)
        if (scene_lights(d)[i].kind == SF_LIGHT_HDRI) return true;
    return false;
}
}  // namespace sfh

extern "C" sf_status sf_session_save(sf_session* s, const char* dir) {
    if (!s || !dir || !*dir) return fail(SF_ERR_INVALID, "null argument");
    if (has_hdri(s->scene)) return fail(SF_ERR_UNSUPPORTED, "scenes with an HDRI panorama are not checkpointed");
    if (s->scene.texture.graph)  // the texture's graph is a caller object, like a panorama
        return fail(SF_ERR_UNSUPPORTED, "textured scenes are not checkpointed");
    sf_context* c = s->ctx;
    cudaSetDevice(c->device);
    CU(cudaStreamSynchronize(c->stream));
    size_t px = size_t(s->cfg.width) * s->cfg.height;
    Writer film;
    // accum | depth | aux (| volume | moments | surface for fog scenes)
    film.buf.resize(px * (s->film.vol ? 84 : 36));
    CU(cudaMemcpy(film.buf.data(), s->film.accum, px * 16, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(film.buf.data() + px * 16, s->film.depth, px * 4, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(film.buf.data() + px * 20, s->film.aux, px * 16, cudaMemcpyDeviceToHost));
    if (s->film.vol) CU(cudaMemcpy(film.buf.data() + px * 36, s->film.vol, px * 48, cudaMemcpyDeviceToHost));
    Writer w;
    w.put(CK_MAGIC);
    w.put(CK_VERSION);
    w.put_str(producer_of(c));
    w.put(s->cfg);
    w.put(s->scene);
    w.put_str(s->graph->topology);
    w.put(uint32_t(s->graph->host.nodes.size()));
    w.put_bytes(s->graph->host.nodes.data(), s->graph->host.nodes.size() * sizeof(sf_node));
    w.put(fnv1a(s->graph->host.placements.data(), s->graph->host.placements.size() * sizeof(sf_placement)));
    w.put(s->dispatches);
    w.put(s->tile_size);
    w.put(uint32_t(s->tiles.size()));
    for (auto& t : s->tiles) w.put(t);
    w.put(uint64_t(film.buf.size()));
    w.put(fnv1a(film.buf.data(), film.buf.size()));
    uint64_t h = fnv1a(w.buf.data(), w.buf.size());
    w.put(h);
    return install_checkpoint(dir, {{"film.bin", &film.buf}, {"state.bin", &w.buf}});
}

extern "C" sf_status sf_session_resume(sf_context* c, sf_graph* g, const char* dir, sf_session** out) {
    if (!c || !g || !dir || !out) return fail(SF_ERR_INVALID, "null argument");
    *out = nullptr;
    std::string d(dir);
    std::vector<uint8_t> state, filmb;
    if (!read_file(d + "/state.bin", state) || !read_file(d + "/film.bin", filmb))
        return fail(SF_ERR_IO, "cannot read checkpoint in " + d);
    if (state.size() < 16) return fail(SF_ERR_CHECKPOINT, "checkpoint state truncated");
    uint64_t stored;
    std::memcpy(&stored, state.data() + state.size() - 8, 8);
    if (fnv1a(state.data(), state.size() - 8) != stored) return fail(SF_ERR_CHECKPOINT, "checkpoint state hash mismatch");
    Reader r{state};
    if (r.get<uint32_t>() != CK_MAGIC || r.get<uint32_t>() != CK_VERSION)
        return fail(SF_ERR_CHECKPOINT, "not a checkpoint of this version");
    std::string producer = r.get_str();
    if (producer != producer_of(c))
        return fail(SF_ERR_CHECKPOINT, "checkpoint from another producer: " + producer);
    sf_render_config cfg = r.get<sf_render_config>();
    sf_scene_desc scene = r.get<sf_scene_desc>();
    std::string topo = r.get_str();
    uint32_t nn = r.get<uint32_t>();
    // bounded before anything is sized from it: the hash does not authenticate the file
    if (!r.ok || nn > 4096) return fail(SF_ERR_CHECKPOINT, "checkpoint graph too large or truncated");
    std::vector<sf_node> nodes(nn);
    r.get_bytes(nodes.data(), nn * sizeof(sf_node));
    const uint64_t placements_hash = r.get<uint64_t>();
    uint32_t dispatches = r.get<uint32_t>();
    uint32_t tile_size = r.get<uint32_t>();
    uint32_t nt = r.get<uint32_t>();
    if (!r.ok || nt > (1u << 24)) return fail(SF_ERR_CHECKPOINT, "checkpoint state truncated");
    std::vector<sf_tile> tiles(nt);
    for (auto& t : tiles) t = r.get<sf_tile>();
    uint64_t film_bytes = r.get<uint64_t>();
    uint64_t film_hash = r.get<uint64_t>();
    if (!r.ok) return fail(SF_ERR_CHECKPOINT, "checkpoint state truncated");
    if (film_bytes != filmb.size() || fnv1a(filmb.data(), filmb.size()) != film_hash)
        return fail(SF_ERR_CHECKPOINT, "checkpoint film hash mismatch");
    if (topo != g->topology || nn != g->host.nodes.size() ||
        std::memcmp(nodes.data(), g->host.nodes.data(), nn * sizeof(sf_node)) != 0 ||
        placements_hash != fnv1a(g->host.placements.data(), g->host.placements.size() * sizeof(sf_placement)))
        return fail(SF_ERR_CHECKPOINT, "checkpoint was made with another graph");
    size_t px = size_t(cfg.width) * cfg.height;
    if (filmb.size() != px * (has_fog(scene) ? 84 : 36)) return fail(SF_ERR_CHECKPOINT, "checkpoint film size mismatch");
    sf_session* s = nullptr;
    sf_status st = sf_session_create(c, g, &scene, &cfg, &s);
    if (st != SF_OK) return st;
    if (s->tile_size != tile_size || s->tiles.size() != tiles.size()) {
        sf_session_destroy(s);
        return fail(SF_ERR_CHECKPOINT, "checkpoint tile layout mismatch");
    }
    for (size_t i = 0; i < tiles.size(); ++i) {
        const sf_tile& a = tiles[i];
        const sf_tile& b = s->tiles[i];
        if (a.x != b.x || a.y != b.y || a.w != b.w || a.h != b.h || a.done > cfg.samples_per_pixel) {
            sf_session_destroy(s);
            return fail(SF_ERR_CHECKPOINT, "checkpoint tile layout mismatch");
        }
    }
    s->tiles = tiles;
    s->dispatches = dispatches;
    cudaError_t e = cudaMemcpy(s->film.accum, filmb.data(), px * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->film.depth, filmb.data() + px * 16, px * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->film.aux, filmb.data() + px * 20, px * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && s->film.vol)
        e = cudaMemcpy(s->film.vol, filmb.data() + px * 36, px * 48, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        sf_session_destroy(s);
        return cuda_fail(e, "checkpoint upload");
    }
    *out = s;
    return SF_OK;
}

// ------------------------------------------------------------------ escape time
namespace sfh {
void planar_dev(const sf_planar_desc& f, PlanarDev& o) {
    std::memset(&o, 0, sizeof o);
    o.family = f.family;
    o.power = f.power;
    o.iterations = f.iterations;
    o.julia[0] = f.julia[0];
    o.julia[1] = f.julia[1];
    o.center[0] = f.center[0];
    o.center[1] = f.center[1];
    o.zoom = f.zoom;
    o.inversion = f.inversion;
    o.relaxation = f.relaxation;
    o.memory = f.memory;
    o.bailout = f.bailout;
    o.trap_radius = f.trap_radius;
    o.stripes = f.stripes;
    // f32::to_radians then sin_cos, evaluated on the host in binary32 (planar.rs:79-80, :97)
    const float k = 3.14159265358979323846f / 180.0f;
    float a = f.angle * k, t = f.twist * k;
    o.angle_sin = sinf(a);
    o.angle_cos = cosf(a);
    o.twist_sin = sinf(t);
    o.twist_cos = cosf(t);
    o.bail_t = sqrt_threshold(f.bailout);
    o.stripe_k = f.stripes == std::floor(f.stripes) && std::fabs(f.stripes) <= 64.0f ? int32_t(f.stripes)
                                                                                      : SF_STRIPES_GENERAL;
}
sf_status planar_check(const sf_planar_desc* f) {
    if (!f) return fail(SF_ERR_INVALID, "null planar descriptor");
    if (f->family > 5) return fail(SF_ERR_INVALID, "unknown planar family");
    if (f->power < 1 || f->power > 8) return fail(SF_ERR_INVALID, "power must be between 1 and 8");
    if (!(f->zoom != 0.0f)) return fail(SF_ERR_INVALID, "zoom must be non-zero");
    return SF_OK;
}
}  // namespace sfh

extern "C" sf_status sf_planar_probe(sf_context* c, const sf_planar_desc* f, const float* xy, size_t n, float* dist,
                                     float* traps, uint32_t* iters) {
    if (!c) return fail(SF_ERR_INVALID, "null context");
    sf_status st = planar_check(f);
    if (st != SF_OK) return st;
    if (n == 0) return SF_OK;
    if (!xy || !dist || !traps || !iters) return fail(SF_ERR_INVALID, "null buffer");
    cudaSetDevice(c->device);
    PlanarDev F;
    planar_dev(*f, F);
    std::vector<float> soa(2 * n);
    for (size_t i = 0; i < n; ++i) { soa[i] = xy[2 * i]; soa[n + i] = xy[2 * i + 1]; }
    size_t bytes = 256 + n * 4 * (2 + 1 + 4 + 1);
    void* buf = nullptr;
    st = ctx_alloc(c, bytes, &buf);
    if (st != SF_OK) return st;
    PlanarDev* dF = static_cast<PlanarDev*>(buf);
    float* din = reinterpret_cast<float*>(static_cast<char*>(buf) + 256);
    float* dd = din + 2 * n;
    float* dt = dd + n;
    uint32_t* di = reinterpret_cast<uint32_t*>(dt + 4 * n);
    cudaError_t e = cudaMemcpyAsync(dF, &F, sizeof F, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(din, soa.data(), 2 * n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        LaunchTimer t(c, true);
        e = sf_launch_planar(dF, din, din + n, n, dd, dt, di, c->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(dist, dd, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(traps, dt, 4 * n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(iters, di, n * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, buf, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "sf_planar_probe");
    return SF_OK;
}

extern "C" sf_status sf_escape2d(sf_context* c, const sf_planar_desc* f, const sf_canvas* canvas, sf_tile tile,
                                 uint32_t sample, float* dist, float* traps, uint32_t* iters) {
    if (!c || !canvas) return fail(SF_ERR_INVALID, "null argument");
    sf_status st = planar_check(f);
    if (st != SF_OK) return st;
    if (!canvas->width || !canvas->height || tile.x + tile.w > canvas->width || tile.y + tile.h > canvas->height)
        return fail(SF_ERR_INVALID, "tile outside the canvas");
    size_t n = size_t(tile.w) * tile.h;
    if (n == 0) return SF_OK;
    if (!dist || !traps || !iters) return fail(SF_ERR_INVALID, "null buffer");
    cudaSetDevice(c->device);
    PlanarDev F;
    planar_dev(*f, F);
    CanvasDev K;
    std::memset(&K, 0, sizeof K);
    K.center[0] = canvas->center[0];
    K.center[1] = canvas->center[1];
    K.zoom = canvas->zoom;
    K.aspect = float(canvas->width) / float(canvas->height);
    float r = canvas->rotation_deg * (3.14159265358979323846f / 180.0f);
    K.rot_sin = sinf(r);
    K.rot_cos = cosf(r);
    K.width = canvas->width;
    K.height = canvas->height;
    K.seed = uint32_t(canvas->seed) ^ uint32_t(canvas->seed >> 32);
    size_t bytes = 768 + n * 4 * 6;  // descriptors | pixel counter | outputs
    // the context's device scratch and pinned staging, kept between calls
    std::unique_lock<std::mutex> lk(c->stage_mu);
    st = ensure_scratch(c, bytes);
    if (st != SF_OK) return st;
    void* buf = c->scratch;
    PlanarDev* dF = static_cast<PlanarDev*>(buf);
    CanvasDev* dK = reinterpret_cast<CanvasDev*>(static_cast<char*>(buf) + 256);
    uint32_t* dW = reinterpret_cast<uint32_t*>(static_cast<char*>(buf) + 512);
    float* dd = reinterpret_cast<float*>(static_cast<char*>(buf) + 768);
    float* dt = dd + n;
    uint32_t* di = reinterpret_cast<uint32_t*>(dt + 4 * n);
    cudaError_t e = cudaMemcpyAsync(dF, &F, sizeof F, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dK, &K, sizeof K, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(dW, 0, 4, c->stream);
    if (e == cudaSuccess) {
        LaunchTimer t(c, true);
        e = sf_launch_escape2d(dF, dK, tile.x, tile.y, tile.w, tile.h, sample, dd, dt, di, c->d_stats, dW, 1,
                               F.family == 3 || F.family == 4, c->stream);
    }
    // distance, traps and iterations are contiguous: one copy into the pinned staging,
    // then host threads split it into the caller's arrays
    if (e == cudaSuccess) e = ensure_stage(c, n * 24);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->stage, dd, n * 24, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "sf_escape2d");
    const char* stg = static_cast<const char*>(c->stage);
    host_parallel(n, [&](size_t b0, size_t b1) {
        std::memcpy(dist + b0, stg + b0 * 4, (b1 - b0) * 4);
        for (int k = 0; k < 4; ++k)  // traps are four planes of n
            std::memcpy(traps + k * n + b0, stg + (n + k * n + b0) * 4, (b1 - b0) * 4);
        std::memcpy(iters + b0, stg + (5 * n + b0) * 4, (b1 - b0) * 4);
    });
    return SF_OK;
}

// The reference orbit Z_n of c_ref in FP64 on the host, as the device writes it
// (hi = float(Z), lo = float(Z - hi), two copies of the last entry past the end) and
// with the same operations: |Z|^2 = fma(x, x, y*y); Re Z' = fma(x, x, -y*y) + Re c;
// Im Z' = fma(x + x, y, Im c) (this file is compiled without contraction, so the
// explicit fma calls are the only fused operations), so the two orbits are equal.
// One host core runs the sequential recurrence in well under a millisecond per 10^5
// iterations. Returns the length.
static uint32_t host_ref_orbit(double cx, double cy, uint32_t max_iter, double bailout, float* lo, float* hi) {
    double zx = 0.0, zy = 0.0;
    const double b2 = bailout * bailout;
    uint32_t n = 0;
    for (;;) {
        const float hx = float(zx), hy = float(zy);
        hi[2 * n] = hx;
        hi[2 * n + 1] = hy;
        lo[2 * n] = float(zx - double(hx));
        lo[2 * n + 1] = float(zy - double(hy));
        const double y2 = zy * zy;
        if (n >= max_iter || std::fma(zx, zx, y2) > b2) break;
        const double nx = std::fma(zx, zx, -y2) + cx;
        zy = std::fma(zx + zx, zy, cy);
        zx = nx;
        ++n;
    }
    for (uint32_t k = 1; k <= 2; ++k)
        for (int j = 0; j < 2; ++j) {
            hi[2 * (n + k) + j] = hi[2 * n + j];
            lo[2 * (n + k) + j] = lo[2 * n + j];
        }
    return n + 1;
}

extern "C" sf_status sf_deep_zoom(sf_context* c, const sf_deep_zoom_desc* d, uint32_t* iters, float* smooth,
                                  int reference_f64, uint32_t* iters64, float* smooth64, uint64_t* rebases) {
    if (!c || !d) return fail(SF_ERR_INVALID, "null argument");
    if (!d->width || !d->height || !d->max_iter) return fail(SF_ERR_INVALID, "empty deep-zoom request");
    if (!iters || !smooth) return fail(SF_ERR_INVALID, "null output");
    if (reference_f64 && (!iters64 || !smooth64)) return fail(SF_ERR_INVALID, "null FP64 output");
    if (!(d->bailout >= 2.0f)) return fail(SF_ERR_INVALID, "bailout must be at least 2");
    // the perturbation kernel indexes pixels with 32-bit counters
    if (uint64_t(d->width) * d->height > (1ull << 31)) return fail(SF_ERR_INVALID, "deep-zoom frames hold at most 2^31 pixels");
    if (d->orbit_mode > SF_ORBIT_GIVEN) return fail(SF_ERR_INVALID, "unknown orbit_mode");
    if (d->orbit_mode == SF_ORBIT_GIVEN && (!d->orbit || d->orbit_len < 1 || d->orbit_len > uint64_t(d->max_iter) + 1))
        return fail(SF_ERR_INVALID, "a given orbit needs 1 to max_iter + 1 entries");
    cudaSetDevice(c->device);
    size_t n = size_t(d->width) * d->height;
    size_t M = size_t(d->max_iter) + 4;  // the orbit, two entries past its end, one spare
    const size_t Mb = (M * 8 + 255) & ~size_t(255);
    // the device orbit's FP64 values (split into hi/lo pairs by a parallel kernel)
    const size_t Zb = d->orbit_mode == SF_ORBIT_DEVICE ? ((M * 16 + 255) & ~size_t(255)) : 0;
    const size_t z_off = (2 * Mb + 256 + n * 8 * (reference_f64 ? 2 : 1) + 255) & ~size_t(255);
    size_t bytes = z_off + Zb;
    void* buf = nullptr;
    sf_status st = ctx_alloc(c, bytes, &buf);
    if (st != SF_OK) return st;
    char* b = static_cast<char*>(buf);
    float2* olo = reinterpret_cast<float2*>(b);
    float2* of = reinterpret_cast<float2*>(b + Mb);
    uint32_t* olen = reinterpret_cast<uint32_t*>(b + 2 * Mb);  // orbit length | pixel counter
    uint32_t* work = olen + 1;
    uint32_t* di = reinterpret_cast<uint32_t*>(b + 2 * Mb + 256);
    float* ds = reinterpret_cast<float*>(di + n);
    uint32_t* di64 = reinterpret_cast<uint32_t*>(ds + n);
    float* ds64 = reinterpret_cast<float*>(di64 + n);
    double2* oz = Zb ? reinterpret_cast<double2*>(b + z_off) : nullptr;  // 256-byte aligned
    // the orbit of c_ref = centre hi; the centre's lo part joins every pixel's offset
    const double cx = d->center_hi[0], cy = d->center_hi[1];
    const float2 c_lo = make_float2(float(d->center_lo[0]), float(d->center_lo[1]));
    double pitch = d->width_units / double(d->width);
    cudaError_t e = cudaSuccess;
    unsigned long long before[SF_STAT_COUNT];
    e = cudaMemcpyAsync(before, c->d_stats, sizeof before, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(work, 0, 4, c->stream);
    const size_t planes = reference_f64 ? 4 : 2;
    std::unique_lock<std::mutex> lk(c->stage_mu);
    if (e == cudaSuccess) e = ensure_stage(c, std::max(2 * Mb + 16, n * 4 * planes));
    if (e == cudaSuccess && d->orbit_mode == SF_ORBIT_DEVICE) {
        LaunchTimer t(c, false);
        e = sf_launch_ref_orbit_split(cx, cy, d->max_iter, d->bailout, oz, olo, of, olen, c->stream);
    } else if (e == cudaSuccess) {
        // the host's orbit, or the caller's, uploaded from the pinned staging (lo, hi, then its length)
        char* stg = static_cast<char*>(c->stage);
        float* lo = reinterpret_cast<float*>(stg);
        float* hi = reinterpret_cast<float*>(stg + Mb);
        uint32_t len = 0;
        if (d->orbit_mode == SF_ORBIT_HOST) {
            len = host_ref_orbit(cx, cy, d->max_iter, double(d->bailout), lo, hi);
        } else {
            len = d->orbit_len;
            for (uint32_t k = 0; k < len + 2; ++k) {  // two copies of the last entry past the end
                const float* z = d->orbit + 4 * size_t(std::min(k, len - 1));
                hi[2 * k] = z[0];
                hi[2 * k + 1] = z[1];
                lo[2 * k] = z[2];
                lo[2 * k + 1] = z[3];
            }
        }
        std::memcpy(stg + 2 * Mb, &len, 4);
        e = cudaMemcpyAsync(olo, stg, 2 * Mb + 4, cudaMemcpyHostToDevice, c->stream);
    }
    if (e == cudaSuccess) {
        LaunchTimer t(c, true);
        e = sf_launch_perturb(olo, of, olen, d->width, d->height, float(pitch), c_lo, d->max_iter, d->bailout, di, ds,
                              c->d_stats, work, c->stream);
    }
    if (e == cudaSuccess && reference_f64) {
        LaunchTimer t(c, false);
        e = sf_launch_direct_f64(cx, cy, d->center_lo[0], d->center_lo[1], d->width, d->height, pitch, d->max_iter,
                                 d->bailout, di64, ds64, c->stream);
    }
    // the output planes are contiguous from di: one copy into the pinned staging (after
    // the orbit's upload from it, in stream order), then host threads split it into the
    // caller's arrays
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->stage, di, n * 4 * planes, cudaMemcpyDeviceToHost, c->stream);
    unsigned long long after[SF_STAT_COUNT];
    if (e == cudaSuccess) e = cudaMemcpyAsync(after, c->d_stats, sizeof after, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, buf, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "sf_deep_zoom");
    {
        const char* stg = static_cast<const char*>(c->stage);
        void* outs[4] = {iters, smooth, iters64, smooth64};
        host_parallel(n, [&](size_t b0, size_t b1) {
            for (size_t k = 0; k < planes; ++k)
                std::memcpy(static_cast<char*>(outs[k]) + b0 * 4, stg + k * n * 4 + b0 * 4, (b1 - b0) * 4);
        });
    }
    lk.unlock();
    if (rebases) *rebases = after[SF_STAT_STEPS] - before[SF_STAT_STEPS];
    return SF_OK;
}

// ------------------------------------------------------------------ FP32 peak
extern "C" sf_status sf_device_fp32_peak(sf_context* c, double* tflops) {
    if (!c || !tflops) return fail(SF_ERR_INVALID, "null argument");
    cudaSetDevice(c->device);
    void* buf = nullptr;
    sf_status s = ctx_alloc(c, 256, &buf);
    if (s != SF_OK) return s;
    const int blocks = c->sm_count * 8;
    const uint32_t iters = 4096;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    // warm-up: three full-length launches bring the clocks and power state to where the
    // timed launches will run
    cudaError_t e = cudaSuccess;
    for (int w = 0; w < 3 && e == cudaSuccess; ++w) e = sf_launch_ffma_peak(static_cast<float*>(buf), iters, blocks, c->stream);
    // the median of 7 timed launches: a single fastest run can land on a clock excursion
    std::vector<float> times;
    for (int rep = 0; rep < 7 && e == cudaSuccess; ++rep) {
        cudaEventRecord(a, c->stream);
        e = sf_launch_ffma_peak(static_cast<float*>(buf), iters, blocks, c->stream);
        cudaEventRecord(b, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
        if (ms > 0) times.push_back(ms);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx_free(c, buf, 256);
    if (e != cudaSuccess) return cuda_fail(e, "fp32 peak probe");
    if (times.empty()) return fail(SF_ERR_CUDA, "fp32 peak probe: no timing");
    std::sort(times.begin(), times.end());
    const float median = times[times.size() / 2];
    double flops = double(blocks) * 256.0 * iters * 16.0 * 8.0 * 2.0;
    *tflops = flops / (median * 1e-3) / 1e12;
    return SF_OK;
}

