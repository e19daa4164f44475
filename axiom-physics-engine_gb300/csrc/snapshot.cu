// snapshot.cu — world checkpoint / resume and the headless debug feed.
//
// Snapshot: every body is packed on the device into its axiom_snapshot_body record and
// the previous-step warm-start table is compacted into axiom_snapshot_contact entries,
// then both come back in two copies; the host sorts the entries by key so the bytes do
// not depend on hash-table slot order.  Loading rebuilds the packed body layout from the
// records (inverse masses and inertias are taken as stored, not recomputed from mass, so
// the resumed step is bit-identical) and reinserts the entries into the table the next
// step's warm start reads.
//
// Debug feed: the records of debug::PhysicsDebugDraw (DebugRigidBody, DebugShape,
// DebugContactPoint; include/axiom/debug/physics_debug_draw.hpp:97-132), packed on the
// device and copied out in one piece per array.  The reference draws them with Vulkan;
// here they go to host memory for a recorder or remote viewer.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "body_pack.h"
#include "solver_math.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

#define AX_CUDA(call)                                             \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED;  \
    } while (0)

constexpr char kMagic[8] = {'A', 'X', 'S', 'N', 'A', 'P', '0', '1'};

__global__ void __launch_bounds__(256) kSnapBodies(uint32_t n, const uint32_t* __restrict__ info,
                                                   const float4* __restrict__ pos, const float4* __restrict__ rot,
                                                   const SolverBody* __restrict__ sb, const float4* __restrict__ shp,
                                                   const float4* __restrict__ mat, const float4* __restrict__ iloc,
                                                   const uint4* __restrict__ filt,
                                                   const float* __restrict__ sleepTime,
                                                   const uint32_t* __restrict__ island,
                                                   axiom_snapshot_body* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t inf = info[i];
    const uint32_t t = inf & kInfoTypeMask;
    const float4 p = pos[i], q = rot[i], e = shp[i], m = mat[i], ii = iloc[i];
    const SolverBody b = sb[i];
    const uint4 f = filt[i];
    axiom_snapshot_body r;
    r.type = t == kTypeSleeping ? (uint32_t)AXIOM_BODY_DYNAMIC : t;
    r.shape = (inf >> 4) & 0xFu;
    r.flags = (t == kTypeSleeping ? 1u : 0u) | ((inf & kInfoNoSleep) ? 2u : 0u);
    const bool dyn = t == AXIOM_BODY_DYNAMIC || t == kTypeSleeping;
    r.island = island && dyn ? island[i] : kNoIsland;
    r.position[0] = p.x, r.position[1] = p.y, r.position[2] = p.z;
    r.rotation[0] = q.x, r.rotation[1] = q.y, r.rotation[2] = q.z, r.rotation[3] = q.w;
    r.linear_velocity[0] = b.v.x, r.linear_velocity[1] = b.v.y, r.linear_velocity[2] = b.v.z;
    r.angular_velocity[0] = b.w.x, r.angular_velocity[1] = b.w.y, r.angular_velocity[2] = b.w.z;
    r.shape_extents[0] = e.x, r.shape_extents[1] = e.y, r.shape_extents[2] = e.z;
    r.inv_mass = b.v.w;
    r.inv_inertia[0] = ii.x, r.inv_inertia[1] = ii.y, r.inv_inertia[2] = ii.z;
    r.friction = m.x, r.restitution = m.y, r.linear_damping = m.z, r.angular_damping = m.w;
    r.filter_category = f.x, r.filter_mask = f.y, r.filter_group = (int32_t)f.z;
    r.sleep_time = sleepTime && dyn ? sleepTime[i] : 0.0f;
    r.rolling_friction = ii.w;
    r.reserved[0] = r.reserved[1] = r.reserved[2] = 0u;
    out[i] = r;
}

// Non-empty slots of a warm-start table -> (lo, hi, point, impulse) entries, unordered.
__global__ void __launch_bounds__(256) kSnapWarm(uint32_t slots, const WarmSlot* __restrict__ table, uint32_t gen,
                                                 axiom_snapshot_contact* __restrict__ out, uint32_t cap,
                                                 uint32_t* counter) {
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= slots) return;
    const WarmSlot sl = table[h];
    if (sl.gen != gen) return;
    const unsigned long long key = sl.key;
    const uint32_t idx = atomicAdd(counter, 1u);
    if (idx >= cap) return;
    const float4 v = sl.val;
    axiom_snapshot_contact c;
    c.body_lo = (uint32_t)(key >> 34);  // key = ((lo << 32) | hi) * 4 + point
    c.body_hi = (uint32_t)((key >> 2) & 0xFFFFFFFFull);
    c.point = (uint32_t)(key & 3ull) | ((sl.tag & 0xFFu) << 8);  // tag: 1 + colour on point 0
    c.impulse[0] = v.x, c.impulse[1] = v.y, c.impulse[2] = v.z;
    out[idx] = c;
}

__global__ void __launch_bounds__(256) kLoadWarm(uint32_t m, const axiom_snapshot_contact* __restrict__ in,
                                                 WarmSlot* __restrict__ table, uint32_t* __restrict__ claim,
                                                 uint32_t gen, uint32_t log2T, DevCounters* cnt) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const axiom_snapshot_contact c = in[k];
    if (!warmInsert(table, claim, log2T, gen, warmKey(c.body_lo, c.body_hi, c.point & 0xFFu), c.point >> 8,
                    make_float4(c.impulse[0], c.impulse[1], c.impulse[2], 0.0f)))
        atomicOr(&cnt->errorFlags, 2u);
}

__global__ void __launch_bounds__(256) kDebugBodies(uint32_t n, uint32_t flags, uint32_t nAabb,
                                                    const uint32_t* __restrict__ info,
                                                    const float4* __restrict__ pos, const float4* __restrict__ rot,
                                                    const float4* __restrict__ shp, const float4* __restrict__ aabbMin,
                                                    const float4* __restrict__ aabbMax,
                                                    const SolverBody* __restrict__ sb,
                                                    const uint32_t* __restrict__ island,
                                                    axiom_debug_body* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    axiom_debug_body r{};
    const uint32_t inf = info[i];
    const uint32_t t = inf & kInfoTypeMask;
    if (flags & AXIOM_DEBUG_SHAPES) {
        const float4 p = pos[i], q = rot[i], e = shp[i];
        r.position[0] = p.x, r.position[1] = p.y, r.position[2] = p.z;
        r.rotation[0] = q.x, r.rotation[1] = q.y, r.rotation[2] = q.z, r.rotation[3] = q.w;
        r.shape = (inf >> 4) & 0xFu;
        const bool convex = isHullShape(r.shape);  // packed (radius, offset, count)
        r.shape_extents[0] = e.x, r.shape_extents[1] = convex ? 0.0f : e.y, r.shape_extents[2] = convex ? 0.0f : e.z;
    }
    if ((flags & AXIOM_DEBUG_AABBS) && i < nAabb) {
        const float4 a = aabbMin[i], b = aabbMax[i];
        r.aabb_min[0] = a.x, r.aabb_min[1] = a.y, r.aabb_min[2] = a.z;
        r.aabb_max[0] = b.x, r.aabb_max[1] = b.y, r.aabb_max[2] = b.z;
    }
    if (flags & AXIOM_DEBUG_VELOCITIES) {
        const SolverBody b = sb[i];
        r.linear_velocity[0] = b.v.x, r.linear_velocity[1] = b.v.y, r.linear_velocity[2] = b.v.z;
        r.angular_velocity[0] = b.w.x, r.angular_velocity[1] = b.w.y, r.angular_velocity[2] = b.w.z;
    }
    if (flags & AXIOM_DEBUG_ISLANDS) {
        r.is_awake = (t == AXIOM_BODY_DYNAMIC || t == AXIOM_BODY_KINEMATIC) ? 1u : 0u;
        r.island_index = island && (t == AXIOM_BODY_DYNAMIC || t == kTypeSleeping) ? island[i] : kNoIsland;
    }
    out[i] = r;
}

struct ManifoldPtrs {
    const uint4* hdr;
    const float4* n;
    const float4* p[kMaxPoints];
};

__global__ void __launch_bounds__(256) kDebugContacts(uint32_t nM, ManifoldPtrs mf,
                                                      axiom_debug_contact* __restrict__ out, uint32_t cap,
                                                      uint32_t* counter) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    const uint4 h = mf.hdr[m];
    const float4 nn = mf.n[m];
    const uint32_t np = h.z < (uint32_t)kMaxPoints ? h.z : (uint32_t)kMaxPoints;
    const uint32_t base = atomicAdd(counter, np);
    for (uint32_t k = 0; k < np; ++k) {
        if (base + k >= cap) return;
        const float4 p = mf.p[k][m];
        axiom_debug_contact c;
        c.position[0] = p.x, c.position[1] = p.y, c.position[2] = p.z;
        c.normal[0] = nn.x, c.normal[1] = nn.y, c.normal[2] = nn.z;
        c.penetration_depth = p.w;
        c.body_a = h.x;
        c.body_b = h.y;
        out[base + k] = c;
    }
}

// Entries of the warm-start table the next step reads, sorted by key.
int32_t warmEntries(World& w, std::vector<axiom_snapshot_contact>* out) {
    out->clear();
    if (!w.wsValid) return AXIOM_SUCCESS;
    const uint32_t slot = w.wsCur ^ 1u;
    const uint32_t slots = 1u << w.wsLog2[slot];
    const size_t need = 8 + sizeof(axiom_snapshot_contact) * (size_t)slots;
    AX_CUDA(w.stage.reserve(need));
    uint32_t* counter = reinterpret_cast<uint32_t*>(w.stage.p);
    auto* rec = reinterpret_cast<axiom_snapshot_contact*>(w.stage.p + 8);
    AX_CUDA(cudaMemsetAsync(counter, 0, 4, w.stream));
    kSnapWarm<<<gridFor(slots, 256), 256, 0, w.stream>>>(slots, w.wsSlots[slot].p, w.wsGen[slot], rec, slots,
                                                         counter);
    AX_CUDA(cudaGetLastError());
    uint32_t count = 0;
    AX_CUDA(cudaMemcpyAsync(&count, counter, 4, cudaMemcpyDeviceToHost, w.stream));
    AX_CUDA(cudaStreamSynchronize(w.stream));
    out->resize(count);
    if (count) {
        AX_CUDA(cudaMemcpyAsync(out->data(), rec, sizeof(axiom_snapshot_contact) * count, cudaMemcpyDeviceToHost,
                                w.stream));
        AX_CUDA(cudaStreamSynchronize(w.stream));
    }
    std::sort(out->begin(), out->end(), [](const axiom_snapshot_contact& a, const axiom_snapshot_contact& b) {
        if (a.body_lo != b.body_lo) return a.body_lo < b.body_lo;
        if (a.body_hi != b.body_hi) return a.body_hi < b.body_hi;
        return (a.point & 0xFFu) < (b.point & 0xFFu);
    });
    return AXIOM_SUCCESS;
}

uint32_t recordHull(const axiom_snapshot_body& r) {
    uint32_t id;
    std::memcpy(&id, &r.shape_extents[1], 4);
    return id;
}

bool validRecord(const axiom_snapshot_body& r, uint32_t hullCount) {
    if (r.type > AXIOM_BODY_KINEMATIC) return false;
    if (!(r.rolling_friction >= 0.0f) || !std::isfinite(r.rolling_friction)) return false;
    const uint32_t s = r.shape;
    if (s == AXIOM_SHAPE_MESH && r.type == AXIOM_BODY_DYNAMIC) return false;
    if (isHullShape(s)) return recordHull(r) < hullCount;
    if (s != AXIOM_SHAPE_SPHERE && s != AXIOM_SHAPE_BOX && s != AXIOM_SHAPE_CAPSULE && s != AXIOM_SHAPE_PLANE &&
        s != AXIOM_SHAPE_CYLINDER)
        return false;
    if (s == AXIOM_SHAPE_PLANE && r.type == AXIOM_BODY_DYNAMIC) return false;
    if ((r.flags & 1u) && r.type != AXIOM_BODY_DYNAMIC) return false;
    const float* e = r.shape_extents;
    if (s == AXIOM_SHAPE_SPHERE && !(e[0] > 0.0f)) return false;
    if (s == AXIOM_SHAPE_BOX && !(e[0] > 0.0f && e[1] > 0.0f && e[2] > 0.0f)) return false;
    if (s == AXIOM_SHAPE_CAPSULE && !(e[0] > 0.0f && e[1] >= 0.0f)) return false;
    if (s == AXIOM_SHAPE_CYLINDER && !(e[0] > 0.0f && e[1] > 0.0f)) return false;
    return true;
}

uint64_t hullBytes(const World& w) { return 4ull * w.hulls.size() + 4ull * w.hullPoints.size(); }

}  // namespace
}  // namespace axiom_gb300

using namespace axiom_gb300;

extern "C" {

AXIOM_API int32_t axiom_world_snapshot_size(void* world, uint64_t* bytes) {
    World* w = static_cast<World*>(world);
    if (!w || !bytes) return AXIOM_NULL_POINTER;
    std::vector<axiom_snapshot_contact> warm;
    int32_t st = warmEntries(*w, &warm);
    if (st != AXIOM_SUCCESS) return st;
    *bytes = sizeof(axiom_snapshot_header) + sizeof(axiom_snapshot_body) * (uint64_t)w->n +
             sizeof(axiom_snapshot_contact) * (uint64_t)warm.size() + hullBytes(*w);
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_save_snapshot(void* world, void* buffer, uint64_t capacity, uint64_t* written) {
    World* w = static_cast<World*>(world);
    if (!w || !buffer || !written) return AXIOM_NULL_POINTER;
    std::vector<axiom_snapshot_contact> warm;
    int32_t st = warmEntries(*w, &warm);
    if (st != AXIOM_SUCCESS) return st;
    const uint64_t n = w->n;
    const uint64_t total = sizeof(axiom_snapshot_header) + sizeof(axiom_snapshot_body) * n +
                           sizeof(axiom_snapshot_contact) * (uint64_t)warm.size() + hullBytes(*w);
    *written = total;
    if (capacity < total) return AXIOM_OUT_OF_RANGE;
    axiom_snapshot_header h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = AXIOM_SNAPSHOT_VERSION;
    h.body_count = (uint32_t)n;
    h.contact_count = (uint32_t)warm.size();
    h.flags = w->wsValid ? 1u : 0u;
    h.hull_count = (uint32_t)w->hulls.size();
    h.hull_vertex_count = (uint32_t)(w->hullPoints.size() / 3);
    h.total_bytes = total;
    h.config = w->cfg;
    unsigned char* out = static_cast<unsigned char*>(buffer);
    std::memcpy(out, &h, sizeof(h));
    if (n) {
        AX_CUDA(w->stage.reserve(sizeof(axiom_snapshot_body) * n));
        auto* rec = reinterpret_cast<axiom_snapshot_body*>(w->stage.p);
        const bool sl = w->cfg.allow_sleep != 0;
        kSnapBodies<<<gridFor(n, 256), 256, 0, w->stream>>>(
            (uint32_t)n, w->info.p, w->pos.p, w->rot.p, w->body.p, w->shp.p, w->mat.p, w->iloc.p, w->filt.p,
            sl ? w->sleepTime.p : nullptr, sl ? w->island.p : nullptr, rec);
        AX_CUDA(cudaGetLastError());
        AX_CUDA(cudaMemcpyAsync(out + sizeof(h), rec, sizeof(axiom_snapshot_body) * n, cudaMemcpyDeviceToHost,
                                w->stream));
        AX_CUDA(cudaStreamSynchronize(w->stream));
        if (!w->hulls.empty()) {  // convex records: pool offset bits -> hull id bits
            auto* hr = reinterpret_cast<axiom_snapshot_body*>(out + sizeof(h));
            for (uint64_t i = 0; i < n; ++i) {
                if (!isHullShape(hr[i].shape)) continue;
                uint32_t off;
                std::memcpy(&off, &hr[i].shape_extents[1], 4);
                const auto it = std::lower_bound(w->hulls.begin(), w->hulls.end(), off,
                                                 [](const HullInfo& x, uint32_t o) { return x.offset < o; });
                const uint32_t id = (uint32_t)(it - w->hulls.begin());
                std::memcpy(&hr[i].shape_extents[1], &id, 4);
                hr[i].shape_extents[2] = 0.0f;
            }
        }
    }
    unsigned char* tail = out + sizeof(h) + sizeof(axiom_snapshot_body) * n;
    if (!warm.empty()) std::memcpy(tail, warm.data(), sizeof(axiom_snapshot_contact) * warm.size());
    tail += sizeof(axiom_snapshot_contact) * warm.size();
    for (const HullInfo& hi : w->hulls) {
        std::memcpy(tail, &hi.count, 4);
        tail += 4;
    }
    if (!w->hullPoints.empty()) std::memcpy(tail, w->hullPoints.data(), 4 * w->hullPoints.size());
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_load_snapshot(void* world, const void* buffer, uint64_t size) {
    World* w = static_cast<World*>(world);
    if (!w || !buffer) return AXIOM_NULL_POINTER;
    if (size < sizeof(axiom_snapshot_header)) return AXIOM_INVALID_PARAMETER;
    axiom_snapshot_header h;
    std::memcpy(&h, buffer, sizeof(h));
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != AXIOM_SNAPSHOT_VERSION) return AXIOM_INVALID_PARAMETER;
    const uint64_t n = h.body_count, m = h.contact_count;
    const uint64_t total = sizeof(h) + sizeof(axiom_snapshot_body) * n + sizeof(axiom_snapshot_contact) * m +
                           4ull * h.hull_count + 12ull * h.hull_vertex_count;
    if (h.total_bytes != total || size < total || n >= (1ull << 30)) return AXIOM_INVALID_PARAMETER;
    axiom_world_config cfg = h.config;
    cfg.device = w->cfg.device;
    cfg.pair_capacity = w->cfg.pair_capacity;
    cfg.contact_capacity = w->cfg.contact_capacity;
    if (!(cfg.time_step > 0.0f) || cfg.warm_start > AXIOM_WARM_START_LEARNED || cfg.temporal_colouring > 1u)
        return AXIOM_INVALID_PARAMETER;
    if (cfg.allow_sleep && !(cfg.sleep_time_threshold > 0.0f && cfg.sleep_linear_threshold >= 0.0f &&
                             cfg.sleep_angular_threshold >= 0.0f))
        return AXIOM_INVALID_PARAMETER;
    const unsigned char* in = static_cast<const unsigned char*>(buffer);
    std::vector<axiom_snapshot_body> rec(n);
    if (n) std::memcpy(rec.data(), in + sizeof(h), sizeof(axiom_snapshot_body) * n);
    std::vector<axiom_snapshot_contact> warm(m);
    if (m) std::memcpy(warm.data(), in + sizeof(h) + sizeof(axiom_snapshot_body) * n, sizeof(axiom_snapshot_contact) * m);
    // hulls: per-hull vertex counts, then the points
    const unsigned char* hsec = in + sizeof(h) + sizeof(axiom_snapshot_body) * n + sizeof(axiom_snapshot_contact) * m;
    std::vector<uint32_t> hullCounts(h.hull_count);
    if (h.hull_count) std::memcpy(hullCounts.data(), hsec, 4ull * h.hull_count);
    std::vector<float> hullPoints(3ull * h.hull_vertex_count);
    if (h.hull_vertex_count) std::memcpy(hullPoints.data(), hsec + 4ull * h.hull_count, 12ull * h.hull_vertex_count);
    std::vector<HullInfo> hulls(h.hull_count);
    uint64_t off = 0;
    for (uint32_t k = 0; k < h.hull_count; ++k) {
        if (off + hullCounts[k] > h.hull_vertex_count ||
            !makeHullInfo(hullPoints.data() + 3 * off, hullCounts[k], (uint32_t)off, &hulls[k], 3))
            return AXIOM_INVALID_PARAMETER;
        off += hullCounts[k];
    }
    if (off != h.hull_vertex_count) return AXIOM_INVALID_PARAMETER;
    for (const auto& r : rec)
        if (!validRecord(r, h.hull_count)) return AXIOM_INVALID_PARAMETER;
    for (const auto& c : warm)
        if (c.body_lo >= n || c.body_hi >= n || (c.point & 0xFFu) >= (uint32_t)kMaxPoints ||
            (c.point >> 8) > (uint32_t)kMaxColours || ((c.point & 0xFFu) != 0u && (c.point >> 8) != 0u))
            return AXIOM_INVALID_PARAMETER;
    AX_CUDA(cudaStreamSynchronize(w->stream));
    resetBodies(*w);
    w->cfg = cfg;
    if (h.hull_vertex_count) {
        AX_CUDA(w->hullVerts.reserve(h.hull_vertex_count));
        std::vector<float4> v4(h.hull_vertex_count);
        for (uint64_t i = 0; i < h.hull_vertex_count; ++i)
            v4[i] = make_float4(hullPoints[3 * i], hullPoints[3 * i + 1], hullPoints[3 * i + 2], 0.0f);
        AX_CUDA(cudaMemcpyAsync(w->hullVerts.p, v4.data(), sizeof(float4) * v4.size(), cudaMemcpyHostToDevice,
                                w->stream));
        AX_CUDA(cudaStreamSynchronize(w->stream));
    }
    w->hulls = hulls;
    w->hullPoints = hullPoints;
    if (n == 0) return AXIOM_SUCCESS;
    const bool sleepOn = cfg.allow_sleep != 0;
    PackedBodies pk;
    pk.pos.resize(n), pk.rot.resize(n), pk.shp.resize(n), pk.mat.resize(n), pk.iloc.resize(n);
    pk.body.resize(n), pk.info.resize(n), pk.filt.resize(n);
    std::vector<float> sleepTime(n);
    std::vector<uint32_t> island(n);
    for (uint64_t i = 0; i < n; ++i) {
        const axiom_snapshot_body& r = rec[i];
        const float* ii = r.inv_inertia;
        const bool iso = ii[0] == ii[1] && ii[1] == ii[2];
        pk.pos[i] = make_float4(r.position[0], r.position[1], r.position[2], 0.0f);
        pk.rot[i] = make_float4(r.rotation[0], r.rotation[1], r.rotation[2], r.rotation[3]);
        pk.body[i].v = make_float4(r.linear_velocity[0], r.linear_velocity[1], r.linear_velocity[2], r.inv_mass);
        pk.body[i].w = make_float4(r.angular_velocity[0], r.angular_velocity[1], r.angular_velocity[2],
                                   iso ? ii[0] : -1.0f);
        pk.shp[i] = isHullShape(r.shape) ? convexShp(hulls[recordHull(r)])
                                                   : make_float4(r.shape_extents[0], r.shape_extents[1],
                                                                 r.shape_extents[2], 0.0f);
        pk.mat[i] = make_float4(r.friction, r.restitution, r.linear_damping, r.angular_damping);
        pk.iloc[i] = make_float4(ii[0], ii[1], ii[2], r.rolling_friction);
        pk.filt[i] = make_uint4(r.filter_category, r.filter_mask, (uint32_t)r.filter_group, 0u);
        const bool filtered = r.filter_category != 0x0001u || r.filter_mask != 0xFFFFu || r.filter_group != 0;
        const bool asleep = sleepOn && (r.flags & 1u);
        const bool noSleep = sleepOn && (r.flags & 2u) && r.type == AXIOM_BODY_DYNAMIC;
        pk.info[i] = (asleep ? kTypeSleeping : r.type) | (r.shape << 4) | (filtered ? kInfoFiltered : 0u) |
                     (noSleep ? kInfoNoSleep : 0u);
        sleepTime[i] = r.sleep_time;
        island[i] = r.island;
    }
    int32_t st = appendPackedBodies(*w, pk, (uint32_t)n, sleepTime.data(), island.data());
    if (st != AXIOM_SUCCESS) return st;
    if (h.flags & 1u) {
        const uint32_t slot = w->wsCur ^ 1u;
        if ((st = reserveWarmTable(*w, slot, (uint32_t)m)) != AXIOM_SUCCESS) return st;
        const uint32_t gen = nextWarmGen(*w, slot);  // the table's older entries turn empty
        if (m) {
            AX_CUDA(w->stage.reserve(sizeof(axiom_snapshot_contact) * m));
            AX_CUDA(cudaMemcpyAsync(w->stage.p, warm.data(), sizeof(axiom_snapshot_contact) * m,
                                    cudaMemcpyHostToDevice, w->stream));
            AX_CUDA(cudaMemsetAsync(&w->dcnt->errorFlags, 0, 4, w->stream));
            kLoadWarm<<<gridFor(m, 256), 256, 0, w->stream>>>(
                (uint32_t)m, reinterpret_cast<const axiom_snapshot_contact*>(w->stage.p), w->wsSlots[slot].p,
                w->wsClaim[slot].p, gen,
                w->wsLog2[slot], w->dcnt);
            AX_CUDA(cudaGetLastError());
        }
        AX_CUDA(cudaStreamSynchronize(w->stream));
        w->wsValid = true;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_debug(void* world, uint32_t flags, axiom_debug_body* bodies, uint32_t body_capacity,
                                         axiom_debug_contact* contacts, uint32_t contact_capacity,
                                         uint32_t* body_count, uint32_t* contact_count) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    const uint32_t n = w->n;
    const uint32_t nPts = (flags & AXIOM_DEBUG_CONTACTS) ? w->lastPoints : 0u;
    if (body_count) *body_count = n;
    if (contact_count) *contact_count = nPts;
    const uint32_t nb = bodies ? std::min(n, body_capacity) : 0u;
    const uint32_t nc = contacts ? std::min(nPts, contact_capacity) : 0u;
    if (!nb && !nc) return AXIOM_SUCCESS;
    const size_t bodyBytes = sizeof(axiom_debug_body) * (size_t)n;
    const size_t cOff = (bodyBytes + 255) & ~(size_t)255;
    AX_CUDA(w->stage.reserve(cOff + 8 + sizeof(axiom_debug_contact) * (size_t)nPts));
    auto* dbody = reinterpret_cast<axiom_debug_body*>(w->stage.p);
    uint32_t* counter = reinterpret_cast<uint32_t*>(w->stage.p + cOff);
    auto* dcon = reinterpret_cast<axiom_debug_contact*>(w->stage.p + cOff + 8);
    if (nb) {
        kDebugBodies<<<gridFor(n, 256), 256, 0, w->stream>>>(n, flags, w->aabbCount, w->info.p, w->pos.p, w->rot.p,
                                                             w->shp.p, w->aabbMin.p, w->aabbMax.p, w->body.p,
                                                             w->cfg.allow_sleep ? w->island.p : nullptr, dbody);
        AX_CUDA(cudaGetLastError());
        AX_CUDA(cudaMemcpyAsync(bodies, dbody, sizeof(axiom_debug_body) * nb, cudaMemcpyDeviceToHost, w->stream));
    }
    if (nc) {
        ManifoldPtrs mp;
        mp.hdr = w->mhdr.p;
        mp.n = w->mn.p;
        for (int k = 0; k < kMaxPoints; ++k) mp.p[k] = w->mp[k].p;
        AX_CUDA(cudaMemsetAsync(counter, 0, 4, w->stream));
        kDebugContacts<<<gridFor(w->lastManifolds, 256), 256, 0, w->stream>>>(w->lastManifolds, mp, dcon, nPts,
                                                                              counter);
        AX_CUDA(cudaGetLastError());
        AX_CUDA(cudaMemcpyAsync(contacts, dcon, sizeof(axiom_debug_contact) * nc, cudaMemcpyDeviceToHost, w->stream));
    }
    AX_CUDA(cudaStreamSynchronize(w->stream));
    return AXIOM_SUCCESS;
}

}  // extern "C"
