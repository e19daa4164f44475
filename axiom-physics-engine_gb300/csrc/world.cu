// world.cu — C ABI of the GB300 step (include/axiom_c.h) and its stage orchestration.
//
// Stage order follows the reference's step: broadphase, narrowphase, solver,
// integration (examples/profiling_example.cpp:132-165; PhysicsWorldStats timing fields,
// include/axiom/gui/physics_panel.hpp:24-29).  Everything runs on the world's own
// stream; the host synchronises only to size the variable-length stages (pair count,
// manifold count, colour count) and at the end of the step for the statistics.
#include <algorithm>
#include <functional>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "body_pack.h"
#include "host_math.h"
#include "world.h"

namespace axiom_gb300 {

const char* const kKernelGroupNames[KG_COUNT] = {
    "integrate_velocities", "radix_sort",        "broadphase_gather", "broadphase_sweep",
    "narrowphase",          "colouring",         "solver_prepare",    "warm_start_apply",
    "pgs_colour",           "store_impulses",    "integrate_positions", "sleep_islands"};

ProfRange::ProfRange(World& world, int g) : w(&world), group(g) {
    if (!w->prof.enabled || !((w->prof.mask >> g) & 1u)) return;
    if (w->prof.pool.empty()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        w->prof.pool.push_back(e);
    }
    a = w->prof.pool.back();
    w->prof.pool.pop_back();
    cudaEventRecord(a, w->stream);
}

ProfRange::~ProfRange() {
    if (!a) return;
    cudaEvent_t b;
    if (w->prof.pool.empty()) {
        if (cudaEventCreate(&b) != cudaSuccess) {
            w->prof.pool.push_back(a);
            return;
        }
    } else {
        b = w->prof.pool.back();
        w->prof.pool.pop_back();
    }
    cudaEventRecord(b, w->stream);
    w->prof.pending.push_back({group, a, b});
}

void resolveProfile(World& w) {
    for (const auto& p : w.prof.pending) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            w.prof.ms[p.group] += ms;
            w.prof.ranges[p.group] += 1;
        }
        w.prof.pool.push_back(p.a);
        w.prof.pool.push_back(p.b);
    }
    w.prof.pending.clear();
}

namespace {

#define AX_CUDA(call)                                         \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED; \
    } while (0)

uint32_t ceilLog2(uint64_t v) {
    uint32_t l = 0;
    while ((1ull << l) < v) ++l;
    return l;
}

// Packs .xyz of every `stride`-th float4 into a dense 3-float array.
__global__ void kPack3(uint32_t n, const float4* __restrict__ src, uint32_t stride, float* __restrict__ dst) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = src[(size_t)i * stride];
    dst[3 * i] = v.x;
    dst[3 * i + 1] = v.y;
    dst[3 * i + 2] = v.z;
}

// Writes a dense 3-float array into .xyz of every `stride`-th float4 (keeps .w).
__global__ void kUnpack3(uint32_t n, const float* __restrict__ src, float4* __restrict__ dst, uint32_t stride) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = dst[(size_t)i * stride];
    v.x = src[3 * i];
    v.y = src[3 * i + 1];
    v.z = src[3 * i + 2];
    dst[(size_t)i * stride] = v;
}

// Body state in the caller's layout (position, linear and angular velocity [3n] each,
// rotation [4n]; any may be null) <-> the device layout, in one pass over device staging
// regions that the copy engines fill or drain back to back.  (Kernels reading or writing
// page-locked host arrays in place over the host-device link measured slower than these
// bulk copies: 3.2e8 vs 3.9e8 body-steps/s end to end on the 1M pile.)
struct StateIO {
    float* pos;
    float* rot;
    float* lin;
    float* ang;
};

__global__ void __launch_bounds__(256) kStateIn(uint32_t n, StateIO in, float4* __restrict__ pos,
                                                float4* __restrict__ rot, SolverBody* __restrict__ sb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (in.pos) {
        float4 p = pos[i];
        p.x = in.pos[3 * i];
        p.y = in.pos[3 * i + 1];
        p.z = in.pos[3 * i + 2];
        pos[i] = p;
    }
    if (in.rot) rot[i] = make_float4(in.rot[4 * i], in.rot[4 * i + 1], in.rot[4 * i + 2], in.rot[4 * i + 3]);
    if (in.lin) {
        float4 v = sb[i].v;
        v.x = in.lin[3 * i];
        v.y = in.lin[3 * i + 1];
        v.z = in.lin[3 * i + 2];
        sb[i].v = v;
    }
    if (in.ang) {
        float4 v = sb[i].w;
        v.x = in.ang[3 * i];
        v.y = in.ang[3 * i + 1];
        v.z = in.ang[3 * i + 2];
        sb[i].w = v;
    }
}

__global__ void __launch_bounds__(256) kStateOut(uint32_t n, StateIO out, const float4* __restrict__ pos,
                                                 const float4* __restrict__ rot, const SolverBody* __restrict__ sb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (out.pos) {
        const float4 p = pos[i];
        out.pos[3 * i] = p.x;
        out.pos[3 * i + 1] = p.y;
        out.pos[3 * i + 2] = p.z;
    }
    if (out.rot) {
        const float4 q = rot[i];
        out.rot[4 * i] = q.x;
        out.rot[4 * i + 1] = q.y;
        out.rot[4 * i + 2] = q.z;
        out.rot[4 * i + 3] = q.w;
    }
    if (out.lin) {
        const float4 v = sb[i].v;
        out.lin[3 * i] = v.x;
        out.lin[3 * i + 1] = v.y;
        out.lin[3 * i + 2] = v.z;
    }
    if (out.ang) {
        const float4 v = sb[i].w;
        out.ang[3 * i] = v.x;
        out.ang[3 * i + 1] = v.y;
        out.ang[3 * i + 2] = v.z;
    }
}

// Device staging for the pageable arrays of a state transfer: 13 floats per body at most.
float* stateStaging(World& w) {
    if (w.stage.cap < 52ull * w.n && w.stage.reserve(52ull * w.n) != cudaSuccess) return nullptr;
    return reinterpret_cast<float*>(w.stage.p);
}

int32_t ensureBodyCapacity(World& w, uint32_t n) {
    DevBuf<float4>* f4[] = {&w.pos, &w.rot, &w.shp, &w.mat, &w.iloc, &w.iw0, &w.iw1};
    for (auto* b : f4) AX_CUDA(b->grow(n, w.stream));
    AX_CUDA(w.body.grow(n, w.stream));
    AX_CUDA(w.info.grow(n, w.stream));
    AX_CUDA(w.filt.grow(n, w.stream));
    if (w.cfg.allow_sleep) {
        AX_CUDA(w.sleepTime.grow(n, w.stream));
        AX_CUDA(w.island.grow(n, w.stream));
        AX_CUDA(w.wakeGen.grow(n, w.stream));
        AX_CUDA(w.ufParent.reserve(n));
        AX_CUDA(w.islandMin.reserve(n));
    }
    AX_CUDA(w.aabbMin.reserve(n));
    AX_CUDA(w.nbody.reserve(n));
    AX_CUDA(w.aabbMax.reserve(n));
    AX_CUDA(w.sbox.reserve(n));
    AX_CUDA(w.bodyMask.reserve(n));
    AX_CUDA(w.bodyDeg.reserve(n));
    AX_CUDA(w.bodySlots.reserve((size_t)kMaxColours * n));
    const uint32_t log2T = ceilLog2(std::max<uint64_t>(2ull * n, 1024ull));
    if (log2T > w.cellTableLog2) {
        AX_CUDA(w.cellTable.reserve(1ull << log2T));
        w.cellTableLog2 = log2T;
    }
    return AXIOM_SUCCESS;
}

// Scratch sized by max(bodies, manifolds).  keyA / valA keep their contents: they hold the
// step's sorted cell keys and ids while the narrowphase may still grow the manifold arrays.
int32_t ensureSortCapacity(World& w, uint32_t items) {
    AX_CUDA(w.keyA.grow(items, w.stream));
    AX_CUDA(w.keyB.reserve(items));
    AX_CUDA(w.valA.grow(items, w.stream));
    AX_CUDA(w.valB.reserve(items));
    AX_CUDA(w.hist.reserve(std::max<uint32_t>(radixHistWords(items), 1100u)));
    return AXIOM_SUCCESS;
}

int32_t ensureManifoldCapacity(World& w, uint32_t want) {
    AX_CUDA(w.mhdr.reserve(want));
    // every per-manifold array holds the header list's capacity: counts up to it are valid
    const size_t m = w.mhdr.cap;
    AX_CUDA(w.mn.reserve(m));
    for (int k = 0; k < kMaxPoints; ++k) AX_CUDA(w.mp[k].reserve(m));
    AX_CUDA(w.work0.reserve(m));
    AX_CUDA(w.manRec.reserve(m));
    AX_CUDA(w.manSucc.reserve(m));
    AX_CUDA(w.manPending.reserve(m));
    AX_CUDA(w.mcolour.reserve(m));
    AX_CUDA(w.order.reserve(m));
    AX_CUDA(w.orderInv.reserve(m));
    AX_CUDA(w.shdr.reserve(m));
    AX_CUDA(w.sn.reserve(m));
    for (int k = 0; k < kMaxPoints; ++k) {
        AX_CUDA(w.sra[k].reserve(m));
        AX_CUDA(w.srb[k].reserve(m));
        AX_CUDA(w.skt[k].reserve(m));
        AX_CUDA(w.slam[k].reserve(m));
    }
    if (w.needFeatures || w.recording || w.cfg.warm_start == AXIOM_WARM_START_LEARNED) {
        AX_CUDA(w.feat.reserve(64ull * m));
    }
    return ensureSortCapacity(w, std::max<uint32_t>(m, w.n));
}

int32_t ensureWarmTable(World& w, uint32_t slot, uint32_t points) {
    const uint32_t log2T = ceilLog2(std::max<uint64_t>(2ull * points, 1024ull));
    if (log2T > w.wsLog2[slot]) {
        // a new table starts with every slot at generation 0 (empty)
        AX_CUDA(w.wsSlots[slot].reserve(1ull << log2T));
        AX_CUDA(w.wsClaim[slot].reserve(1ull << log2T));
        AX_CUDA(cudaMemsetAsync(w.wsSlots[slot].p, 0, sizeof(WarmSlot) << log2T, w.stream));
        AX_CUDA(cudaMemsetAsync(w.wsClaim[slot].p, 0, sizeof(uint32_t) << log2T, w.stream));
        w.wsLog2[slot] = log2T;
        w.wsGen[slot] = 0;
    }
    return AXIOM_SUCCESS;
}


int32_t syncCounters(World& w) {
    AX_CUDA(cudaMemcpyAsync(w.hcnt, w.dcnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, w.stream));
    AX_CUDA(cudaStreamSynchronize(w.stream));
    return AXIOM_SUCCESS;
}

StepParams makeParams(const World& w, float dt) {
    StepParams sp{};
    sp.dt = dt;
    sp.invDt = 1.0f / dt;
    sp.hdt = 0.5f * dt;
    sp.gx = w.cfg.gravity[0];
    sp.gy = w.cfg.gravity[1];
    sp.gz = w.cfg.gravity[2];
    sp.biasCoeff = w.cfg.baumgarte * sp.invDt;
    sp.slop = w.cfg.linear_slop;
    sp.margin = w.cfg.aabb_margin;
    sp.restThreshold = w.cfg.restitution_threshold;
    const float gw = w.nLarge ? w.gridWidth : w.maxWidth;  // large bodies are not in the grid
    const float cell = gw > 0.0f ? gw * 1.0625f : 1.0f;
    sp.invCell = 1.0f / cell;
    sp.cellWidth = w.maxWidth;
    sp.spec = w.cfg.speculative_contacts ? 1u : 0u;
    sp.warmFactor = w.cfg.warm_start_factor;
    sp.tolerance = w.cfg.residual_tolerance;
    sp.n = w.n;
    sp.nPlanes = w.nPlanes;
    sp.warmStart = w.cfg.warm_start;
    const float* g = w.cfg.gravity;
    sp.gdt = sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) * dt;
    sp.sleepLin2 = w.cfg.sleep_linear_threshold * w.cfg.sleep_linear_threshold;
    sp.sleepAng2 = w.cfg.sleep_angular_threshold * w.cfg.sleep_angular_threshold;
    sp.sleepTime = w.cfg.sleep_time_threshold;
    return sp;
}

// Zeroes the counters the narrowphase accumulates (before it runs again).
int32_t resetNarrowCounters(World& w) {
    AX_CUDA(cudaMemsetAsync(&w.dcnt->manifolds, 0, 2 * sizeof(uint32_t), w.stream));  // manifolds, points
    AX_CUDA(cudaMemsetAsync(&w.dcnt->gjkPairs, 0, sizeof(uint32_t), w.stream));
    AX_CUDA(cudaMemsetAsync(&w.dcnt->mixedPairs, 0, sizeof(uint32_t), w.stream));
    AX_CUDA(cudaMemsetAsync(&w.dcnt->gjkFailures, 0, 2 * sizeof(uint32_t), w.stream));  // gjk, epa
    AX_CUDA(cudaMemsetAsync(&w.dcnt->planeQueue, 0, sizeof(uint32_t), w.stream));
    return AXIOM_SUCCESS;
}

// Broadphase sweep and narrowphase with one host sync: the narrowphase reads the pair count
// on the device.  A pair list that overflowed (the narrowphase then saw only the listed
// pairs) is grown and both stages run again; a manifold list that overflowed is grown and
// the narrowphase runs again.  Neither stage changes body state, so a redo needs no rollback.
int32_t sweepAndCollide(World& w, const StepParams& sp, uint32_t nSorted, uint32_t* nPairs, uint32_t* nM) {
    int32_t st;
    const uint32_t expected =
        w.pairsValid ? std::min<uint32_t>(w.lastPairs + w.lastPairs / 4 + 1024u, (uint32_t)w.pairs.cap)
                     : (uint32_t)w.pairs.cap;
    launchBroadphase(w, sp, nSorted);
    launchLargePairs(w);
    AX_CUDA(cudaEventRecord(w.ev[1], w.stream));
    launchNarrowphase(w, sp, expected);
    if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
    *nPairs = w.hcnt->pairs;
    *nM = w.hcnt->manifolds;
    if (*nPairs > w.pairs.cap) {
        AX_CUDA(w.pairs.reserve(*nPairs + *nPairs / 4));
        AX_CUDA(w.gjkQueue.reserve(w.pairs.cap));
        AX_CUDA(cudaMemsetAsync(&w.dcnt->pairs, 0, sizeof(uint32_t), w.stream));
        if ((st = resetNarrowCounters(w)) != AXIOM_SUCCESS) return st;
        launchBroadphase(w, sp, nSorted);
        launchLargePairs(w);
        launchNarrowphase(w, sp, *nPairs);
        if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
        *nPairs = w.hcnt->pairs;
        *nM = w.hcnt->manifolds;
    }
    if (*nM > w.mhdr.cap) {
        if ((st = ensureManifoldCapacity(w, *nM + *nM / 4)) != AXIOM_SUCCESS) return st;
        if ((st = resetNarrowCounters(w)) != AXIOM_SUCCESS) return st;
        launchNarrowphase(w, sp, *nPairs);
        if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
        *nM = w.hcnt->manifolds;
    }
    return AXIOM_SUCCESS;
}

int32_t step(World& w, float dt, axiom_step_stats* stats) {
    if (!(dt > 0.0f)) dt = w.cfg.time_step;
    const StepParams sp = makeParams(w, dt);
    cudaStream_t s = w.stream;
    int32_t st;
    AX_CUDA(cudaMemsetAsync(w.dcnt, 0, sizeof(DevCounters), s));
    AX_CUDA(cudaEventRecord(w.ev[0], s));
    uint32_t nPairs = 0, nM = 0, nPts = 0, nColours = 0, iters = 0;
    bool small = false;  // the solve ran as one single-CTA launch (smallSolve)
    bool mid = false;    // the solve ran as one cluster launch (clusterSolve)
    float residual = 0.0f;
    int32_t status = AXIOM_SUCCESS;
    if (w.n > 0) {
        // ---- broadphase ----
        launchIntegrateVelocities(w, sp);
        launchMarkLarge(w);
        w.aabbCount = w.n;
        radixSortPairs(w, w.n);
        const uint32_t nSorted = w.n - w.nPlanes - w.nLarge;
        launchBroadphaseGather(w, nSorted);
        // ---- broadphase sweep and narrowphase (one host sync) ----
        if ((st = sweepAndCollide(w, sp, nSorted, &nPairs, &nM)) != AXIOM_SUCCESS) return st;
        // ---- wake: sleeping islands touched by awake bodies wake in this step, and the
        // contacts are computed again with them awake (sorted order and AABBs unchanged) ----
        for (int pass = 0; w.cfg.allow_sleep && w.nSleeping > 0 && pass < kMaxWakePasses; ++pass) {
            launchWake(w, sp, nM);
            if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
            const uint32_t woken = w.hcnt->woken;
            if (woken == 0) break;
            w.nSleeping -= std::min(woken, w.nSleeping);
            AX_CUDA(cudaMemsetAsync(&w.dcnt->pairs, 0, sizeof(uint32_t), s));
            if ((st = resetNarrowCounters(w)) != AXIOM_SUCCESS) return st;
            launchBroadphaseGather(w, nSorted);
            if ((st = sweepAndCollide(w, sp, nSorted, &nPairs, &nM)) != AXIOM_SUCCESS) return st;
        }
        nPts = w.hcnt->points;
        AX_CUDA(cudaEventRecord(w.ev[2], s));
        // ---- solver ----
        AX_CUDA(colourManifolds(w, nM));
        // a small or mid-size world solves in one launch that reads the colouring on the
        // device: no sync here, the colour count and status come with the step's last sync
        // a small world with multi-point manifolds and more than 1,024 of them solves faster
        // in the cluster, whose hoisted point rows shorten the four-point chain
        small = smallSolve(w, nM) && !(nPts > nM && nM > 1024u);
        mid = !small && clusterSolve(w, nM, nPts > nM);
        if (!small && !mid) {
            if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
            if (w.lastRounds == kRoundsFromCounters) w.lastRounds = w.hcnt->colourRounds;
            nColours = w.hcnt->maxColour;
            if (w.hcnt->colourOverflow) status = AXIOM_CONSTRAINT_SOLVER_FAILURE;
            // the crowded batch (grouped last) goes into descending priority for its serial solve
            w.lastCrowded = nM ? w.hcnt->colourStart[kMaxColours + 1] - w.hcnt->colourStart[kMaxColours] : 0u;
            AX_CUDA(sortCrowded(w, w.lastCrowded));
        }
        if (status == AXIOM_SUCCESS && nM > 0) {
            w.needFeatures = w.recording || sp.warmStart == AXIOM_WARM_START_LEARNED;
            if (w.needFeatures) AX_CUDA(w.feat.reserve(64ull * w.mhdr.cap));
            launchPrepare(w, sp, nM);
            if (sp.warmStart == AXIOM_WARM_START_LEARNED && w.mlpLoaded) {
                // network warm start on the contact points only: nPts rows, gathered from
                // the feature rows slot * nM + s
                const uint32_t rows = nPts;
                AX_CUDA(w.mlp.reserveRows(rows));
                AX_CUDA(w.learnRows.reserve(4ull * nM));
                AX_CUDA(w.learnRowOf.reserve(4ull * nM));
                launchLearnRows(w, nM);
                w.mlp.infer(w.feat.p, 16, w.learnRows.p, rows, s);  // the fused tcgen05 network
                launchApplyLearned(w, sp, nM, w.mlp.Y);
            }
            const bool tolMode = w.cfg.residual_tolerance > 0.0f;
            if (small) {
                AX_CUDA(launchSolveSmall(w, sp, tolMode ? w.cfg.max_iterations : w.cfg.velocity_iterations, tolMode));
            } else if (mid) {
                AX_CUDA(launchSolveCluster(w, sp, nM, tolMode ? w.cfg.max_iterations : w.cfg.velocity_iterations,
                                           tolMode));
            } else {
                w.hoistRows = nPts > nM;  // multi-point manifolds: the hoisted-rows colour kernel
                launchWarmStartApply(w, nM, nColours);
                if (!tolMode) {
                    // one profiler range for all sweeps: events between launches would break the
                    // programmatic-dependent-launch chain
                    ProfRange pr(w, KG_PGS_COLOUR);
                    launchSweeps(w, sp, nM, nColours, w.cfg.velocity_iterations, false);
                } else {
                    // chunks of 8 sweeps; the first convergence test (a host sync) comes two
                    // chunks short of the last step's sweep count (sweeps launched after
                    // convergence return at once, so launching ahead costs little)
                    const uint32_t ahead = w.last.iterations > 16u ? (w.last.iterations - 16u) / 8u * 8u : 0u;
                    uint32_t launched = 0;
                    while (launched < w.cfg.max_iterations) {
                        const uint32_t chunk = std::min<uint32_t>(8u, w.cfg.max_iterations - launched);
                        {
                            ProfRange pr(w, KG_PGS_COLOUR);
                            launchSweeps(w, sp, nM, nColours, chunk, true);
                        }
                        launched += chunk;
                        if (launched < ahead) continue;
                        if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
                        if (w.hcnt->converged) break;
                    }
                }
            }
        }
        if ((st = ensureWarmTable(w, w.wsCur, nPts)) != AXIOM_SUCCESS) return st;
        launchStoreImpulses(w, status == AXIOM_SUCCESS ? nM : 0);
        AX_CUDA(cudaEventRecord(w.ev[3], s));
        // ---- integration ----
        launchIntegratePositions(w, sp);
        // ---- islands and sleeping ----
        if (w.cfg.allow_sleep) launchIslands(w, sp, nM);
    } else {
        for (int k = 1; k < 4; ++k) AX_CUDA(cudaEventRecord(w.ev[k], s));
    }
    AX_CUDA(cudaEventRecord(w.ev[4], s));
    AX_CUDA(cudaGetLastError());
    if ((st = syncCounters(w)) != AXIOM_SUCCESS) return st;
    resolveProfile(w);
    if (small || mid) {
        if (w.lastRounds == kRoundsFromCounters) w.lastRounds = w.hcnt->colourRounds;
        nColours = w.hcnt->maxColour;
        if (w.hcnt->colourOverflow) status = AXIOM_CONSTRAINT_SOLVER_FAILURE;
        w.lastCrowded = w.hcnt->colourStart[kMaxColours + 1] - w.hcnt->colourStart[kMaxColours];
    }
    iters = w.hcnt->iterations;
    residual = w.hcnt->residual;
    if (w.hcnt->errorFlags) status = AXIOM_GPU_INVALID_OPERATION;
    if (w.cfg.residual_tolerance > 0.0f && nM > 0 && !w.hcnt->converged && status == AXIOM_SUCCESS)
        status = AXIOM_CONSTRAINT_SOLVER_FAILURE;
    // the step completes either way; the status names the first convergence failure met
    const uint32_t gjkFail = w.n > 0 ? w.hcnt->gjkFailures : 0u, epaFail = w.n > 0 ? w.hcnt->epaFailures : 0u;
    if (status == AXIOM_SUCCESS && gjkFail) status = AXIOM_GJK_FAILED_TO_CONVERGE;
    if (status == AXIOM_SUCCESS && epaFail) status = AXIOM_EPA_FAILED_TO_CONVERGE;
    w.wsValid = true;
    w.wsCur ^= 1u;
    w.lastPairs = nPairs;
    w.pairsValid = true;
    w.lastManifolds = nM;
    w.lastPoints = nPts;
    w.lastColours = nColours;
    if (w.cfg.allow_sleep && w.n > 0) {
        w.nSleeping = w.hcnt->sleeping;
        w.lastIslands = w.hcnt->islands;
    }

    axiom_step_stats& o = w.last;
    std::memset(&o, 0, sizeof(o));
    o.total_bodies = w.n;
    o.static_bodies = w.nStatic;
    o.dynamic_bodies = w.nDynamic;
    o.kinematic_bodies = w.nKinematic;
    o.active_bodies = w.nDynamic - std::min(w.nSleeping, w.nDynamic);
    o.sleeping_bodies = w.nSleeping;
    o.island_count = w.cfg.allow_sleep ? w.lastIslands : 0u;
    o.contact_point_count = nPts;
    float t[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k) cudaEventElapsedTime(&t[k], w.ev[k], w.ev[k + 1]);
    cudaEventElapsedTime(&o.total_step_time, w.ev[0], w.ev[4]);
    o.broadphase_time = t[0];
    o.narrowphase_time = t[1];
    o.solver_time = t[2];
    o.integration_time = t[3];
    o.pair_count = nPairs;
    o.manifold_count = nM;
    o.colour_count = nColours;
    o.iterations = iters;
    o.residual = residual;
    o.status = status;
    o.colour_rounds = w.lastRounds;
    o.gjk_failures = gjkFail;
    o.epa_failures = epaFail;
    if (stats) *stats = o;
    return status;
}

}  // namespace

bool makeHullInfo(const float* points, uint32_t count, uint32_t offset, HullInfo* h, uint32_t minCount) {
    if (count < minCount || count > AXIOM_CONVEX_MAX_VERTICES) return false;
    h->offset = offset;
    h->count = count;
    float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f}, r2 = 0.0f;
    for (uint32_t i = 0; i < count; ++i) {
        const float* v = points + 3 * i;
        if (!std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2])) return false;
        for (int k = 0; k < 3; ++k) {
            mn[k] = i == 0 || v[k] < mn[k] ? v[k] : mn[k];
            mx[k] = i == 0 || v[k] > mx[k] ? v[k] : mx[k];
        }
        const float d2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
        r2 = d2 > r2 ? d2 : r2;
    }
    h->radius = std::sqrt(r2);
    for (int k = 0; k < 3; ++k) h->halfExtents[k] = 0.5f * (mx[k] - mn[k]);
    return h->radius > 0.0f;
}

int32_t appendHull(World& w, const float* points, uint32_t count, uint32_t minCount, uint32_t* id) {
    HullInfo h{};
    if (!makeHullInfo(points, count, (uint32_t)(w.hullPoints.size() / 3), &h, minCount)) return AXIOM_INVALID_SHAPE;
    AX_CUDA(w.hullVerts.grow(h.offset + count, w.stream));
    std::vector<float4> v4(count);
    for (uint32_t i = 0; i < count; ++i) v4[i] = make_float4(points[3 * i], points[3 * i + 1], points[3 * i + 2], 0.0f);
    AX_CUDA(cudaMemcpyAsync(w.hullVerts.p + h.offset, v4.data(), sizeof(float4) * count, cudaMemcpyHostToDevice,
                            w.stream));
    AX_CUDA(cudaStreamSynchronize(w.stream));
    w.hullPoints.insert(w.hullPoints.end(), points, points + 3 * count);
    *id = (uint32_t)w.hulls.size();
    w.hulls.push_back(h);
    return AXIOM_SUCCESS;
}

// Validates a triangle mesh and gives each triangle its centroid and its three points
// about it: centre = (v0 + v1 + v2) / 3 (in that order), point k = v_k - centre.
int32_t checkMesh(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nt, float* centre, float* pts) {
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t i0 = tri[3 * t], i1 = tri[3 * t + 1], i2 = tri[3 * t + 2];
        if (i0 >= nv || i1 >= nv || i2 >= nv) return AXIOM_OUT_OF_RANGE;
        const float* a = v + 3ull * i0;
        const float* b = v + 3ull * i1;
        const float* c = v + 3ull * i2;
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(a[k]) || !std::isfinite(b[k]) || !std::isfinite(c[k])) return AXIOM_INVALID_SHAPE;
        const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const float cx = e1[1] * e2[2] - e1[2] * e2[1];
        const float cy = e1[2] * e2[0] - e1[0] * e2[2];
        const float cz = e1[0] * e2[1] - e1[1] * e2[0];
        if (!((cx * cx + cy * cy) + cz * cz > 0.0f)) return AXIOM_INVALID_SHAPE;  // no area
        float* ce = centre + 3ull * t;
        for (int k = 0; k < 3; ++k) ce[k] = ((a[k] + b[k]) + c[k]) / 3.0f;
        float* p = pts + 9ull * t;
        for (int k = 0; k < 3; ++k) {
            p[k] = a[k] - ce[k];
            p[3 + k] = b[k] - ce[k];
            p[6 + k] = c[k] - ce[k];
        }
    }
    return AXIOM_SUCCESS;
}

// Size disparity.  A uniform grid needs cells as wide as its widest body, so one body far
// wider than the rest (a big static box under a pile, a big mesh triangle) would put
// everything into a few huge cells.  With at least 64 bodies, a body is large when it is
// wider than 8 x the median width; at most kMaxLarge of the widest such bodies are taken
// (the threshold T is the widest width not taken, and large = wider than T), the grid is
// sized for T, and each large body is tested against every body instead.  Speculative
// contacts size their grid on the device from swept AABBs and take no large bodies.
int32_t classifyLarge(World& w) {
    w.nLarge = 0;
    w.gridWidth = w.maxWidth;
    if (w.cfg.speculative_contacts) return AXIOM_SUCCESS;
    std::vector<float> widths;
    widths.reserve(w.hostWidth.size());
    for (float x : w.hostWidth)
        if (x >= 0.0f) widths.push_back(x);
    if (widths.size() < 64) return AXIOM_SUCCESS;
    std::vector<float> med(widths);
    std::nth_element(med.begin(), med.begin() + med.size() / 2, med.end());
    const float limit = 8.0f * med[med.size() / 2];
    const size_t top = std::min<size_t>(kMaxLarge + 1, widths.size());
    std::partial_sort(widths.begin(), widths.begin() + top, widths.end(), std::greater<float>());
    size_t taken = 0;
    while (taken < top - 1 && widths[taken] > limit) ++taken;
    if (taken == 0) return AXIOM_SUCCESS;
    const float T = widths[taken];
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < (uint32_t)w.hostWidth.size(); ++i)
        if (w.hostWidth[i] > T) ids.push_back(i);
    if (ids.empty()) return AXIOM_SUCCESS;
    AX_CUDA(w.largeIds.reserve(ids.size()));
    AX_CUDA(cudaMemcpyAsync(w.largeIds.p, ids.data(), 4ull * ids.size(), cudaMemcpyHostToDevice, w.stream));
    AX_CUDA(cudaStreamSynchronize(w.stream));
    w.nLarge = (uint32_t)ids.size();
    w.gridWidth = T;
    return AXIOM_SUCCESS;
}

int32_t appendPackedBodies(World& w0, const PackedBodies& pk, uint32_t n, const float* sleepTime,
                           const uint32_t* island) {
    World* w = &w0;
    int32_t st;
    std::vector<float4> zero(n, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t s = (pk.info[i] >> 4) & 0xFu, t = pk.info[i] & kInfoTypeMask;
        if (s == AXIOM_SHAPE_PLANE) {
            w->planeIds.push_back(w->n + i);
            w->hostWidth.push_back(-1.0f);
        } else {
            const float wdt = 2.0f * (boundingRadius(s, &pk.shp[i].x) + w->cfg.aabb_margin);
            w->maxWidth = wdt > w->maxWidth ? wdt : w->maxWidth;
            w->hostWidth.push_back(wdt);
        }
        w->nStatic += t == AXIOM_BODY_STATIC;
        w->nDynamic += t == AXIOM_BODY_DYNAMIC || t == kTypeSleeping;
        w->nKinematic += t == AXIOM_BODY_KINEMATIC;
    }
    const uint32_t base = w->n, total = w->n + n;
    if ((st = ensureBodyCapacity(*w, total)) != AXIOM_SUCCESS) return st;
    auto up = [&](DevBuf<float4>& d, const std::vector<float4>& h) {
        return cudaMemcpyAsync(d.p + base, h.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, w->stream);
    };
    AX_CUDA(up(w->pos, pk.pos));
    AX_CUDA(up(w->rot, pk.rot));
    AX_CUDA(cudaMemcpyAsync(w->body.p + base, pk.body.data(), sizeof(SolverBody) * n, cudaMemcpyHostToDevice,
                            w->stream));
    AX_CUDA(up(w->shp, pk.shp));
    AX_CUDA(up(w->mat, pk.mat));
    AX_CUDA(up(w->iloc, pk.iloc));
    AX_CUDA(up(w->iw0, zero));
    AX_CUDA(up(w->iw1, zero));
    AX_CUDA(cudaMemcpyAsync(w->info.p + base, pk.info.data(), 4ull * n, cudaMemcpyHostToDevice, w->stream));
    AX_CUDA(cudaMemcpyAsync(w->filt.p + base, pk.filt.data(), sizeof(uint4) * n, cudaMemcpyHostToDevice,
                            w->stream));
    std::vector<float> st0;
    std::vector<uint32_t> isl, gen0;
    if (w->cfg.allow_sleep) {
        // sleep time 0; a body added asleep is an island of its own until contacts wake it
        st0.assign(n, 0.0f);
        isl.resize(n);
        gen0.assign(n, 0u);
        for (uint32_t i = 0; i < n; ++i) {
            const bool asleep = (pk.info[i] & kInfoTypeMask) == kTypeSleeping;
            isl[i] = island ? island[i] : (asleep ? base + i : kNoIsland);
            if (sleepTime) st0[i] = sleepTime[i];
            w->nSleeping += asleep ? 1u : 0u;
        }
        AX_CUDA(cudaMemcpyAsync(w->sleepTime.p + base, st0.data(), 4ull * n, cudaMemcpyHostToDevice, w->stream));
        AX_CUDA(cudaMemcpyAsync(w->island.p + base, isl.data(), 4ull * n, cudaMemcpyHostToDevice, w->stream));
        AX_CUDA(cudaMemcpyAsync(w->wakeGen.p + base, gen0.data(), 4ull * n, cudaMemcpyHostToDevice, w->stream));
    }
    w->n = total;
    w->nPlanes = (uint32_t)w->planeIds.size();
    if ((st = classifyLarge(*w)) != AXIOM_SUCCESS) return st;
    AX_CUDA(w->planes.reserve(std::max<uint32_t>(w->nPlanes, 1u)));
    if (w->nPlanes)
        AX_CUDA(cudaMemcpyAsync(w->planes.p, w->planeIds.data(), 4ull * w->nPlanes,
                                cudaMemcpyHostToDevice, w->stream));
    // Stage capacities: pairs 16 / body, manifolds 4 / body unless configured.
    const uint64_t pairCap = w->cfg.pair_capacity ? w->cfg.pair_capacity : 16ull * total;
    AX_CUDA(w->pairs.reserve(pairCap));
    AX_CUDA(w->gjkQueue.reserve(w->pairs.cap));
    const uint64_t mCap = w->cfg.contact_capacity ? w->cfg.contact_capacity : 4ull * total;
    if ((st = ensureManifoldCapacity(*w, (uint32_t)std::min<uint64_t>(mCap, 0xFFFFFFF0ull))) != AXIOM_SUCCESS)
        return st;
    if ((st = ensureWarmTable(*w, 0, 1024)) != AXIOM_SUCCESS) return st;
    if ((st = ensureWarmTable(*w, 1, 1024)) != AXIOM_SUCCESS) return st;
    w->wsValid = false;  // body ids of old impulses stay valid, but keep it simple: restart
    w->pairsValid = false;  // the pair and manifold buffers may have been reallocated
    w->lastManifolds = w->lastPoints = 0;
    AX_CUDA(cudaStreamSynchronize(w->stream));  // the host vectors go out of scope
    return AXIOM_SUCCESS;
}

void resetBodies(World& w) {
    w.n = 0;
    w.hulls.clear();
    w.hullPoints.clear();
    w.aabbCount = 0;
    w.nPlanes = 0;
    w.planeIds.clear();
    w.maxWidth = 0.0f;
    w.hostWidth.clear();
    w.nLarge = 0;
    w.gridWidth = 0.0f;
    w.nStatic = w.nDynamic = w.nKinematic = 0;
    w.nSleeping = 0;
    w.lastIslands = 0;
    w.wsValid = false;
    w.pairsValid = false;
    w.lastPairs = w.lastManifolds = w.lastPoints = w.lastColours = w.lastRounds = 0;
    std::memset(&w.last, 0, sizeof(w.last));
}

int32_t reserveWarmTable(World& w, uint32_t slot, uint32_t points) { return ensureWarmTable(w, slot, points); }
uint32_t nextWarmGen(World& w, uint32_t slot) {
    if (++w.wsGen[slot] == 0u) {
        cudaMemsetAsync(w.wsSlots[slot].p, 0, sizeof(WarmSlot) << w.wsLog2[slot], w.stream);
        cudaMemsetAsync(w.wsClaim[slot].p, 0, sizeof(uint32_t) << w.wsLog2[slot], w.stream);
        w.wsGen[slot] = 1u;
    }
    return w.wsGen[slot];
}

}  // namespace axiom_gb300

using namespace axiom_gb300;

extern "C" {

AXIOM_API void axiom_world_config_default(axiom_world_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->gravity[1] = -9.81f;
    c->time_step = 1.0f / 60.0f;
    c->velocity_iterations = 8;
    c->position_iterations = 3;
    c->residual_tolerance = 0.0f;
    c->max_iterations = 200;
    c->baumgarte = 0.2f;
    c->linear_slop = 0.005f;
    c->aabb_margin = 0.0f;
    c->restitution_threshold = 1.0f;
    c->warm_start = AXIOM_WARM_START_PREVIOUS;
    c->warm_start_factor = 1.0f;
    c->device = -1;
    c->allow_sleep = 0;
    c->sleep_linear_threshold = 0.01f;
    c->sleep_angular_threshold = 0.01f;
    c->sleep_time_threshold = 0.5f;
    c->speculative_contacts = 0;
}

AXIOM_API int32_t axiom_world_create(const axiom_world_config* config, void** world) {
    if (!config || !world) return AXIOM_NULL_POINTER;
    *world = nullptr;
    if (!(config->time_step > 0.0f) || config->warm_start > AXIOM_WARM_START_LEARNED ||
        config->temporal_colouring > 1u)
        return AXIOM_INVALID_PARAMETER;
    if (config->allow_sleep && !(config->sleep_time_threshold > 0.0f && config->sleep_linear_threshold >= 0.0f &&
                                 config->sleep_angular_threshold >= 0.0f))
        return AXIOM_INVALID_PARAMETER;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return AXIOM_GPU_OPERATION_FAILED;
    if (config->device >= dev) return AXIOM_INVALID_PARAMETER;
    if (config->device >= 0 && cudaSetDevice(config->device) != cudaSuccess)
        return AXIOM_GPU_OPERATION_FAILED;
    World* w = new (std::nothrow) World();
    if (!w) return AXIOM_OUT_OF_MEMORY;
    w->cfg = *config;
    bool ok = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&w->dcnt, sizeof(DevCounters)) == cudaSuccess &&
              cudaMallocHost(&w->hcnt, sizeof(DevCounters)) == cudaSuccess;
    for (int k = 0; ok && k < 6; ++k) ok = cudaEventCreate(&w->ev[k]) == cudaSuccess;
    if (!ok) {
        axiom_world_destroy(w);
        return AXIOM_GPU_OPERATION_FAILED;
    }
    std::memset(w->hcnt, 0, sizeof(DevCounters));
    *world = w;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_destroy(void* world) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_SUCCESS;
    if (w->stream) cudaStreamSynchronize(w->stream);
    w->body.release();
    DevBuf<float4>* f4[] = {&w->pos, &w->rot, &w->shp, &w->mat, &w->iloc,
                            &w->iw0, &w->iw1, &w->aabbMin, &w->aabbMax, &w->mn, &w->sn};
    for (auto* b : f4) b->release();
    for (int k = 0; k < kMaxPoints; ++k) {
        w->mp[k].release();
        w->sra[k].release();
        w->srb[k].release();
        w->skt[k].release();
        w->slam[k].release();
    }
    w->filt.release();
    w->largeIds.release();
    w->stage.release();
    w->hullVerts.release();
    w->sleepTime.release();
    DevBuf<uint32_t>* u[] = {&w->island, &w->ufParent, &w->islandMin, &w->wakeGen,&w->info, &w->planes, &w->keyA, &w->keyB, &w->valA, &w->valB, &w->hist,
                             &w->work0, &w->mcolour, &w->order, &w->orderInv, &w->bodyDeg,
                             &w->bodySlots, &w->colourChunkNext,
                             &w->manPending};
    for (auto* b : u) b->release();
    w->manRec.release();
    w->warm0.release();
    w->manSucc.release();
    w->nbody.release();
    w->sbox.release();
    w->colourPool.release();
    w->cellTable.release();
    w->pairs.release();
    w->gjkQueue.release();
    w->mhdr.release();
    w->shdr.release();
    w->bodyMask.release();
    for (int k = 0; k < 2; ++k) {
        w->wsSlots[k].release();
        w->wsClaim[k].release();
    }
    for (CachedGraph* g : {&w->warmGraph, &w->sweepGraph})
        if (g->exec) cudaGraphExecDestroy(g->exec);
    w->mlp.release(true);
    w->feat.release();
    w->learnRows.release();
    w->learnRowOf.release();
    for (int k = 0; k < 2; ++k) {
        w->crowdKey[k].release();
        w->crowdVal[k].release();
    }
    w->crowdHist.release();
    w->clusterKey.release();
    w->clusterPos.release();
    for (int k = 0; k < 6; ++k)
        if (w->ev[k]) cudaEventDestroy(w->ev[k]);
    resolveProfile(*w);
    for (cudaEvent_t e : w->prof.pool) cudaEventDestroy(e);
    if (w->dcnt) cudaFree(w->dcnt);
    if (w->hcnt) cudaFreeHost(w->hcnt);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_add_bodies(void* world, const axiom_body_soa* b, uint32_t n,
                                         uint32_t* first_id) {
    World* w = static_cast<World*>(world);
    if (!w || !b) return AXIOM_NULL_POINTER;
    if (first_id) *first_id = w->n;
    if (n == 0) return AXIOM_SUCCESS;
    if ((uint64_t)w->n + n >= (1ull << 30)) return AXIOM_OUT_OF_RANGE;
    int32_t st = validateBodies(b, n, (int64_t)w->hulls.size());
    if (st != AXIOM_SUCCESS) return st;
    PackedBodies pk;
    packBodies(b, 0, n, &pk, w->cfg.allow_sleep != 0, &w->hulls);
    return appendPackedBodies(*w, pk, n, nullptr, nullptr);
}

AXIOM_API int32_t axiom_world_check_bodies(void* world, const axiom_body_soa* b, uint32_t n) {
    World* w = static_cast<World*>(world);
    if (!w || !b) return AXIOM_NULL_POINTER;
    if (n == 0) return AXIOM_SUCCESS;
    if ((uint64_t)w->n + n >= (1ull << 30)) return AXIOM_OUT_OF_RANGE;
    return validateBodies(b, n, (int64_t)w->hulls.size());
}

AXIOM_API int32_t axiom_world_add_convex_hull(void* world, const float* points, uint32_t count, uint32_t* hull_id) {
    World* w = static_cast<World*>(world);
    if (!w || !points) return AXIOM_NULL_POINTER;
    uint32_t id = 0;
    const int32_t st = appendHull(*w, points, count, 4, &id);
    if (st == AXIOM_SUCCESS && hull_id) *hull_id = id;
    return st;
}

AXIOM_API int32_t axiom_world_add_triangle_mesh(void* world, const float* vertices, uint32_t vertex_count,
                                                const uint32_t* triangles, uint32_t triangle_count, float friction,
                                                float restitution, uint32_t* first_id) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    if (first_id) *first_id = w->n;
    if (triangle_count == 0) return AXIOM_SUCCESS;
    if (!vertices || !triangles) return AXIOM_NULL_POINTER;
    std::vector<float> centre(3ull * triangle_count), pts(9ull * triangle_count);
    const int32_t chk = checkMesh(vertices, vertex_count, triangles, triangle_count, centre.data(), pts.data());
    if (chk != AXIOM_SUCCESS) return chk;
    const uint32_t firstHull = (uint32_t)w->hulls.size();
    for (uint32_t t = 0; t < triangle_count; ++t) {
        uint32_t id;
        const int32_t st = appendHull(*w, pts.data() + 9ull * t, 3, 3, &id);
        if (st != AXIOM_SUCCESS) return st;
    }
    std::vector<uint32_t> type(triangle_count, AXIOM_BODY_STATIC), shape(triangle_count, AXIOM_SHAPE_MESH), hull(triangle_count);
    std::vector<float> ext(3ull * triangle_count, 0.0f), fr(triangle_count, friction), re(triangle_count, restitution);
    for (uint32_t t = 0; t < triangle_count; ++t) hull[t] = firstHull + t;
    axiom_body_soa soa{};
    soa.type = type.data();
    soa.shape = shape.data();
    soa.position = centre.data();
    soa.shape_extents = ext.data();
    soa.friction = fr.data();
    soa.restitution = re.data();
    soa.convex_hull = hull.data();
    return axiom_world_add_bodies(world, &soa, triangle_count, first_id);
}

AXIOM_API int32_t axiom_world_body_count(void* world, uint32_t* n) {
    World* w = static_cast<World*>(world);
    if (!w || !n) return AXIOM_NULL_POINTER;
    *n = w->n;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_step(void* world, float dt, axiom_step_stats* stats) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    try {
        return step(*w, dt, stats);
    } catch (...) {
        return AXIOM_GPU_OPERATION_FAILED;
    }
}

AXIOM_API int32_t axiom_world_read_state(void* world, float* position, float* rotation,
                                         float* linear_velocity, float* angular_velocity) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    if (w->n == 0) return AXIOM_SUCCESS;
    const uint32_t n = w->n;
    // one kernel writes every requested array to its staging region, then the copies
    float* host[4] = {position, rotation, linear_velocity, angular_velocity};
    const uint32_t width[4] = {3, 4, 3, 3};
    float* dev[4] = {nullptr, nullptr, nullptr, nullptr};
    float* stage = nullptr;
    size_t off = 0;
    for (int k = 0; k < 4; ++k) {
        if (!host[k]) continue;
        if (!stage && !(stage = stateStaging(*w))) return AXIOM_OUT_OF_MEMORY;
        dev[k] = stage + off;
        off += (size_t)width[k] * n;
    }
    kStateOut<<<gridFor(n, 256), 256, 0, w->stream>>>(n, StateIO{dev[0], dev[1], dev[2], dev[3]}, w->pos.p, w->rot.p,
                                                      w->body.p);
    AX_CUDA(cudaGetLastError());
    for (int k = 0; k < 4; ++k)
        if (host[k]) AX_CUDA(cudaMemcpyAsync(host[k], dev[k], 4ull * width[k] * n, cudaMemcpyDeviceToHost, w->stream));
    AX_CUDA(cudaStreamSynchronize(w->stream));
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_write_state(void* world, const float* position, const float* rotation,
                                          const float* linear_velocity, const float* angular_velocity) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    if (w->n == 0) return AXIOM_SUCCESS;
    const uint32_t n = w->n;
    const float* host[4] = {position, rotation, linear_velocity, angular_velocity};
    const uint32_t width[4] = {3, 4, 3, 3};
    float* dev[4] = {nullptr, nullptr, nullptr, nullptr};
    float* stage = nullptr;
    size_t off = 0;
    for (int k = 0; k < 4; ++k) {
        if (!host[k]) continue;
        if (!stage && !(stage = stateStaging(*w))) return AXIOM_OUT_OF_MEMORY;
        dev[k] = stage + off;
        off += (size_t)width[k] * n;
        AX_CUDA(cudaMemcpyAsync(dev[k], host[k], 4ull * width[k] * n, cudaMemcpyHostToDevice, w->stream));
    }
    kStateIn<<<gridFor(n, 256), 256, 0, w->stream>>>(n, StateIO{dev[0], dev[1], dev[2], dev[3]}, w->pos.p, w->rot.p,
                                                     w->body.p);
    AX_CUDA(cudaGetLastError());
    AX_CUDA(cudaStreamSynchronize(w->stream));
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_sleep(void* world, uint8_t* sleeping, float* sleep_time, uint32_t* island) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    const uint32_t n = w->n;
    if (n == 0) return AXIOM_SUCCESS;
    if (!w->cfg.allow_sleep) {
        if (sleeping) std::memset(sleeping, 0, n);
        if (sleep_time) std::fill(sleep_time, sleep_time + n, 0.0f);
        if (island) std::fill(island, island + n, kNoIsland);
        return AXIOM_SUCCESS;
    }
    std::vector<uint32_t> info(n), isl(n);
    std::vector<float> st(n);
    AX_CUDA(cudaMemcpyAsync(info.data(), w->info.p, 4ull * n, cudaMemcpyDeviceToHost, w->stream));
    AX_CUDA(cudaMemcpyAsync(isl.data(), w->island.p, 4ull * n, cudaMemcpyDeviceToHost, w->stream));
    AX_CUDA(cudaMemcpyAsync(st.data(), w->sleepTime.p, 4ull * n, cudaMemcpyDeviceToHost, w->stream));
    AX_CUDA(cudaStreamSynchronize(w->stream));
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t t = info[i] & kInfoTypeMask;
        const bool dyn = t == AXIOM_BODY_DYNAMIC || t == kTypeSleeping;
        if (sleeping) sleeping[i] = t == kTypeSleeping ? 1u : 0u;
        if (sleep_time) sleep_time[i] = dyn ? st[i] : 0.0f;
        if (island) island[i] = dyn ? isl[i] : kNoIsland;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_sleeping(void* world, const uint32_t* ids, uint32_t n, int32_t sleeping) {
    World* w = static_cast<World*>(world);
    if (!w || (n && !ids)) return AXIOM_NULL_POINTER;
    for (uint32_t k = 0; k < n; ++k)
        if (ids[k] >= w->n) return AXIOM_OUT_OF_RANGE;
    if (sleeping && !w->cfg.allow_sleep) return AXIOM_INVALID_PARAMETER;
    if (n == 0 || !w->cfg.allow_sleep) return AXIOM_SUCCESS;  // nothing sleeps: waking is a no-op
    // ids go through the sort scratch (>= n words once bodies exist), grown if needed
    if (w->keyB.cap < n) AX_CUDA(w->keyB.reserve(n));
    AX_CUDA(cudaMemcpyAsync(w->keyB.p, ids, 4ull * n, cudaMemcpyHostToDevice, w->stream));
    launchSetSleeping(*w, w->keyB.p, n, sleeping != 0);
    launchCountSleeping(*w);
    AX_CUDA(cudaGetLastError());
    AX_CUDA(cudaMemcpyAsync(&w->hcnt->sleeping, &w->dcnt->sleeping, 4, cudaMemcpyDeviceToHost, w->stream));
    AX_CUDA(cudaStreamSynchronize(w->stream));
    w->nSleeping = w->hcnt->sleeping;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_aabbs(void* world, float* aabb_min, float* aabb_max) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    if (w->n == 0) return AXIOM_SUCCESS;
    const uint32_t n = w->n;
    if (w->keyB.cap < 4ull * n) AX_CUDA(w->keyB.reserve(4ull * n));
    float* stage = reinterpret_cast<float*>(w->keyB.p);
    auto pack = [&](const DevBuf<float4>& src, float* dst) -> cudaError_t {
        kPack3<<<gridFor(n, 256), 256, 0, w->stream>>>(n, src.p, 1, stage);
        return cudaMemcpyAsync(dst, stage, 12ull * n, cudaMemcpyDeviceToHost, w->stream);
    };
    if (aabb_min) AX_CUDA(pack(w->aabbMin, aabb_min));
    if (aabb_max) AX_CUDA(pack(w->aabbMax, aabb_max));
    AX_CUDA(cudaStreamSynchronize(w->stream));
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_pairs(void* world, uint32_t* pairs, uint32_t capacity, uint32_t* count) {
    World* w = static_cast<World*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    *count = w->pairsValid ? w->lastPairs : 0u;  // none since bodies were added or loaded
    const uint32_t k = std::min(*count, capacity);
    if (pairs && k) {
        AX_CUDA(cudaMemcpyAsync(pairs, w->pairs.p, 8ull * k, cudaMemcpyDeviceToHost, w->stream));
        AX_CUDA(cudaStreamSynchronize(w->stream));
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_contacts(void* world, axiom_contact_point* out, uint32_t capacity,
                                            uint32_t* count) {
    World* w = static_cast<World*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    const uint32_t nM = w->lastManifolds;
    *count = w->lastPoints;
    if (!out || nM == 0) return AXIOM_SUCCESS;
    std::vector<uint4> mh(nM), sh(nM);
    std::vector<float4> mn(nM);
    std::vector<std::vector<float4>> mp(kMaxPoints, std::vector<float4>(nM)),
        lam(kMaxPoints, std::vector<float4>(nM));
    std::vector<uint32_t> order(nM), colour(nM);
    cudaStream_t s = w->stream;
    AX_CUDA(cudaMemcpyAsync(mh.data(), w->mhdr.p, 16ull * nM, cudaMemcpyDeviceToHost, s));
    AX_CUDA(cudaMemcpyAsync(sh.data(), w->shdr.p, 16ull * nM, cudaMemcpyDeviceToHost, s));
    AX_CUDA(cudaMemcpyAsync(mn.data(), w->mn.p, 16ull * nM, cudaMemcpyDeviceToHost, s));
    AX_CUDA(cudaMemcpyAsync(order.data(), w->order.p, 4ull * nM, cudaMemcpyDeviceToHost, s));
    AX_CUDA(cudaMemcpyAsync(colour.data(), w->mcolour.p, 4ull * nM, cudaMemcpyDeviceToHost, s));
    for (int k = 0; k < kMaxPoints; ++k) {
        AX_CUDA(cudaMemcpyAsync(mp[k].data(), w->mp[k].p, 16ull * nM, cudaMemcpyDeviceToHost, s));
        AX_CUDA(cudaMemcpyAsync(lam[k].data(), w->slam[k].p, 16ull * nM, cudaMemcpyDeviceToHost, s));
    }
    AX_CUDA(cudaStreamSynchronize(s));
    uint32_t q = 0;
    for (uint32_t sIdx = 0; sIdx < nM; ++sIdx) {
        const uint32_t m = order[sIdx];
        const uint4 h = mh[m];
        for (uint32_t k = 0; k < h.z && k < (uint32_t)kMaxPoints; ++k, ++q) {
            if (q >= capacity) continue;
            axiom_contact_point& o = out[q];
            o.body_a = h.x;
            o.body_b = h.y;
            o.position[0] = mp[k][m].x;
            o.position[1] = mp[k][m].y;
            o.position[2] = mp[k][m].z;
            o.penetration_depth = mp[k][m].w;
            o.normal[0] = mn[m].x;
            o.normal[1] = mn[m].y;
            o.normal[2] = mn[m].z;
            o.impulse[0] = lam[k][sIdx].x;
            o.impulse[1] = lam[k][sIdx].y;
            o.impulse[2] = lam[k][sIdx].z;
            o.colour = colour[m];
            o.point_index = k;
        }
    }
    *count = q;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_warm_start_model(void* world, const float* params, uint32_t count) {
    World* w = static_cast<World*>(world);
    if (!w || !params) return AXIOM_NULL_POINTER;
    if (count != AXIOM_MLP_PARAM_COUNT) return AXIOM_INVALID_PARAMETER;
    if (!w->mlpReady) {
        AX_CUDA(w->mlp.init());
        w->mlpReady = true;
    }
    AX_CUDA(w->mlp.setParams(params, w->stream));
    AX_CUDA(cudaStreamSynchronize(w->stream));
    w->mlpLoaded = true;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_recording(void* world, int32_t enable) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    w->recording = enable != 0;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_samples(void* world, float* features, float* targets, uint32_t* keys,
                                           uint32_t capacity, uint32_t* count) {
    World* w = static_cast<World*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    const uint32_t nM = w->lastManifolds;
    *count = 0;
    if (!w->needFeatures || nM == 0) return AXIOM_SUCCESS;
    std::vector<float> f(64ull * nM);
    std::vector<uint4> sh(nM);
    std::vector<std::vector<float4>> lam(kMaxPoints, std::vector<float4>(nM));
    cudaStream_t s = w->stream;
    AX_CUDA(cudaMemcpyAsync(f.data(), w->feat.p, 256ull * nM, cudaMemcpyDeviceToHost, s));
    AX_CUDA(cudaMemcpyAsync(sh.data(), w->shdr.p, 16ull * nM, cudaMemcpyDeviceToHost, s));
    for (int k = 0; k < kMaxPoints; ++k)
        AX_CUDA(cudaMemcpyAsync(lam[k].data(), w->slam[k].p, 16ull * nM, cudaMemcpyDeviceToHost, s));
    AX_CUDA(cudaStreamSynchronize(s));
    uint32_t q = 0;
    for (uint32_t si = 0; si < nM; ++si)
        for (uint32_t k = 0; k < sh[si].z && k < (uint32_t)kMaxPoints; ++k, ++q) {
            if (q >= capacity) continue;
            const float* row = &f[((size_t)k * nM + si) * 16u];
            const float inv = row[14] > 0.0f ? 1.0f / row[14] : 0.0f;
            if (features) std::memcpy(features + 14ull * q, row, 14 * 4);
            if (targets) {  // correction from the previous-step impulse, in impulse units
                targets[3ull * q] = lam[k][si].x * inv - row[9];
                targets[3ull * q + 1] = lam[k][si].y * inv - row[10];
                targets[3ull * q + 2] = lam[k][si].z * inv - row[11];
            }
            if (keys) {
                keys[3ull * q] = sh[si].x;
                keys[3ull * q + 1] = sh[si].y;
                keys[3ull * q + 2] = k;
            }
        }
    *count = q;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_profiling(void* world, int32_t enable) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    w->prof.enabled = enable != 0;
    w->prof.mask = ~0u;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_profiling_groups(void* world, uint32_t group_mask) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    w->prof.enabled = group_mask != 0u;
    w->prof.mask = group_mask;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_reset_profile(void* world) {
    World* w = static_cast<World*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    resolveProfile(*w);
    for (int g = 0; g < KG_COUNT; ++g) {
        w->prof.launches[g] = 0;
        w->prof.ranges[g] = 0;
        w->prof.ms[g] = 0.0;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_profile(void* world, axiom_kernel_profile* out, uint32_t capacity,
                                           uint32_t* count) {
    World* w = static_cast<World*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    *count = KG_COUNT;
    for (uint32_t g = 0; g < (uint32_t)KG_COUNT && out && g < capacity; ++g) {
        std::memset(out[g].name, 0, sizeof(out[g].name));
        std::strncpy(out[g].name, kKernelGroupNames[g], sizeof(out[g].name) - 1);
        out[g].launches = w->prof.launches[g];
        out[g].ranges = w->prof.ranges[g];
        out[g].total_ms = w->prof.ms[g];
    }
    return AXIOM_SUCCESS;
}

AXIOM_API const char* axiom_version(void) { return "axiom-gb300 0.1 (sm_103a)"; }

}  // extern "C"
