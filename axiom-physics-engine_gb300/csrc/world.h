// world.h — device-resident state of one world and the launchers of its kernels.
//
// HBM layout (all arrays are indexed by body id unless noted; float4 so that every
// per-body field is one 16-byte load):
//   pos   (x, y, z, 0)                rot   (qx, qy, qz, qw)
//   vel   (vx, vy, vz, invMass)       ang   (wx, wy, wz, invI_iso or -1 if anisotropic)
//   shp   (e0, e1, e2, 0)             mat   (friction, restitution, linDamp, angDamp)
//   iloc  (1/Ix, 1/Iy, 1/Iz, 0)       iw0/iw1  world inverse inertia (xx,yy,zz,xy),(xz,yz,-,-)
//   info  type | shape << 4           (uint32)
// Broadphase (sorted order): skey (Morton cell key), sbox (one 32-byte record: min.xyz
//   with the id bits, max.xyz with the sweep flag bits).  Planes get key 0xFFFFFFFF and
//   sort last.
// Manifolds (narrowphase order): mhdr (a, b, npts, dyn: bit0 a, bit1 b dynamic), mn (n.xyz, 0), mp[k] (p.xyz, depth)
//   for point slot k = 0..3 (slot-major, so single-point manifolds read one dense array).
// Solver (colour order): shdr (a, b, npts, flags), sn (n.xyz, mu), per slot k:
//   sra[k] (rA.xyz, kn), srb[k] (rB.xyz, bias), skt[k] (kt1, kt2), slam[k] (λn, λt1, λt2, 0).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/axiom_c.h"
#include "mlp.h"
#include "shapes.h"

namespace axiom_gb300 {

constexpr uint32_t kInfoTypeMask = 0xFu;
constexpr uint32_t kHdrDynA = 1u, kHdrDynB = 2u;  // mhdr.w bits written by the narrowphase
constexpr uint32_t kInfoFiltered = 1u << 8;  // info: the body's collision filter is not the default
constexpr uint32_t kInfoNoSleep = 1u << 9;   // info: SleepInfo::allowSleep is false for this body
// info type of a dynamic body while it sleeps: every "is it dynamic?" test then treats it
// like an immovable body (no gravity, no integration, no solver writes, no contacts with
// static or other sleeping bodies) until it wakes and takes AXIOM_BODY_DYNAMIC back.
constexpr uint32_t kTypeSleeping = 3u;
// Sweep flag bits of a sorted box (SortedBox::mx.w): 1 awake dynamic, 2 non-default
// filter, 4 sleeping, 8 kinematic with a non-zero velocity (wakes sleeping bodies it
// touches), 16 the next sorted box is in the same cell.
constexpr uint32_t kSweepDynamic = 1u, kSweepFiltered = 2u, kSweepSleeping = 4u, kSweepMover = 8u,
                   kSweepRunNext = 16u;

// One slot of a warm-start table (open addressing on warmKey): the key, the generation
// that wrote it, the tag (on point 0 of a manifold: 1 + the manifold's colour, 0 for none)
// and the impulses, in one 32-byte sector.  A slot whose generation is not the table's
// current one is empty, so a table is reused without clearing.  Inserters claim a slot in
// a separate array of generations (4 bytes per slot, so the claims stay in L2) and then
// write the whole sector, which needs no fill from DRAM.
struct alignas(32) WarmSlot {
    unsigned long long key;
    uint32_t gen;
    uint32_t tag;
    float4 val;
};

// A body's AABB in the broadphase's sorted order: one 32-byte sector per candidate test.
struct alignas(32) SortedBox {
    float4 mn;  // min.xyz, id bits
    float4 mx;  // max.xyz, sweep flag bits
};
constexpr uint32_t kNoIsland = 0xFFFFFFFFu;
constexpr int kMaxWakePasses = 8;  // wake -> redo-contacts passes in one step

#ifdef __CUDACC__
// Collision filter of two bodies, each (category, mask, group as int32, 0).
__host__ __device__ inline bool filterPass(uint4 fa, uint4 fb) {
    const int32_t ga = (int32_t)fa.z, gb = (int32_t)fb.z;
    if (ga == gb && ga != 0) return ga > 0;
    return (fa.y & fb.x) != 0u && (fa.x & fb.y) != 0u;
}
#endif
constexpr uint32_t kEmptyKey32 = 0xFFFFFFFFu;
constexpr unsigned long long kEmpty64 = 0xFFFFFFFFFFFFFFFFull;
constexpr int kMaxPoints = 4;
constexpr int kMaxColours = 64;
constexpr uint32_t kMaxLarge = 64;  // bodies at most that leave the grid for their size
// A manifold at a dynamic body with more than kCrowdDegree manifolds is "crowded": it takes
// no colour (kCrowdColour) and is solved in one serial batch after the colours, in
// descending priority.  Every other manifold then finds a free colour: its two bodies
// hold at most 2 x (kCrowdDegree - 1) = 62 other manifolds.
constexpr uint32_t kCrowdDegree = 32;
constexpr uint32_t kCrowdColour = kMaxColours;
constexpr uint32_t kRoundsFromCounters = 0xFFFFFFFFu;  // World::lastRounds: read dcnt->colourRounds

// A convex hull in the world's vertex pool (axiom_world_add_convex_hull).
struct HullInfo {
    uint32_t offset, count;  // first vertex in the pool, vertex count
    float radius;            // max |vertex|: bounding sphere about the body origin
    float halfExtents[3];    // half the body-frame bounding box (mass properties)
};

// Velocity state of one body as the solver reads and writes it: both halves share one
// 32-byte sector, so a body gather or scatter touches a single sector.
struct __align__(32) SolverBody {
    float4 v;  // (vx, vy, vz, invMass)
    float4 w;  // (wx, wy, wz, invI_iso or -1 if anisotropic)
};

// Grow-only device buffer.  Allocation happens only at world creation, when bodies are
// added, or when a capacity check after a stage finds it too small.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap) return cudaSuccess;
        size_t want = cap ? cap : 1;
        while (want < n) want *= 2;
        T* q = nullptr;
        cudaError_t e = cudaMalloc(&q, want * sizeof(T));
        if (e != cudaSuccess) return e;
        if (p) cudaFree(p);
        p = q;
        cap = want;
        return cudaSuccess;
    }
    // keeps contents
    cudaError_t grow(size_t n, cudaStream_t s) {
        if (n <= cap) return cudaSuccess;
        size_t want = cap ? cap : 1;
        while (want < n) want *= 2;
        T* q = nullptr;
        cudaError_t e = cudaMalloc(&q, want * sizeof(T));
        if (e != cudaSuccess) return e;
        if (p) {
            cudaMemcpyAsync(q, p, cap * sizeof(T), cudaMemcpyDeviceToDevice, s);
            cudaStreamSynchronize(s);
            cudaFree(p);
        }
        p = q;
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// What the pair narrowphase gathers per body, in one 32-byte sector: position (w: the
// speculative sweep length) and shape extents with the info word (w).  Written with the
// AABBs at the start of a step; the wake pass refreshes the info word.
struct alignas(32) NarrowBody {
    float4 p;
    float4 s;
};

// An instantiated CUDA graph and the launch parameters it was captured with.
struct CachedGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> key;
};

// Counters the kernels update on the device; copied to the host once per stage.
struct DevCounters {
    uint32_t pairs;
    uint32_t manifolds;
    uint32_t points;
    uint32_t colourOverflow; // a manifold found no free colour among 64
    uint32_t maxColour;      // highest colour + 1
    uint32_t converged;      // tolerance mode: residual reached
    uint32_t iterations;     // PGS sweeps performed
    uint32_t errorFlags;     // bounds / invariant violations seen by kernels
    uint32_t maxDeltaBits;   // current sweep: max |dλ| (float bits, non-negative)
    uint32_t maxLambdaBits;  // current sweep: max |λ|
    float residual;          // residual of the last sweep
    uint32_t colourStart[kMaxColours + 2];  // colour c at [c, c + 1); crowded at [64, 65)
    uint32_t gjkPairs;       // box-box / box-capsule pairs queued for GJK + EPA
    uint32_t sweepDone;      // blocks of the closing colour launch that finished (ticket)
    uint32_t mixedPairs;     // analytic pairs other than sphere-sphere, queued for kPairsMixed
    uint32_t colourRounds;   // dependency depth of the colouring (Jones-Plassmann rounds)
    uint32_t colourChunks;   // colouring queue chunks taken from the pool
    uint32_t woken;          // sleeping bodies woken by this wake pass
    uint32_t islands;        // islands of the awake dynamic bodies (end of step)
    uint32_t sleeping;       // bodies asleep at the end of the step
    uint32_t sweptWidthBits; // speculative contacts: widest swept AABB of the step (float bits)
    uint32_t learnRows;      // learned warm start: rows listed for the network (contact points)
    uint32_t gjkFailures;    // pairs whose GJK ran out of iterations (treated as separated)
    uint32_t epaFailures;    // pairs whose EPA stopped at a cap before its tolerance
    uint32_t crowdSeen;      // colouring: some dynamic body has more than kCrowdDegree manifolds
    uint32_t colourConflict; // temporal colouring: two manifolds at a body share a previous colour
    uint32_t planeQueue;     // dynamic bodies other than spheres queued for their plane contacts
    uint32_t clusterMax[6];  // cluster solve: sweep maxima (|dλ|, |λ| float bits), three rotating pairs
};

struct StepParams {
    float dt, invDt, hdt;
    float gx, gy, gz;
    float biasCoeff, slop, margin, restThreshold;
    float invCell;
    float warmFactor;
    float tolerance;
    float gdt;  // |g| * dt: the velocity unit of the warm-start features
    uint32_t n;          // bodies
    uint32_t nPlanes;
    uint32_t warmStart;
    // sleeping
    float sleepLin2, sleepAng2;  // squared thresholds
    float sleepTime;             // island sleep time threshold
    float cellWidth;             // widest unswept AABB (the grid cell before sweeping)
    uint32_t spec;               // speculative contacts: swept AABBs, sweep length in pos.w
};

// Kernel groups timed by the optional profiler (axiom_world_set_profiling).
enum KernelGroup {
    KG_INTEGRATE_VELOCITIES = 0,
    KG_RADIX_SORT,
    KG_BROADPHASE_GATHER,
    KG_BROADPHASE_SWEEP,
    KG_NARROWPHASE,
    KG_COLOURING,
    KG_SOLVER_PREPARE,
    KG_WARM_START_APPLY,
    KG_PGS_COLOUR,
    KG_STORE_IMPULSES,
    KG_INTEGRATE_POSITIONS,
    KG_SLEEP,  // wake passes and the island / sleep pass (allow_sleep only)
    KG_COUNT
};
extern const char* const kKernelGroupNames[KG_COUNT];

struct World;

// Launch counts (always) and CUDA-event durations (when enabled) per kernel group.  A
// range brackets one or more launches of one group on the world's stream.
struct Profiler {
    bool enabled = false;
    uint32_t mask = ~0u;  // kernel groups timed while enabled (bit g = group g)
    uint64_t launches[KG_COUNT] = {};
    uint64_t ranges[KG_COUNT] = {};
    double ms[KG_COUNT] = {};
    std::vector<cudaEvent_t> pool;
    struct Pending {
        int group;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
};

struct ProfRange {
    World* w;
    int group;
    cudaEvent_t a = nullptr;
    ProfRange(World& world, int g);
    ~ProfRange();
};

struct World {
    axiom_world_config cfg{};
    Profiler prof;
    cudaStream_t stream = nullptr;
    uint32_t n = 0;
    float maxWidth = 0.0f;  // widest AABB (2 * (bounding radius + margin)) over non-plane bodies
    // Size disparity: bodies far wider than the rest ("large": see classifyLarge in
    // world.cu) stay out of the grid, whose cells then fit the widest other body, and are
    // tested against every body instead.
    std::vector<float> hostWidth;  // per body: 2 * (bounding radius + margin); -1 for planes
    DevBuf<uint32_t> largeIds;     // the large bodies, ascending id
    uint32_t nLarge = 0;
    float gridWidth = 0.0f;        // widest non-large body (the grid cell is 1.0625 x this)
    uint32_t nPlanes = 0;
    uint32_t nStatic = 0, nDynamic = 0, nKinematic = 0;
    std::vector<uint32_t> planeIds;

    // bodies
    DevBuf<float4> pos, rot, shp, mat, iloc, iw0, iw1;
    DevBuf<SolverBody> body;  // (v, invMass), (ω, invI_iso) in one 32-byte record
    DevBuf<uint32_t> info;
    DevBuf<uint4> filt;  // collision filter (category, mask, group, 0); read only for filtered bodies
    DevBuf<float4> aabbMin, aabbMax;
    DevBuf<NarrowBody> nbody;             // per-body narrowphase record (see NarrowBody)
    DevBuf<uint32_t> planes;
    // convex hulls: body-frame vertices (x, y, z, 0) of every hull, back to back
    std::vector<HullInfo> hulls;
    std::vector<float> hullPoints;  // host copy, 3 floats per vertex (snapshots)
    DevBuf<float4> hullVerts;
    // sleeping and islands (allow_sleep): per body
    DevBuf<float> sleepTime;      // seconds below the sleep thresholds
    DevBuf<uint32_t> island;      // island label (lowest body id of the island)
    DevBuf<uint32_t> ufParent;    // union-find forest of the island pass
    DevBuf<uint32_t> islandMin;   // per island root: min sleep time (float bits)
    DevBuf<uint32_t> wakeGen;     // per island label: generation of the wake pass that marked it
    uint32_t wakeGeneration = 0;
    uint32_t nSleeping = 0;       // bodies asleep after the last step / set_sleeping
    uint32_t lastIslands = 0;
    // broadphase
    DevBuf<uint32_t> keyA, keyB, valA, valB, hist;
    DevBuf<SortedBox> sbox;
    DevBuf<unsigned long long> cellTable;
    uint32_t cellTableLog2 = 0;
    DevBuf<uint2> pairs;
    DevBuf<uint2> gjkQueue;  // pairs.cap entries: GJK/EPA pairs from the front, other analytic
                             // non-sphere pairs from the back
    // narrowphase
    DevBuf<uint4> mhdr;
    DevBuf<float4> mn;
    DevBuf<float4> mp[kMaxPoints];
    // colouring
    DevBuf<unsigned long long> bodyMask;  // colours taken at each body
    DevBuf<uint32_t> bodyDeg, bodySlots;  // manifolds per dynamic body, 64-slot lists
    DevBuf<uint4> manRec;                 // colouring record per manifold: priority, previous colour, flags
    DevBuf<float4> warm0;                 // point 0's previous impulses per manifold (temporal colouring)
    bool warm0Valid = false;              // warm0 holds this step's (the colouring probed the table)
    DevBuf<uint2> manSucc;                // successor in the chain of body a / body b
    DevBuf<uint32_t> manPending;          // chain predecessors not yet coloured
    DevBuf<uint32_t> work0;               // colouring seeds
    DevBuf<uint2> colourPool;             // colouring queue chunks (manifold, level)
    DevBuf<uint32_t> colourChunkNext;     // chunk links of the colouring queues
    DevBuf<uint32_t> mcolour, order;
    DevBuf<uint32_t> orderInv;            // position in colour order of each manifold
    // solver
    DevBuf<uint4> shdr;
    DevBuf<float4> sn;
    DevBuf<float4> sra[kMaxPoints], srb[kMaxPoints], slam[kMaxPoints];
    DevBuf<float2> skt[kMaxPoints];
    // warm-start tables (previous step / this step)
    DevBuf<WarmSlot> wsSlots[2];
    DevBuf<uint32_t> wsClaim[2];  // per slot: the generation that claimed it
    uint32_t wsLog2[2] = {0, 0};
    uint32_t wsGen[2] = {0, 0};  // generation of the entries each table holds (0: none yet)
    uint32_t wsCur = 0;
    bool wsValid = false;
    // learned warm start
    MlpState mlp;             // network weights and inference buffers
    bool mlpReady = false;    // mlp.init() done
    bool mlpLoaded = false;   // parameters set
    bool recording = false;   // keep features of every step (training samples)
    bool needFeatures = false;
    DevBuf<float> feat;       // [4 * manifold capacity][16]: features, impulse scale, valid
    DevBuf<uint32_t> learnRows, learnRowOf;  // network rows (contact points) <-> slot * nM + s
    DevBuf<uint32_t> crowdKey[2], crowdVal[2], crowdHist;  // priority sort of the crowded batch
    uint32_t lastCrowded = 0;  // crowded manifolds of the last colouring
    bool smallSolveReady = false;  // the small-world solve's shared-memory opt-in is set
    int clusterCtas = -1;          // CTAs of the cluster solve's cluster (0: unavailable; -1: not probed)
    DevBuf<unsigned long long> clusterKey;  // cluster solve: crowded-batch priority sort scratch
    DevBuf<uint32_t> clusterPos;

    DevBuf<unsigned char> stage;   // snapshot / debug-feed staging (grown on first use)
    uint32_t aabbCount = 0;        // bodies whose AABB the last step computed

    unsigned solveGrid = 0;        // one resident wave of the PGS colour kernel (set on first use)
    unsigned solveGridHoist = 0;   // the same for its hoisted-rows form (one CTA per SM)
    bool hoistRows = false;        // this step's manifolds include multi-point ones
    CachedGraph warmGraph, sweepGraph;  // the solve's colour launches, captured per colour count
    bool graphsOff = false;        // capture failed once: launch directly
    unsigned colourResident = 0;   // resident CTAs of the colouring dataflow kernel
    DevCounters* dcnt = nullptr;   // device
    DevCounters* hcnt = nullptr;   // pinned host mirror
    cudaEvent_t ev[6] = {};

    // last step
    axiom_step_stats last{};
    uint32_t lastPairs = 0, lastManifolds = 0, lastPoints = 0, lastColours = 0;
    uint32_t lastRounds = 0;  // colouring rounds of the last step
    bool pairsValid = false;  // the pair list belongs to the current bodies (a step ran since the last add)
};

// ---- host-side body management (world.cu) ----
struct PackedBodies;
// Appends n packed bodies (ids w.n .. w.n+n-1).  sleepTime / island (may be NULL) give
// the sleep state of each; by default 0 and "own island if added asleep".
int32_t appendPackedBodies(World& w, const PackedBodies& pk, uint32_t n, const float* sleepTime,
                           const uint32_t* island);
void resetBodies(World& w);  // forgets every body and hull; device buffers are kept for reuse
// Bounding radius and box of a hull of count points (minCount..AXIOM_CONVEX_MAX_VERTICES,
// finite): 4 for convex bodies, 3 for mesh triangles.
bool makeHullInfo(const float* points, uint32_t count, uint32_t offset, HullInfo* h, uint32_t minCount = 4);
// Appends a hull to the pool (host copy and device); *id receives its index.
int32_t appendHull(World& w, const float* points, uint32_t count, uint32_t minCount, uint32_t* id);
// Validates a triangle mesh; per triangle its centroid [3] and its points about it [9].
int32_t checkMesh(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nt, float* centre, float* pts);
int32_t reserveWarmTable(World& w, uint32_t slot, uint32_t points);
// The generation the next fill of warm-start table `slot` writes (clears the table when the
// counter wraps, so that no old slot can look current).
uint32_t nextWarmGen(World& w, uint32_t slot);

// ---- kernel launchers (one .cu file each stage) ----
// integrate.cu
void launchIntegrateVelocities(World& w, const StepParams& sp);
void launchIntegratePositions(World& w, const StepParams& sp);
// sort.cu
bool radixSort(cudaStream_t s, uint32_t* kA, uint32_t* vA, uint32_t* kB, uint32_t* vB,
               uint32_t* hist, uint32_t n, uint32_t passes);
void radixSortPairs(World& w, uint32_t n);  // sorts (keyA, valA) in place through keyB/valB
void groupByColour(cudaStream_t s, const uint32_t* colour, uint32_t* order, uint32_t* inv, uint32_t* hist,
                   uint32_t n, DevCounters* cnt);
uint32_t radixHistWords(uint32_t n);
// broadphase.cu
void launchBroadphaseGather(World& w, uint32_t nSorted);
void launchBroadphase(World& w, const StepParams& sp, uint32_t nSorted);
// Large bodies: their cell keys set empty (after the keys are written, before the sort),
// and their pairs with every other body (after the sweep, same pair list and counter).
void launchMarkLarge(World& w);
void launchLargePairs(World& w);
void launchSweepOnBuffers(cudaStream_t s, uint32_t nSorted, const uint32_t* skey, const SortedBox* sbox,
                          const unsigned long long* table, uint32_t log2T,
                          uint2* pairs, uint32_t cap, DevCounters* cnt);
// narrowphase.cu
void launchNarrowphase(World& w, const StepParams& sp, uint32_t expectedPairs);
// sleep.cu
void launchWake(World& w, const StepParams& sp, uint32_t nManifolds);  // counts woken bodies in dcnt->woken
void launchIslands(World& w, const StepParams& sp, uint32_t nManifolds);
void launchSetSleeping(World& w, const uint32_t* ids, uint32_t n, bool sleeping);  // ids: device
void launchCountSleeping(World& w);  // dcnt->sleeping
// colour.cu
cudaError_t colourManifolds(World& w, uint32_t nManifolds);
// solver.cu
void launchPrepare(World& w, const StepParams& sp, uint32_t nManifolds);
void launchWarmStartApply(World& w, uint32_t nM, uint32_t nColours);
void launchSweeps(World& w, const StepParams& sp, uint32_t nM, uint32_t nColours, uint32_t sweeps, bool tolMode);
void launchStoreImpulses(World& w, uint32_t nManifolds);
// Small worlds (at most 4,096 manifolds and bodies): warm start and every sweep in one
// single-CTA launch that reads the colour bounds and tests convergence on the device.
bool smallSolve(const World& w, uint32_t nM);
cudaError_t launchSolveSmall(World& w, const StepParams& sp, uint32_t sweeps, bool tolMode);
bool clusterSolve(World& w, uint32_t nM, bool multiPoint);
cudaError_t launchSolveCluster(World& w, const StepParams& sp, uint32_t nM, uint32_t sweeps, bool tolMode);
void launchLearnRows(World& w, uint32_t nM);
cudaError_t sortCrowded(World& w, uint32_t K);
void launchApplyLearned(World& w, const StepParams& sp, uint32_t nM, const float* Y);

void resolveProfile(World& w);  // after a stream sync

inline unsigned gridFor(uint64_t n, unsigned block) {
    uint64_t g = (n + block - 1) / block;
    return g == 0 ? 1u : (unsigned)g;
}

// Launch with programmatic dependent launch: the kernel may start while the previous
// kernel on the stream drains, and must call gridDependencyWait() before it touches
// anything that kernel writes.  Kernels launched this way form a chain whose launch
// latency and wave tails overlap with the next kernel's prologue.
template <typename... KArgs, typename... Args>
inline cudaError_t launchDependent(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s,
                                   Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

#ifdef __CUDACC__
// Device side of launchDependent: wait until the previous kernel on the stream has
// completed and its writes are visible (no-op for a normal launch) ...
__device__ __forceinline__ void gridDependencyWait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
// ... and let the next dependent kernel start launching (its blocks take SM slots as this
// kernel's blocks exit).
__device__ __forceinline__ void launchDependents() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
#endif

}  // namespace axiom_gb300
