// C ABI of the solver: handle lifetime, validation, device memory, setup and the time loop.
//
// Replaces the host side of the reference's hot path: the allocation, setup-kernel order and time
// loop of marchingLoop (fdtdrav.h:3425-4387) and the per-step driver solver (fdtdrav.h:3188-3422).
// Differences by design: one resident grid on one GPU (no z-slabs, ghost planes or peer copies),
// status codes instead of exit(), a compact layout (6 field arrays, a uint8 material index, CPML
// memory on the faces only) instead of 84 per-cell arrays, and stream-ordered asynchronous steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fdtd_api.h"
#include "adjoint.h"
#include "batch.h"
#include "planner.h"
#include "ports.h"
#include "yee_kernels.h"

using namespace fdtd;

namespace {

thread_local std::string t_err;

int fail(int code, const std::string& msg) {
    t_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                        \
    do {                                                                                      \
        cudaError_t _e = (expr);                                                              \
        if (_e != cudaSuccess) {                                                              \
            return fail(_e == cudaErrorMemoryAllocation ? FDTD_ERR_OOM : FDTD_ERR_CUDA,       \
                        std::string(#expr) + ": " + cudaGetErrorString(_e));                  \
        }                                                                                     \
    } while (0)

struct LumpedDef {
    int box[6];
    float resistance;
    int source;    // waveform index or -1
    int axis = 2;  // 2: Ez edges (defineSourceZ / defineResistor); 0: Ex edges (defineSourceX)
};

// The edges of a lumped element: Ez edges i in [is,ie], j in [js,je], k in [ks,ke); Ex edges of
// defineSourceX i in [is,ie), j in [js,ie] (its j bound is the box's ie, fdtdrav.h:1351), k in
// [ks,ke]. f(i, j, k) for each, k outer.
template <class F>
void lumped_edges(const LumpedDef& L, F f) {
    const int* b = L.box;
    if (L.axis == 0) {
        for (int k = b[2]; k <= b[5]; ++k)
            for (int j = b[1]; j <= b[3]; ++j)
                for (int i = b[0]; i < b[3]; ++i) f(i, j, k);
    } else {
        for (int k = b[2]; k < b[5]; ++k)
            for (int j = b[1]; j <= b[4]; ++j)
                for (int i = b[0]; i <= b[3]; ++i) f(i, j, k);
    }
}

// A zero-thickness plate (definePlateX / Y / Z): normal axis, box, sigma_e of its two tangential
// components in axis order.
struct PlateDef {
    int axis;
    int box[6];
    float sigma[2];
};

// A port: the point probes of its voltage edges (Ez, k outer, then j, then i, as voltMgpu sums
// them), then four groups of H probes s1..s4 of its current loop; I = a1 s1 + a2 s2 - a1 s3 - a2 s4
// (currMgpu, the groups and cell sizes per direction in port_groups).
struct PortDef {
    int vbox[6], ibox[6];
    int current_axis, voltage_axis;
    int first;  // probe id of the first voltage edge
    int n_v;
    int n[4];   // probes of s1..s4
};

}  // namespace

struct fdtd_handle {
    fdtd_grid grid{};
    DeviceGrid g{};
    cudaStream_t stream = nullptr;
    int schedule = FDTD_SCHEDULE_AUTO;
    int auto_choice = FDTD_SCHEDULE_AUTO;  // AUTO: the schedule its trial chose (AUTO = none yet)
    int device = 0;

    // device state: two field buffers and two CPML memory sets; `cur` holds the current step.
    // The two-pass schedule updates buffer `cur` in place, the fused sweep reads `cur` and writes
    // the other one (allocated on first use).
    float* field[2][6] = {};
    PsiSet psi[2] = {};
    int cur = 0;
    bool have_second = false;
    FusedMaps maps[2];
    CpmlMaps cmaps[2];  // the CPML sweep's maps per input buffer
    char* psi_base[2] = {nullptr, nullptr};  // the allocation holding each CPML memory set
    FusedFork fork{};  // second stream and events of the fused step (created with the fused buffers)
    struct PlanCache {  // the last fused plan and what it was made for (chunk, schedule, design box)
        bool valid = false;
        int key[9] = {};
        FusedPlan plan;
    } plan_cache;
    int kc = 0;  // planes per CTA chunk of the fused sweep
    FusedWork work{};
    bool replan = false;  // the design region or the CPML-sweep choice changed since the fused work was planned
    uint8_t* mat = nullptr;
    uint8_t* cls = nullptr;  // node classes, built by ensure_prepared
    uint16_t* rec = nullptr;          // coefficient row per node, built with the classes
    MatCoef* coef_rows = nullptr;     // material rows then interface rows (StepParams::coef)
    int n_iface_rows = 0;
    // interface-key hash set and its lists (launch_iface_set / launch_iface_rows)
    unsigned long long* iface_table = nullptr;
    unsigned long long* iface_keys = nullptr;
    int* iface_slot_row = nullptr;
    int* iface_counters = nullptr;
    int n_lumped_edges = 0;
    MatProps* props = nullptr;
    MatCoef* coef = nullptr;
    float* prof[18] = {};
    float* bg_curl[12] = {};           // per axis {E slot 0, E slot 1, H slot 0, H slot 1}
    float** d_kappa_ptrs = nullptr;    // device copies of the pointer tables the setup kernel reads
    float** d_bg_ptrs = nullptr;
    std::vector<void*> allocs;
    long long psi_elems[6] = {};  // elements per psi array of each face

    // host-side definitions
    std::vector<fdtd_material_axes> materials;
    std::vector<LumpedDef> lumped;
    std::vector<std::vector<float>> waves;  // per source, per-edge signal
    std::vector<Probe> probes;
    std::vector<PortDef> ports;

    // prepared device tables
    bool prepared = false;
    bool dirty_lumped = true, dirty_probes = true, dirty_materials = true;
    bool dirty_cpml = false;  // the CPML grading changed after the profiles were built
    float cpml_r0 = 0.f;      // 0: the reference's sigma_opt grading; else the reflection coefficient
    LumpedEdge* d_lumped = nullptr;
    int* d_lumped_k = nullptr;
    std::vector<PlateDef> plates;
    PlateEdges* d_plates = nullptr;
    int* d_plate_k = nullptr;
    int4* d_plate_nodes = nullptr;
    int n_plate_nodes = 0;
    Probe* d_probes = nullptr;
    int* d_probe_k = nullptr;
    int* d_probe_ids = nullptr;
    float** d_waves = nullptr;
    long long* d_wave_len = nullptr;
    std::vector<float*> d_wave_bufs;
    int* d_lumped_box = nullptr;
    float* d_lumped_r = nullptr;
    int* d_lumped_owner = nullptr;
    float* ring = nullptr;
    long long ring_cap = 4096;
    int* status = nullptr;
    int* small = nullptr;  // device scratch of a few ints for results read back by entry points

    long long step = 0;
    long long bytes = 0;

    // design region (cells of material kDesign, per-cell eps_r)
    bool has_design = false;
    int dbox[6] = {};
    fdtd_material design_base{};
    float* d_deps = nullptr;

    // adjoint: buffers of fdtd_adjoint_forward / fdtd_adjoint_backward
    struct Adjoint {
        bool ready = false;            // a forward has run and its records are valid
        long long n = 0, start = 0;    // steps and first step of the forward
        int K = 0;                     // checkpoint interval (0: design E of every step kept)
        long long probe = 0;           // node index of the FoM probe
        AdjState st{};
        PsiSet psa{};                  // CPML adjoint memory
        float* samples = nullptr;      // Ez(p) per forward step (device)
        std::vector<float> host_samples;
        float* hist = nullptr;         // design-edge-box E snapshots
        long long hist_slots = 0;
        char* ckpt = nullptr;          // checkpoints (K > 0) and the final state
        long long ckpt_slots = 0;
        double* acc = nullptr;         // per-edge gradient accumulators
        double* grad = nullptr;        // per-cell gradient
        int* no_probe_k = nullptr;     // per-plane probe offsets, all zero: the recompute samples nothing
        int S = 0;                     // box checkpoints every S steps inside a segment (0: none)
        long long sub_per_seg = 0;     // box checkpoints per segment
        NodeBox sub_box{};             // the design edge box grown by S nodes
        float* sub = nullptr;          // the fields over sub_box at those steps
        std::vector<void*> bufs;       // everything above, for release
        float* pinned_samples = nullptr;  // host copies (pinned: asynchronous copies)
        double* pinned_grad = nullptr;
        cudaStream_t rev = nullptr;    // the reverse sweep's stream (K > 0) and its events
        cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // recompute[2], reverse[2], start / end
        long long key[8] = {};         // steps, interval and design box the buffers were sized for
    } adj;

    // work list of fdtd_step_static_scratch (interior items first) in pinned host memory, planned
    // on first use; each call uploads it into the scratch with one asynchronous copy
    int4* static_items = nullptr;
    size_t static_n_items = 0;
    int static_counts[6] = {};     // items per list (interior, the four shell lists, CPML items)
    bool static_planned = false;

    std::vector<size_t> alloc_sizes;  // bytes of each entry of allocs

    cudaError_t alloc(void** p, size_t n) {
        cudaError_t e = cudaMalloc(p, n);
        if (e == cudaSuccess) {
            allocs.push_back(*p);
            alloc_sizes.push_back(n);
            bytes += (long long)n;
        }
        return e;
    }
    void release(void* p) {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) {
            const size_t q = (size_t)(it - allocs.begin());
            bytes -= (long long)alloc_sizes[q];
            alloc_sizes.erase(alloc_sizes.begin() + (long)q);
            allocs.erase(it);
        }
        cudaFree(p);
    }
};

namespace {

long long vol(const fdtd_handle* h) { return h->g.plane * (long long)h->g.nz; }

fdtd_material_axes axes_of(const fdtd_material& m) {
    fdtd_material_axes r;
    for (int a = 0; a < 3; ++a) {
        r.eps_r[a] = m.eps_r; r.sigma_e[a] = m.sigma_e; r.mu_r[a] = m.mu_r; r.sigma_m[a] = m.sigma_m;
    }
    return r;
}

bool in_slab_host(int q, int n, int pn, int pp) { return q < pn || q >= n - pp; }

StepParams make_params(fdtd_handle* h) {
    StepParams p{};
    p.fom_node = p.fom_read = -1;
    p.g = h->g;
    p.mat = h->mat;
    p.cls = h->cls;
    p.rec = h->rec;
    p.props = h->props;
    p.coef = h->coef_rows ? h->coef_rows : h->coef;
    const float* const* P = h->prof;
    p.bex = P[0]; p.aex = P[1]; p.bmx = P[2]; p.amx = P[3]; p.kex = P[4]; p.kmx = P[5];
    p.bey = P[6]; p.aey = P[7]; p.bmy = P[8]; p.amy = P[9]; p.key = P[10]; p.kmy = P[11];
    p.bez = P[12]; p.aez = P[13]; p.bmz = P[14]; p.amz = P[15]; p.kez = P[16]; p.kmz = P[17];
    p.lumped = h->d_lumped;
    p.lumped_k = h->d_lumped_k;
    p.probes = h->d_probes;
    p.probe_k = h->d_probe_k;
    p.probe_ids = h->d_probe_ids;
    p.waves = h->d_waves;
    p.wave_len = h->d_wave_len;
    p.probe_ring = h->ring;
    p.n_probes = (int)h->probes.size();
    p.ring_cap = h->ring_cap;
    p.status = h->status;
    p.deps = h->has_design ? h->d_deps : nullptr;
    for (int q = 0; q < 6; ++q) p.dbox[q] = h->dbox[q];
    p.plates = h->plates.empty() ? nullptr : h->d_plates;
    p.plate_k = h->plates.empty() ? nullptr : h->d_plate_k;
    p.plate_nodes = h->d_plate_nodes;
    p.n_plate_nodes = h->plates.empty() ? 0 : h->n_plate_nodes;
    p.bg.mat = 0;  // the background material fills the CPML slabs in the usual layouts
    for (int a = 0; a < 3; ++a)
        for (int s = 0; s < 2; ++s) {
            p.bg.e[a][s] = h->bg_curl[4 * a + s];
            p.bg.h[a][s] = h->bg_curl[4 * a + 2 + s];
        }
    return p;
}

int validate_grid(const fdtd_grid* g) {
    if (!g) return fail(FDTD_ERR_INVALID, "grid is NULL");
    if (g->nx < 3 || g->ny < 3 || g->nz < 3) return fail(FDTD_ERR_INVALID, "grid needs at least 3 nodes per axis");
    if ((long long)g->nx * g->ny * g->nz > (1LL << 40)) return fail(FDTD_ERR_INVALID, "grid too large");
    const float v[7] = {g->dx, g->dy, g->dz, g->dt, g->eps0, g->mu0, g->pi};
    for (float x : v)
        if (!(x > 0.f) || !std::isfinite(x)) return fail(FDTD_ERR_INVALID, "cell sizes, dt and constants must be positive and finite");
    const int n[3] = {g->nx, g->ny, g->nz};
    for (int a = 0; a < 3; ++a) {
        const int pn = g->pml[2 * a], pp = g->pml[2 * a + 1];
        if (pn < 0 || pp < 0) return fail(FDTD_ERR_INVALID, "negative CPML thickness");
        // the reference applies both faces' blocks where they overlap; require disjoint slabs
        // with at least one node between them
        if (pn + pp > n[a] - 1) return fail(FDTD_ERR_INVALID, "CPML slabs of opposite faces overlap on axis " + std::to_string(a));
    }
    return FDTD_OK;
}

int ensure_prepared(fdtd_handle* h);

// One set of CPML memory slabs (4 arrays per face), initialised to 1.2e-38.
// CPML memory set s: the 24 arrays (4 per face) in one allocation, each array on a 256-byte
// boundary, filled with the initial value by one launch (separate allocations of this size cost
// tens of microseconds each).
int alloc_psi_set(fdtd_handle* h, int s) {
    size_t off[6], bytes[6], total = 0;
    for (int f = 0; f < 6; ++f) {
        bytes[f] = ((size_t)h->psi_elems[f] * sizeof(float) + 255) / 256 * 256;
        off[f] = total;
        total += 4 * bytes[f];
    }
    h->psi[s] = PsiSet{};
    h->psi_base[s] = nullptr;
    if (total == 0) return FDTD_OK;
    char* base = nullptr;
    if (h->alloc((void**)&base, total) != cudaSuccess) return fail(FDTD_ERR_OOM, "CPML memory allocation failed");
    h->psi_base[s] = base;
    if (launch_fill((float*)base, (long long)(total / sizeof(float)), kTiny, nullptr) != cudaSuccess)
        return fail(FDTD_ERR_CUDA, "fill failed");
    for (int f = 0; f < 6; ++f) {
        if (h->psi_elems[f] <= 0) continue;
        float* a[4];
        for (int q = 0; q < 4; ++q) a[q] = (float*)(base + off[f] + (size_t)q * bytes[f]);
        h->psi[s].f[f].e[0] = a[0]; h->psi[s].f[f].e[1] = a[1];
        h->psi[s].f[f].h[0] = a[2]; h->psi[s].f[f].h[1] = a[3];
    }
    return FDTD_OK;
}

float* const* psi_arrays(fdtd_handle* h, int s, int f, float* out[4]) {
    out[0] = h->psi[s].f[f].e[0]; out[1] = h->psi[s].f[f].e[1];
    out[2] = h->psi[s].f[f].h[0]; out[3] = h->psi[s].f[f].h[1];
    return out;
}

void* tensor_map_encoder() {
    static void* fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
    }
    return fn;
}

PlanGrid plan_grid(const DeviceGrid& g) {
    return PlanGrid{g.nx, g.ny, g.nz, g.pxn, g.pxp, g.pyn, g.pyp, g.pzn, g.pzp};
}

// The lists of a plan one after the other (interior, the shell lists, the CPML items) and their
// counts.
constexpr int kWorkLists = 2 + kPlanShellLists;
static_assert(kWorkLists == 6, "fdtd_handle::static_counts holds one count per work list");
std::vector<PlanItem> flatten(const FusedPlan& plan, int counts[kWorkLists]) {
    std::vector<PlanItem> all;
    const std::vector<PlanItem>* lists[kWorkLists] = {&plan.interior, &plan.shell[0], &plan.shell[1], &plan.shell[2],
                                                      &plan.shell[3], &plan.cpml};
    for (int q = 0; q < kWorkLists; ++q) {
        counts[q] = (int)lists[q]->size();
        all.insert(all.end(), lists[q]->begin(), lists[q]->end());
    }
    return all;
}

// The work lists over a device copy of the flattened plan.
FusedWork work_of(const int4* d, const int counts[kWorkLists]) {
    static_assert(kShellLists == kPlanShellLists && kShellZ == kPlanShellZ && kShellYZ == kPlanShellYZ &&
                      kShellX == kPlanShellX && kShellAny == kPlanShellAny,
                  "planner and shell kernels agree on the shell lists");
    FusedWork w{};
    w.interior = d;
    w.n_interior = counts[0];
    const int4* at = d + counts[0];
    for (int q = 0; q < kShellLists; ++q) {
        w.shell.items[q] = at;
        w.shell.n[q] = counts[1 + q];
        at += counts[1 + q];
    }
    w.cpml = at;
    w.n_cpml = counts[1 + kShellLists];
    return w;
}

// The AUTO trial: on grids of at least kAutoTrialCells cells, the first fdtd_step call of at least
// 2 * kAutoTrialSteps steps times kAutoTrialSteps fused steps and then as many two-pass steps (real
// steps: both schedules give the same bits) and keeps the faster schedule for the handle. Which one
// wins depends on the grid: on GB300 random-box cubes with 10-cell CPML, two-pass below about
// 224^3 and fused above. Smaller grids take two-pass without a trial. Grids of at least
// kAutoDirectCells cells whose interior tiles hold at least kAutoDirectInterior of the nodes
// (512^3 with 10-cell CPML: 0.86) take fused without a trial: there fused won by 16-30 % on every
// grid measured, and the trial's two-pass steps and synchronisation cost more than a step. The
// fused buffers are freed when two-pass wins or cannot be allocated.
constexpr int64_t kAutoTrialSteps = 4;
constexpr long long kAutoTrialCells = 8LL << 20;
constexpr long long kAutoDirectCells = 64LL << 20;
constexpr double kAutoDirectInterior = 0.8;

// The fused plan for the handle's current design box and schedule, from the cache when it holds
// that plan (planning a 512^3 grid takes a few hundred microseconds on the host).
const FusedPlan& plan_current(fdtd_handle* h) {
    const PlanGrid pg = plan_grid(h->g);
    const int kc = h->kc > 0 ? h->kc : plan_chunk(pg);
    const bool cpml = h->schedule == FDTD_SCHEDULE_FUSED_CPML;
    int key[9] = {kc, cpml, h->has_design, 0, 0, 0, 0, 0, 0};
    if (h->has_design) std::copy(h->dbox, h->dbox + 6, key + 3);
    auto& C = h->plan_cache;
    if (!(C.valid && std::equal(key, key + 9, C.key))) {
        C.plan = FusedPlan{};
        plan_fused(pg, kc, h->has_design ? h->dbox : nullptr, C.plan, cpml);
        std::copy(key, key + 9, C.key);
        C.valid = true;
    }
    return C.plan;
}

// Work items of the fused schedule (planner.cpp), with CPML items under FDTD_SCHEDULE_FUSED_CPML.
// The design region, if any, stays with the shell; planned again when it or the schedule changes.
int plan_work(fdtd_handle* h) {
    const FusedPlan& plan = plan_current(h);
    int counts[kWorkLists];
    const std::vector<PlanItem> all = flatten(plan, counts);
    h->release((void*)h->work.interior);
    h->work = FusedWork{};
    int4* d = nullptr;
    CUDA_TRY(h->alloc((void**)&d, sizeof(int4) * (all.size() + 1)));
    if (!all.empty()) CUDA_TRY(cudaMemcpy(d, all.data(), sizeof(int4) * all.size(), cudaMemcpyHostToDevice));
    h->work = work_of(d, counts);
    h->replan = false;
    return FDTD_OK;
}

// Second field buffer, second CPML set and the TMA tensor maps of both buffers for the fused sweep.
int ensure_fused(fdtd_handle* h) {
    if (h->have_second && h->replan) return plan_work(h);
    if (h->have_second) return FDTD_OK;
    // no copy of the state and no fill: a fused step writes every node of its target buffer (the
    // planner's items cover each node once; plate and design nodes by their own kernels); only
    // the row padding, which no kernel writes, gets buffer 0's initial value so that saved
    // states agree
    const long long V = vol(h);
    for (int c = 0; c < 6; ++c) {
        CUDA_TRY(h->alloc((void**)&h->field[1][c], (size_t)V * sizeof(float)));
        CUDA_TRY(launch_fill_padding(h->field[1][c], h->g, kTiny, h->stream));
    }
    int rc = alloc_psi_set(h, 1);
    if (rc) return rc;
    void* enc = tensor_map_encoder();
    if (!enc) return fail(FDTD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    for (int b = 0; b < 2; ++b) {
        float* hh[3] = {h->field[b][3], h->field[b][4], h->field[b][5]};
        float* ee[3] = {h->field[b][0], h->field[b][1], h->field[b][2]};
        if (encode_fused_maps(&h->maps[b], h->g, hh, ee, h->rec, enc) != 0 ||
            encode_cpml_maps(&h->cmaps[b], h->g, hh, ee, h->rec, h->psi[b], enc) != 0)
            return fail(FDTD_ERR_CUDA, "tensor map encoding failed");
    }
    CUDA_TRY(fused_configure());
    if (!h->fork.aux) {  // the sweep's stream: as high a priority as the handle's
        int prio = 0;
        CUDA_TRY(cudaStreamGetPriority(h->stream, &prio));
        CUDA_TRY(cudaStreamCreateWithPriority(&h->fork.aux, cudaStreamNonBlocking, prio));
        CUDA_TRY(cudaEventCreateWithFlags(&h->fork.fork, cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&h->fork.join, cudaEventDisableTiming));
    }
    h->kc = plan_chunk(plan_grid(h->g));
    rc = plan_work(h);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->have_second = true;
    return FDTD_OK;
}

// AUTO runs two-pass until a trial on the handle's own grid has chosen (auto_trial).
bool use_fused(const fdtd_handle* h) {
    return h->schedule == FDTD_SCHEDULE_FUSED || h->schedule == FDTD_SCHEDULE_FUSED_CPML ||
           (h->schedule == FDTD_SCHEDULE_AUTO && h->auto_choice == FDTD_SCHEDULE_FUSED);
}

// Frees what ensure_fused allocated; the state must be in buffer 0.
void release_fused(fdtd_handle* h) {
    for (int c = 0; c < 6; ++c) {
        h->release(h->field[1][c]);
        h->field[1][c] = nullptr;
    }
    h->release(h->psi_base[1]);
    h->psi_base[1] = nullptr;
    h->psi[1] = PsiSet{};
    h->release((void*)h->work.interior);
    h->work = FusedWork{};
    h->have_second = false;
}

}  // namespace

namespace fdtd {
// The calling thread's error message for entry points defined in other translation units.
int report_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace fdtd

extern "C" {

const char* fdtd_last_error(void) { return t_err.c_str(); }
const char* fdtd_version(void) { return "fdtd_gb300 0.1 (sm_103a)"; }

int fdtd_create(const fdtd_grid* grid, fdtd_handle** out) {
    if (!out) return fail(FDTD_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int rc = validate_grid(grid);
    if (rc) return rc;
    fdtd_handle* h = new fdtd_handle();
    h->grid = *grid;
    cudaGetDevice(&h->device);
    DeviceGrid& g = h->g;
    g.nx = grid->nx; g.ny = grid->ny; g.nz = grid->nz;
    g.pitch = (grid->nx + 31) / 32 * 32;
    g.plane = (long long)g.pitch * g.ny;
    g.pxn = grid->pml[0]; g.pxp = grid->pml[1]; g.pyn = grid->pml[2]; g.pyp = grid->pml[3];
    g.pzn = grid->pml[4]; g.pzp = grid->pml[5];
    g.dx = grid->dx; g.dy = grid->dy; g.dz = grid->dz; g.dt = grid->dt; g.eps0 = grid->eps0; g.mu0 = grid->mu0;
    auto cleanup = [&](int code) { fdtd_destroy(h); return code; };
    const long long V = vol(h);
    // each field's fill (setZero's 1.2e-38) is launched as soon as it is allocated, so the device
    // fills while the host makes the remaining allocations
    for (int c = 0; c < 6; ++c) {
        cudaError_t e = h->alloc((void**)&h->field[0][c], (size_t)V * sizeof(float));
        if (e != cudaSuccess) return cleanup(fail(FDTD_ERR_OOM, "field allocation failed: " + std::string(cudaGetErrorString(e))));
        if (launch_fill(h->field[0][c], V, kTiny, nullptr) != cudaSuccess) return cleanup(fail(FDTD_ERR_CUDA, "fill failed"));
    }
    if (h->alloc((void**)&h->mat, (size_t)V) != cudaSuccess) return cleanup(fail(FDTD_ERR_OOM, "material index allocation failed"));
    if (h->alloc((void**)&h->props, sizeof(MatProps) * kMaxMaterials) != cudaSuccess ||
        h->alloc((void**)&h->coef, sizeof(MatCoef) * (kMaxMaterials + 1)) != cudaSuccess ||
        h->alloc((void**)&h->status, sizeof(int)) != cudaSuccess || h->alloc((void**)&h->small, 4 * sizeof(int)) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_OOM, "table allocation failed"));
    const int ns[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 6; ++q)
            if (h->alloc((void**)&h->prof[6 * a + q], sizeof(float) * ns[a]) != cudaSuccess)
                return cleanup(fail(FDTD_ERR_OOM, "profile allocation failed"));
    for (int a = 0; a < 3; ++a)
        for (int q = 0; q < 4; ++q)
            if (h->alloc((void**)&h->bg_curl[4 * a + q], sizeof(float) * ns[a]) != cudaSuccess)
                return cleanup(fail(FDTD_ERR_OOM, "profile allocation failed"));
    if (h->alloc((void**)&h->d_kappa_ptrs, sizeof(float*) * 6) != cudaSuccess ||
        h->alloc((void**)&h->d_bg_ptrs, sizeof(float*) * 12) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_OOM, "table allocation failed"));
    {
        float* kp[6];
        for (int a = 0; a < 3; ++a) { kp[2 * a] = h->prof[6 * a + 4]; kp[2 * a + 1] = h->prof[6 * a + 5]; }
        if (cudaMemcpy(h->d_kappa_ptrs, kp, sizeof(kp), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(h->d_bg_ptrs, h->bg_curl, sizeof(h->bg_curl), cudaMemcpyHostToDevice) != cudaSuccess)
            return cleanup(fail(FDTD_ERR_CUDA, "pointer table upload failed"));
    }
    // CPML memory: x faces (nz, ny, P), y faces (nz, P, pitch), z faces (P, ny, pitch)
    const int P[6] = {g.pxn, g.pxp, g.pyn, g.pyp, g.pzn, g.pzp};
    for (int f = 0; f < 6; ++f) {
        long long n = 0;
        if (f < 2) n = (long long)g.nz * g.ny * P[f];
        else if (f < 4) n = (long long)g.nz * P[f] * g.pitch;
        else n = (long long)P[f] * g.ny * g.pitch;
        h->psi_elems[f] = n;
    }
    rc = alloc_psi_set(h, 0);
    if (rc) return cleanup(rc);
    // node classes, coefficient rows and the interface-key set, which every preparation builds:
    // allocated here, while the fills run
    if (h->alloc((void**)&h->cls, (size_t)V) != cudaSuccess ||
        h->alloc((void**)&h->rec, (size_t)V * sizeof(uint16_t)) != cudaSuccess ||
        h->alloc((void**)&h->iface_table, sizeof(unsigned long long) * kIfaceTableSize) != cudaSuccess ||
        h->alloc((void**)&h->iface_keys, sizeof(unsigned long long) * kIfaceTableSize) != cudaSuccess ||
        h->alloc((void**)&h->iface_slot_row, sizeof(int) * kIfaceTableSize) != cudaSuccess ||
        h->alloc((void**)&h->iface_counters, sizeof(int) * 2) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_OOM, "node class allocation failed"));
    if (cudaMemsetAsync(h->cls, kGeneral, (size_t)V, nullptr) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_CUDA, "memset failed"));
    // initial state of setZero: fields (filled above) and psi 1.2e-38, material 0 everywhere
    if (cudaMemset(h->mat, 0, (size_t)V) != cudaSuccess || cudaMemset(h->status, 0, sizeof(int)) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_CUDA, "memset failed"));
    h->materials.push_back(axes_of(fdtd_material{1.0f, kTiny, 1.0f, kTiny}));
    // grids large enough for AUTO to weigh the fused schedule: plan its work on the host while the
    // fills run (the plan is cached for the first step)
    if ((long long)g.nx * g.ny * g.nz >= kAutoTrialCells) plan_current(h);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cleanup(fail(FDTD_ERR_CUDA, std::string("init: ") + cudaGetErrorString(e)));
    *out = h;
    return FDTD_OK;
}

int fdtd_destroy(fdtd_handle* h) {
    if (!h) return FDTD_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    else cudaDeviceSynchronize();
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    h->alloc_sizes.clear();
    if (h->static_items) cudaFreeHost(h->static_items);
    if (h->adj.pinned_samples) cudaFreeHost(h->adj.pinned_samples);
    if (h->adj.pinned_grad) cudaFreeHost(h->adj.pinned_grad);
    if (h->adj.rev) {
        cudaStreamSynchronize(h->adj.rev);
        for (cudaEvent_t e : h->adj.ev)
            if (e) cudaEventDestroy(e);
        cudaStreamDestroy(h->adj.rev);
    }
    if (h->fork.aux) {
        cudaStreamSynchronize(h->fork.aux);
        cudaEventDestroy(h->fork.fork);
        cudaEventDestroy(h->fork.join);
        cudaStreamDestroy(h->fork.aux);
    }
    delete h;
    return FDTD_OK;
}

int fdtd_set_stream(fdtd_handle* h, void* s) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    h->stream = (cudaStream_t)s;
    return FDTD_OK;
}

int fdtd_set_schedule(fdtd_handle* h, int32_t schedule) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (schedule < FDTD_SCHEDULE_AUTO || schedule > FDTD_SCHEDULE_FUSED_CPML)
        return fail(FDTD_ERR_INVALID, "unknown schedule");
    if ((schedule == FDTD_SCHEDULE_FUSED_CPML) != (h->schedule == FDTD_SCHEDULE_FUSED_CPML)) h->replan = true;
    h->schedule = schedule;
    h->auto_choice = FDTD_SCHEDULE_AUTO;  // AUTO runs its trial again
    return FDTD_OK;
}

int fdtd_set_materials_axes(fdtd_handle* h, const fdtd_material_axes* table, int32_t n) {
    if (!h || !table) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (n < 1 || n > kMaxMaterials) return fail(FDTD_ERR_INVALID, "material count must be 1..256");
    for (int q = 0; q < n; ++q)
        for (int a = 0; a < 3; ++a) {
            const fdtd_material_axes& m = table[q];
            const std::string what = "material " + std::to_string(q) + " axis " + std::to_string(a);
            if (!(m.eps_r[a] > 0.f) || !(m.mu_r[a] > 0.f) || !std::isfinite(m.eps_r[a]) || !std::isfinite(m.mu_r[a]))
                return fail(FDTD_ERR_INVALID, what + ": eps_r and mu_r must be positive");
            if (!(m.sigma_e[a] >= 0.f) || !std::isfinite(m.sigma_e[a]))
                return fail(FDTD_ERR_INVALID, what + ": sigma_e must be >= 0");
            // the harmonic mean of two magnetic conductivities (fdtdrav.h:1187) is 0/0 for zeros
            if (!(m.sigma_m[a] > 0.f) || !std::isfinite(m.sigma_m[a]))
                return fail(FDTD_ERR_INVALID, what + ": sigma_m must be > 0 (use 1.2e-38 for a lossless medium)");
        }
    if (h->prepared && n < (int)h->materials.size())
        return fail(FDTD_ERR_STATE, "cannot shrink the material table after the index uses it");
    if (h->has_design && n > kDesign)
        return fail(FDTD_ERR_INVALID, "material index 255 is reserved for the design region: at most 255 materials");
    h->materials.assign(table, table + n);
    h->dirty_materials = true;
    return FDTD_OK;
}

int fdtd_set_materials(fdtd_handle* h, const fdtd_material* table, int32_t n) {
    if (!h || !table) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (n < 1 || n > kMaxMaterials) return fail(FDTD_ERR_INVALID, "material count must be 1..256");
    std::vector<fdtd_material_axes> t((size_t)n);
    for (int q = 0; q < n; ++q) t[q] = axes_of(table[q]);
    return fdtd_set_materials_axes(h, t.data(), n);
}

int fdtd_set_material_index(fdtd_handle* h, const uint8_t* cells) {
    if (!h || !cells) return fail(FDTD_ERR_INVALID, "NULL argument");
    const DeviceGrid& g = h->g;
    CUDA_TRY(cudaMemcpy2DAsync(h->mat, g.pitch, cells, g.nx, g.nx, (size_t)g.ny * g.nz, cudaMemcpyHostToDevice, h->stream));
    // validated on the device: the largest index of the uploaded cells
    CUDA_TRY(launch_index_max(h->mat, g, h->small, h->stream));
    int mx = 0;
    CUDA_TRY(cudaMemcpyAsync(&mx, h->small, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->dirty_lumped = true;
    if (mx >= (int)h->materials.size()) {  // leave a valid index behind: every cell background
        CUDA_TRY(cudaMemsetAsync(h->mat, 0, (size_t)vol(h), h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        return fail(FDTD_ERR_INVALID, "material index " + std::to_string(mx) + " outside the material table (the index "
                                      "is reset to material 0)");
    }
    return FDTD_OK;
}

int fdtd_add_brick(fdtd_handle* h, const int32_t box[6], int32_t material) {
    if (!h || !box) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (material < 0 || material >= (int)h->materials.size()) return fail(FDTD_ERR_INVALID, "material outside the table");
    int b[6];
    for (int q = 0; q < 6; ++q) b[q] = box[q];
    CUDA_TRY(launch_paint(h->mat, h->g, b, (uint8_t)material, h->stream));
    h->dirty_lumped = true;
    return FDTD_OK;
}

static int check_lumped_box(fdtd_handle* h, int32_t axis, const int32_t box[6], float r) {
    if (!box) return fail(FDTD_ERR_INVALID, "box is NULL");
    if (axis != 0 && axis != 2) return fail(FDTD_ERR_INVALID, "lumped elements are x- (axis 0) or z-directed (axis 2)");
    const DeviceGrid& g = h->g;
    const int is = box[0], js = box[1], ks = box[2], ie = box[3], je = box[4], ke = box[5];
    if (axis == 2) {
        // Ez is updated for 0 < i < nx-1, 0 < j < ny-1, k < nz-1 (fdtdrav.h:720)
        if (is < 1 || ie > g.nx - 2 || is > ie || js < 1 || je > g.ny - 2 || js > je || ks < 0 || ke > g.nz - 1 ||
            ks >= ke)
            return fail(FDTD_ERR_INVALID, "lumped box outside the updated Ez edges or empty (k range is half-open)");
    } else {
        // defineSourceX's Ex edges i in [is,ie), j in [js,ie], k in [ks,ke]; Ex is updated for
        // i < nx-1, 0 < j < ny-1, 0 < k < nz-1 (fdtdrav.h:665); je enters only its resistance
        if (is < 0 || ie > g.nx - 1 || is >= ie || js < 1 || ie > g.ny - 2 || js > ie || je < js || ks < 1 ||
            ke > g.nz - 2 || ks > ke)
            return fail(FDTD_ERR_INVALID, "x-directed box outside the updated Ex edges or empty "
                                          "(i in [is,ie), j in [js,ie], k in [ks,ke])");
        if (h->has_design) return fail(FDTD_ERR_STATE, "x-directed lumped elements cannot be combined with a design region");
    }
    if (!(r > 0.f) || !std::isfinite(r)) return fail(FDTD_ERR_INVALID, "resistance must be positive");
    LumpedDef probe;
    std::copy(box, box + 6, probe.box);
    probe.axis = axis;
    std::vector<long long> mine;
    lumped_edges(probe, [&](int i, int j, int k) { mine.push_back(((long long)k * g.ny + j) * g.nx + i); });
    std::sort(mine.begin(), mine.end());
    for (const LumpedDef& L : h->lumped) {
        if (L.axis != axis) continue;  // Ex and Ez edges never coincide
        bool shared = false;
        lumped_edges(L, [&](int i, int j, int k) {
            shared = shared || std::binary_search(mine.begin(), mine.end(), ((long long)k * g.ny + j) * g.nx + i);
        });
        if (shared) return fail(FDTD_ERR_INVALID, "lumped elements may not share edges");
    }
    return FDTD_OK;
}

int fdtd_add_lumped_source(fdtd_handle* h, int32_t axis, const int32_t box[6], float resistance,
                           const float* voltage, int64_t n_samples, int32_t* id_out) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    int rc = check_lumped_box(h, axis, box, resistance);
    if (rc) return rc;
    if (n_samples < 0 || (n_samples > 0 && !voltage)) return fail(FDTD_ERR_INVALID, "bad waveform");
    LumpedDef L;
    std::memcpy(L.box, box, sizeof(L.box));
    L.resistance = resistance;
    if (axis == 0) {  // defineSourceX: coefficients only; the reference never injects it (fdtdrav.h:681)
        L.source = -1;
        L.axis = 0;
        h->lumped.push_back(L);
        h->dirty_lumped = true;
        if (id_out) *id_out = -1;
        return FDTD_OK;
    }
    L.source = (int)h->waves.size();
    // per-edge signal = V / (ke - ks) (setGauss fdtdrav.h:1494 with v_mag_factor fdtdrav.h:3613)
    const float nseg = (float)(box[5] - box[2]);
    std::vector<float> w((size_t)n_samples);
    for (int64_t m = 0; m < n_samples; ++m) w[(size_t)m] = voltage[m] / nseg;
    h->waves.push_back(std::move(w));
    h->lumped.push_back(L);
    h->dirty_lumped = true;
    if (id_out) *id_out = L.source;
    return FDTD_OK;
}

int fdtd_add_resistor(fdtd_handle* h, int32_t axis, const int32_t box[6], float resistance) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (axis != 2) return fail(FDTD_ERR_INVALID, "resistors are z-directed (defineResistor sets Ez edges only)");
    int rc = check_lumped_box(h, axis, box, resistance);
    if (rc) return rc;
    LumpedDef L;
    std::memcpy(L.box, box, sizeof(L.box));
    L.resistance = resistance;
    L.source = -1;
    h->lumped.push_back(L);
    h->dirty_lumped = true;
    return FDTD_OK;
}

int fdtd_add_plate(fdtd_handle* h, int32_t normal_axis, const int32_t box[6], float sigma_1, float sigma_2) {
    if (!h || !box) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (normal_axis < 0 || normal_axis > 2) return fail(FDTD_ERR_INVALID, "normal axis must be 0 (x), 1 (y) or 2 (z)");
    if (h->step > 0) return fail(FDTD_ERR_STATE, "plates must be added before the first step");
    if (h->has_design) return fail(FDTD_ERR_STATE, "plates cannot be combined with a design region");
    const DeviceGrid& g = h->g;
    const int n[3] = {g.nx, g.ny, g.nz};
    for (int a = 0; a < 3; ++a)
        if (box[a] < 0 || box[a] > box[a + 3] || box[a] >= n[a])
            return fail(FDTD_ERR_INVALID, "plate box outside the grid or reversed");
    if (!(sigma_1 >= 0.f) || !(sigma_2 >= 0.f)) return fail(FDTD_ERR_INVALID, "plate conductivities must be >= 0");
    PlateDef P{normal_axis, {box[0], box[1], box[2], box[3], box[4], box[5]}, {sigma_1, sigma_2}};
    h->plates.push_back(P);
    h->dirty_lumped = true;  // node classes and plate tables are rebuilt with the lumped tables
    return FDTD_OK;
}

// The sector test of tricheck (fdtdrav.h:56-128) as the reference's kernel evaluates it: point q
// against the sides p0-p1 and p1-p2 of the triangle p0 p1 p2 (q on the same side of each as the
// third vertex, or on it) and the disk of radius r around p1. Coordinates are node index times the
// cell size in float; a coordinate difference a*d - b*d is one float multiply-add of the first
// product, fma(a, d, -(b*d)), as the reference's compiled kernel forms it (which decides nodes that
// lie exactly on a side); the side tests multiply those differences in double, the distance is a
// float sum of squares, again with the first product fused, then a double square root.
struct SectorPt {
    int i, j;
};
static float sub_f(int a, int b, float d) { return std::fma((float)a, d, -((float)b * d)); }
static double cross_d(double ax, double ay, double bx, double by) { return std::fma(ax, by, -(ay * bx)); }
static bool in_sector(SectorPt q, const int32_t* t, float dx, float dy, float r) {
    const double ax = sub_f(t[2], t[0], dx), ay = sub_f(t[3], t[1], dy);  // p1 - p0
    const double bx = sub_f(t[4], t[2], dx), by = sub_f(t[5], t[3], dy);  // p2 - p1
    const double cx = sub_f(t[4], t[0], dx), cy = sub_f(t[5], t[1], dy);  // p2 - p0
    const double dx0 = sub_f(t[0], t[2], dx), dy0 = sub_f(t[1], t[3], dy);  // p0 - p1
    if (cross_d(ax, ay, cx, cy) * cross_d(ax, ay, sub_f(q.i, t[0], dx), sub_f(q.j, t[1], dy)) < 0) return false;
    if (cross_d(bx, by, dx0, dy0) * cross_d(bx, by, sub_f(q.i, t[2], dx), sub_f(q.j, t[3], dy)) < 0) return false;
    const float u = sub_f(t[2], q.i, dx), v = sub_f(t[3], q.j, dy);
    return !(std::sqrt((double)std::fma(u, u, v * v)) > (double)r);
}

int fdtd_add_sector(fdtd_handle* h, const int32_t tri[6], int32_t pz0, float radius, int32_t max_x, int32_t max_y,
                    float sigma_x, float sigma_y) {
    if (!h || !tri) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (h->step > 0) return fail(FDTD_ERR_STATE, "sectors must be added before the first step");
    if (h->has_design) return fail(FDTD_ERR_STATE, "sectors cannot be combined with a design region");
    const DeviceGrid& g = h->g;
    if (pz0 < 0 || pz0 >= g.nz) return fail(FDTD_ERR_INVALID, "sector plane outside the grid");
    if (max_x < 0 || max_y < 0) return fail(FDTD_ERR_INVALID, "sector bounds must be >= 0");
    if (!(sigma_x >= 0.f) || !(sigma_y >= 0.f)) return fail(FDTD_ERR_INVALID, "sector conductivities must be >= 0");
    auto in = [&](int i, int j) { return in_sector(SectorPt{i, j}, tri, g.dx, g.dy, radius); };
    // Ex edges as one-row z plates (their Ey range is empty), Ey edges as one-column x plates (their
    // Ez range is empty); the set is the same as the reference's, runs split where the test fails
    const int ex_i = std::min(max_x, g.nx), ex_j = std::min(max_y, g.ny - 1);  // Ex: i < max_x, j <= max_y
    const int ey_i = std::min(max_x, g.nx - 1), ey_j = std::min(max_y, g.ny);  // Ey: i <= max_x, j < max_y
    std::vector<PlateDef> add;
    for (int j = 0; j <= ex_j; ++j)
        for (int i = 0; i < ex_i;) {
            if (!in(i, j)) { ++i; continue; }
            int e = i;
            while (e + 1 < ex_i && in(e + 1, j)) ++e;
            add.push_back(PlateDef{2, {i, j, pz0, e + 1, j, pz0}, {sigma_x, 0.f}});
            i = e + 1;
        }
    for (int i = 0; i <= ey_i; ++i)
        for (int j = 0; j < ey_j;) {
            if (!in(i, j)) { ++j; continue; }
            int e = j;
            while (e + 1 < ey_j && in(i, e + 1)) ++e;
            add.push_back(PlateDef{0, {i, j, pz0, i, e + 1, pz0}, {sigma_y, 0.f}});
            j = e + 1;
        }
    h->plates.insert(h->plates.end(), add.begin(), add.end());
    h->dirty_lumped = true;
    return FDTD_OK;
}

int fdtd_add_probe(fdtd_handle* h, int32_t comp, int32_t i, int32_t j, int32_t k, int32_t* id_out) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (comp < 0 || comp > 5) return fail(FDTD_ERR_INVALID, "component must be 0..5");
    if (i < 0 || i >= h->g.nx || j < 0 || j >= h->g.ny || k < 0 || k >= h->g.nz) return fail(FDTD_ERR_INVALID, "probe outside the grid");
    if (h->step > 0) return fail(FDTD_ERR_STATE, "probes must be added before the first step");
    h->probes.push_back(Probe{comp, i, j, k});
    h->dirty_probes = true;
    if (id_out) *id_out = (int)h->probes.size() - 1;
    return FDTD_OK;
}

int fdtd_set_probe_capacity(fdtd_handle* h, int64_t steps) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (steps < 1) return fail(FDTD_ERR_INVALID, "capacity must be >= 1");
    if (h->step > 0) return fail(FDTD_ERR_STATE, "capacity must be set before the first step");
    h->ring_cap = steps;
    h->dirty_probes = true;
    return FDTD_OK;
}

int fdtd_prepare(fdtd_handle* h) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    return ensure_prepared(h);
}

namespace {

int steps_fused(fdtd_handle* h, const StepParams& p, int64_t n) {
    int rc = ensure_fused(h);
    if (rc) return rc;
    for (int64_t s = 0; s < n; ++s) {
        const int a = h->cur, b = 1 - h->cur;
        FieldPtrs fi{h->field[a][0], h->field[a][1], h->field[a][2], h->field[a][3], h->field[a][4], h->field[a][5]};
        FieldPtrs fo{h->field[b][0], h->field[b][1], h->field[b][2], h->field[b][3], h->field[b][4], h->field[b][5]};
        CUDA_TRY(launch_fused(h->maps[a], p, fi, fo, h->psi[a], h->psi[b], h->step, h->work, h->stream,
                              h->fork.aux ? &h->fork : nullptr, &h->cmaps[a]));
        h->cur = b;
        ++h->step;
    }
    return FDTD_OK;
}

int steps_two_pass(fdtd_handle* h, const StepParams& p, int64_t n) {
    const int a = h->cur;
    FieldPtrs f{h->field[a][0], h->field[a][1], h->field[a][2], h->field[a][3], h->field[a][4], h->field[a][5]};
    for (int64_t s = 0; s < n; ++s) {
        CUDA_TRY(launch_two_pass(p, f, h->psi[a], h->step, h->stream));
        ++h->step;
    }
    return FDTD_OK;
}

// Share of the grid's nodes that the interior sweep's tiles hold (overlapping tiles counted once
// per tile, a slight overestimate).
double interior_share(fdtd_handle* h) {
    const FusedPlan& plan = plan_current(h);
    long long n = 0;
    for (const PlanItem& it : plan.interior) n += (long long)(it.w - it.z) * kTileX * kTileY;
    return (double)n / ((double)h->g.nx * h->g.ny * h->g.nz);
}

// AUTO's choice without a trial where it is clear (see above); false: run the trial.
bool auto_direct(fdtd_handle* h) {
    if ((long long)h->g.nx * h->g.ny * h->g.nz < kAutoDirectCells || interior_share(h) < kAutoDirectInterior) return false;
    if (ensure_fused(h) != FDTD_OK) {  // no room for the second buffers
        cudaGetLastError();
        if (h->cur == 0) release_fused(h);
        h->auto_choice = FDTD_SCHEDULE_TWO_PASS;
        return true;
    }
    h->auto_choice = FDTD_SCHEDULE_FUSED;
    return true;
}

int auto_trial(fdtd_handle* h, const StepParams& p) {
    if (ensure_fused(h) != FDTD_OK) {  // no room for the second buffers
        cudaGetLastError();
        if (h->cur == 0) release_fused(h);
        h->auto_choice = FDTD_SCHEDULE_TWO_PASS;
        return FDTD_OK;
    }
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    struct Guard {
        cudaEvent_t* e;
        ~Guard() {
            for (int q = 0; q < 3; ++q)
                if (e[q]) cudaEventDestroy(e[q]);
        }
    } guard{ev};
    for (cudaEvent_t& e : ev) CUDA_TRY(cudaEventCreate(&e));
    CUDA_TRY(cudaEventRecord(ev[0], h->stream));
    int rc = steps_fused(h, p, kAutoTrialSteps);  // an even count
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(ev[1], h->stream));
    if ((rc = steps_two_pass(h, p, kAutoTrialSteps))) return rc;
    CUDA_TRY(cudaEventRecord(ev[2], h->stream));
    CUDA_TRY(cudaEventSynchronize(ev[2]));
    float t_fused = 0.f, t_two = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t_fused, ev[0], ev[1]));
    CUDA_TRY(cudaEventElapsedTime(&t_two, ev[1], ev[2]));
    h->auto_choice = t_fused < t_two ? FDTD_SCHEDULE_FUSED : FDTD_SCHEDULE_TWO_PASS;
    // the fused steps came in pairs, so the state is back in the buffer it started in
    if (h->auto_choice == FDTD_SCHEDULE_TWO_PASS && h->cur == 0) release_fused(h);
    return FDTD_OK;
}

}  // namespace

int fdtd_step(fdtd_handle* h, int64_t n) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (n < 0) return fail(FDTD_ERR_INVALID, "negative step count");
    int rc = ensure_prepared(h);
    if (rc) return rc;
    StepParams p = make_params(h);
    if (h->schedule == FDTD_SCHEDULE_AUTO && h->auto_choice == FDTD_SCHEDULE_AUTO && n >= 2 * kAutoTrialSteps &&
        (long long)h->g.nx * h->g.ny * h->g.nz >= kAutoTrialCells && !auto_direct(h)) {
        if ((rc = auto_trial(h, p))) return rc;
        n -= 2 * kAutoTrialSteps;
    }
    return use_fused(h) ? steps_fused(h, p, n) : steps_two_pass(h, p, n);
}

int32_t fdtd_active_schedule(const fdtd_handle* h) {
    if (!h) return -1;
    if (h->schedule != FDTD_SCHEDULE_AUTO) return h->schedule;
    return h->auto_choice == FDTD_SCHEDULE_AUTO ? FDTD_SCHEDULE_TWO_PASS : h->auto_choice;
}

int fdtd_synchronize(fdtd_handle* h) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    int st = 0;
    CUDA_TRY(cudaMemcpy(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) return fail(FDTD_ERR_DEVICE, "device status word " + std::to_string(st));
    return FDTD_OK;
}

int64_t fdtd_current_step(const fdtd_handle* h) { return h ? h->step : -1; }
int32_t fdtd_probe_count(const fdtd_handle* h) { return h ? (int32_t)h->probes.size() : -1; }

int fdtd_read_probes(fdtd_handle* h, int64_t first, int64_t n, float* out) {
    if (!h || (!out && n > 0)) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (n == 0 || h->probes.empty()) return FDTD_OK;
    if (first < 0 || first + n > h->step) return fail(FDTD_ERR_RANGE, "steps not computed yet");
    if (first < h->step - h->ring_cap) return fail(FDTD_ERR_RANGE, "steps already overwritten in the probe ring buffer");
    const int np = (int)h->probes.size();
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    int64_t done = 0;
    while (done < n) {
        const int64_t m = first + done;
        const int64_t row = m % h->ring_cap;
        const int64_t run = std::min<int64_t>(n - done, h->ring_cap - row);
        CUDA_TRY(cudaMemcpy(out + done * np, h->ring + row * np, (size_t)run * np * sizeof(float), cudaMemcpyDeviceToHost));
        done += run;
    }
    return FDTD_OK;
}

int fdtd_get_field(fdtd_handle* h, int32_t comp, float* out) {
    if (!h || !out) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (comp < 0 || comp > 5) return fail(FDTD_ERR_INVALID, "component must be 0..5");
    const DeviceGrid& g = h->g;
    CUDA_TRY(cudaMemcpy2DAsync(out, (size_t)g.nx * 4, h->field[h->cur][comp], (size_t)g.pitch * 4, (size_t)g.nx * 4,
                               (size_t)g.ny * g.nz, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FDTD_OK;
}

int fdtd_set_field(fdtd_handle* h, int32_t comp, const float* in) {
    if (!h || !in) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (comp < 0 || comp > 5) return fail(FDTD_ERR_INVALID, "component must be 0..5");
    const DeviceGrid& g = h->g;
    for (int b = 0; b < (h->have_second ? 2 : 1); ++b)
        CUDA_TRY(cudaMemcpy2DAsync(h->field[b][comp], (size_t)g.pitch * 4, in, (size_t)g.nx * 4, (size_t)g.nx * 4,
                                   (size_t)g.ny * g.nz, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FDTD_OK;
}

int fdtd_get_field_device(fdtd_handle* h, int32_t comp, float* out) {
    if (!h || !out) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (comp < 0 || comp > 5) return fail(FDTD_ERR_INVALID, "component must be 0..5");
    const DeviceGrid& g = h->g;
    CUDA_TRY(cudaMemcpy2DAsync(out, (size_t)g.nx * 4, h->field[h->cur][comp], (size_t)g.pitch * 4, (size_t)g.nx * 4,
                               (size_t)g.ny * g.nz, cudaMemcpyDeviceToDevice, h->stream));
    return FDTD_OK;
}

int fdtd_set_field_device(fdtd_handle* h, int32_t comp, const float* in) {
    if (!h || !in) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (comp < 0 || comp > 5) return fail(FDTD_ERR_INVALID, "component must be 0..5");
    const DeviceGrid& g = h->g;
    for (int b = 0; b < (h->have_second ? 2 : 1); ++b)
        CUDA_TRY(cudaMemcpy2DAsync(h->field[b][comp], (size_t)g.pitch * 4, in, (size_t)g.nx * 4, (size_t)g.nx * 4,
                                   (size_t)g.ny * g.nz, cudaMemcpyDeviceToDevice, h->stream));
    return FDTD_OK;
}

}  // extern "C"

namespace {

// Copy the dynamic state (6 fields, then the 24 CPML arrays) to or from a device buffer on the
// handle's stream, without synchronising. Loading writes both field buffers of the fused schedule.
int state_copy(fdtd_handle* h, void* buf, bool save) {
    char* p = (char*)buf;
    const size_t V = (size_t)vol(h) * sizeof(float);
    const int a = h->cur, nb = h->have_second ? 2 : 1;
    for (int c = 0; c < 6; ++c, p += V) {
        if (save) CUDA_TRY(cudaMemcpyAsync(p, h->field[a][c], V, cudaMemcpyDeviceToDevice, h->stream));
        else
            for (int b = 0; b < nb; ++b) CUDA_TRY(cudaMemcpyAsync(h->field[b][c], p, V, cudaMemcpyDeviceToDevice, h->stream));
    }
    for (int f = 0; f < 6; ++f) {
        const size_t n = (size_t)h->psi_elems[f] * sizeof(float);
        float* arr[4];
        psi_arrays(h, a, f, arr);
        for (int q = 0; q < 4; ++q, p += n) {
            if (!n) continue;
            if (save) CUDA_TRY(cudaMemcpyAsync(p, arr[q], n, cudaMemcpyDeviceToDevice, h->stream));
            else CUDA_TRY(cudaMemcpyAsync(arr[q], p, n, cudaMemcpyDeviceToDevice, h->stream));
        }
    }
    return FDTD_OK;
}

}  // namespace

extern "C" {

int64_t fdtd_state_bytes(const fdtd_handle* h) {
    if (!h) return -1;
    long long n = 6 * vol(h);
    for (int f = 0; f < 6; ++f) n += 4 * h->psi_elems[f];
    return n * (int64_t)sizeof(float) + 64;
}

int fdtd_save_state(fdtd_handle* h, void* buf) {
    if (!h || !buf) return fail(FDTD_ERR_INVALID, "NULL argument");
    char* p = (char*)buf;
    const size_t V = (size_t)vol(h) * sizeof(float);
    const int a = h->cur;
    for (int c = 0; c < 6; ++c, p += V) CUDA_TRY(cudaMemcpyAsync(p, h->field[a][c], V, cudaMemcpyDeviceToDevice, h->stream));
    for (int f = 0; f < 6; ++f) {
        const size_t n = (size_t)h->psi_elems[f] * sizeof(float);
        float* arr[4];
        psi_arrays(h, a, f, arr);
        for (int q = 0; q < 4; ++q, p += n)
            if (n) CUDA_TRY(cudaMemcpyAsync(p, arr[q], n, cudaMemcpyDeviceToDevice, h->stream));
    }
    long long hdr[8] = {h->step, h->g.nx, h->g.ny, h->g.nz, 0, 0, 0, 0};
    CUDA_TRY(cudaMemcpyAsync(p, hdr, sizeof(hdr), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FDTD_OK;
}

int fdtd_load_state(fdtd_handle* h, const void* buf) {
    if (!h || !buf) return fail(FDTD_ERR_INVALID, "NULL argument");
    const char* p = (const char*)buf;
    const size_t V = (size_t)vol(h) * sizeof(float);
    {
        long long hdr[8];
        const size_t off = 6 * V + [&] { size_t t = 0; for (int f = 0; f < 6; ++f) t += 4 * (size_t)h->psi_elems[f] * sizeof(float); return t; }();
        CUDA_TRY(cudaMemcpyAsync(hdr, p + off, sizeof(hdr), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        if (hdr[1] != h->g.nx || hdr[2] != h->g.ny || hdr[3] != h->g.nz) return fail(FDTD_ERR_INVALID, "state belongs to another grid");
        h->step = hdr[0];
    }
    const int nb = h->have_second ? 2 : 1;
    for (int c = 0; c < 6; ++c, p += V)
        for (int b = 0; b < nb; ++b) CUDA_TRY(cudaMemcpyAsync(h->field[b][c], p, V, cudaMemcpyDeviceToDevice, h->stream));
    for (int f = 0; f < 6; ++f) {
        const size_t n = (size_t)h->psi_elems[f] * sizeof(float);
        float* arr[4];
        psi_arrays(h, h->cur, f, arr);
        for (int q = 0; q < 4; ++q, p += n)
            if (n) CUDA_TRY(cudaMemcpyAsync(arr[q], p, n, cudaMemcpyDeviceToDevice, h->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FDTD_OK;
}

int fdtd_tune_schedule(fdtd_handle* h) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    int rc = ensure_prepared(h);
    if (rc) return rc;
    if (h->schedule != FDTD_SCHEDULE_AUTO || h->auto_choice != FDTD_SCHEDULE_AUTO) return FDTD_OK;
    if ((long long)h->g.nx * h->g.ny * h->g.nz < kAutoTrialCells) {
        h->auto_choice = FDTD_SCHEDULE_TWO_PASS;
        return FDTD_OK;
    }
    if (auto_direct(h)) return FDTD_OK;
    // the trial's steps are undone: state and probe ring saved before, restored after
    const size_t ring = sizeof(float) * (size_t)h->ring_cap * std::max<size_t>(h->probes.size(), 1);
    void* saved = nullptr;
    if (cudaMalloc(&saved, (size_t)fdtd_state_bytes(h) + ring) != cudaSuccess) {
        cudaGetLastError();
        return FDTD_OK;  // no room: the first long fdtd_step call runs the trial instead
    }
    struct Free {
        void* p;
        ~Free() { cudaFree(p); }
    } guard{saved};
    char* ring_copy = (char*)saved + fdtd_state_bytes(h);
    if ((rc = state_copy(h, saved, true))) return rc;
    CUDA_TRY(cudaMemcpyAsync(ring_copy, h->ring, ring, cudaMemcpyDeviceToDevice, h->stream));
    const long long step = h->step;
    if ((rc = auto_trial(h, make_params(h)))) return rc;
    if ((rc = state_copy(h, saved, false))) return rc;
    CUDA_TRY(cudaMemcpyAsync(h->ring, ring_copy, ring, cudaMemcpyDeviceToDevice, h->stream));
    h->step = step;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return FDTD_OK;
}

int fdtd_set_cpml_grading(fdtd_handle* h, float r0) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (!(r0 == 0.f || (r0 > 0.f && r0 < 1.f))) return fail(FDTD_ERR_INVALID, "r0 must be 0 (reference grading) or in (0, 1)");
    if (r0 != h->cpml_r0) {
        h->cpml_r0 = r0;
        h->dirty_cpml = true;
    }
    return FDTD_OK;
}

int fdtd_get_cpml_profile(fdtd_handle* h, int32_t axis, int32_t kind, float* out) {
    if (!h || !out) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (axis < 0 || axis > 2 || kind < 0 || kind > 5) return fail(FDTD_ERR_INVALID, "axis 0..2, kind 0..5");
    int rc = ensure_prepared(h);
    if (rc) return rc;
    const int n = axis == 0 ? h->g.nx : axis == 1 ? h->g.ny : h->g.nz;
    CUDA_TRY(cudaMemcpy(out, h->prof[6 * axis + kind], sizeof(float) * n, cudaMemcpyDeviceToHost));
    return FDTD_OK;
}

int64_t fdtd_device_bytes(const fdtd_handle* h) { return h ? h->bytes : -1; }

}  // extern "C"

namespace {

int build_lumped(fdtd_handle* h) {
    // free the previous tables
    h->release(h->d_lumped); h->release(h->d_lumped_k); h->release(h->d_waves); h->release(h->d_wave_len);
    h->release(h->d_lumped_box); h->release(h->d_lumped_r); h->release(h->d_lumped_owner);
    for (float* w : h->d_wave_bufs) h->release(w);
    h->d_wave_bufs.clear();
    h->d_lumped = nullptr; h->d_lumped_k = nullptr; h->d_waves = nullptr; h->d_wave_len = nullptr;
    h->d_lumped_box = nullptr; h->d_lumped_r = nullptr; h->d_lumped_owner = nullptr;
    const DeviceGrid& g = h->g;
    // edges bucketed by plane k
    std::vector<LumpedEdge> edges;
    std::vector<int> owner;
    for (size_t q = 0; q < h->lumped.size(); ++q) {
        const LumpedDef& L = h->lumped[q];
        lumped_edges(L, [&](int i, int j, int k) {
            edges.push_back(LumpedEdge{i, j, k, L.axis, L.source, 0.f, 0.f, 0.f, 0.f});
            owner.push_back((int)q);
        });
    }
    std::vector<int> order(edges.size());
    for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return edges[a].k < edges[b].k; });
    std::vector<LumpedEdge> se;
    std::vector<int> so;
    for (int q : order) { se.push_back(edges[q]); so.push_back(owner[q]); }
    std::vector<int> koff(g.nz + 1, 0);
    for (const LumpedEdge& e : se) koff[e.k + 1]++;
    for (int k = 0; k < g.nz; ++k) koff[k + 1] += koff[k];
    const size_t ne = se.size();
    h->n_lumped_edges = (int)ne;
    CUDA_TRY(h->alloc((void**)&h->d_lumped_k, sizeof(int) * (g.nz + 1)));
    CUDA_TRY(cudaMemcpy(h->d_lumped_k, koff.data(), sizeof(int) * (g.nz + 1), cudaMemcpyHostToDevice));
    CUDA_TRY(h->alloc((void**)&h->d_lumped, sizeof(LumpedEdge) * std::max<size_t>(ne, 1)));
    if (ne) {
        std::vector<int> boxes;
        std::vector<float> rs;
        for (const LumpedDef& L : h->lumped) { boxes.insert(boxes.end(), L.box, L.box + 6); rs.push_back(L.resistance); }
        CUDA_TRY(h->alloc((void**)&h->d_lumped_box, sizeof(int) * boxes.size()));
        CUDA_TRY(h->alloc((void**)&h->d_lumped_r, sizeof(float) * rs.size()));
        CUDA_TRY(h->alloc((void**)&h->d_lumped_owner, sizeof(int) * ne));
        CUDA_TRY(cudaMemcpy(h->d_lumped, se.data(), sizeof(LumpedEdge) * ne, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_lumped_box, boxes.data(), sizeof(int) * boxes.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_lumped_r, rs.data(), sizeof(float) * rs.size(), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_lumped_owner, so.data(), sizeof(int) * ne, cudaMemcpyHostToDevice));
        CUDA_TRY(launch_lumped_coefs(g, h->mat, h->props, h->d_lumped, h->d_lumped_box, h->d_lumped_r,
                                     h->d_lumped_owner, (int)ne, h->stream));
    }
    // waveforms
    const size_t nw = h->waves.size();
    std::vector<float*> ptrs(std::max<size_t>(nw, 1), nullptr);
    std::vector<long long> lens(std::max<size_t>(nw, 1), 0);
    for (size_t w = 0; w < nw; ++w) {
        float* d = nullptr;
        CUDA_TRY(h->alloc((void**)&d, sizeof(float) * std::max<size_t>(h->waves[w].size(), 1)));
        if (!h->waves[w].empty())
            CUDA_TRY(cudaMemcpy(d, h->waves[w].data(), sizeof(float) * h->waves[w].size(), cudaMemcpyHostToDevice));
        h->d_wave_bufs.push_back(d);
        ptrs[w] = d;
        lens[w] = (long long)h->waves[w].size();
    }
    CUDA_TRY(h->alloc((void**)&h->d_waves, sizeof(float*) * ptrs.size()));
    CUDA_TRY(h->alloc((void**)&h->d_wave_len, sizeof(long long) * lens.size()));
    CUDA_TRY(cudaMemcpy(h->d_waves, ptrs.data(), sizeof(float*) * ptrs.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_wave_len, lens.data(), sizeof(long long) * lens.size(), cudaMemcpyHostToDevice));
    h->dirty_lumped = false;
    return FDTD_OK;
}

// The E edges each plate covers, per component and plane, in the order of definePlateX / Y / Z
// (fdtdrav.h:1574-1679), clipped to the grid: X plate at i = is: Ey j in [js, je), k in [ks, ke];
// Ez j in [js, je], k in [ks, ke). Y plate at j = js: Ez i in [is, ie], k in [ks, ke); Ex i in
// [is, ie), k in [ks, ke]. Z plate at k = ks: Ex i in [is, ie), j in [js, je]; Ey i in [is, ie],
// j in [js, je).
struct PlateRange {
    int comp;
    int lo[3], hi[3];  // inclusive node ranges
    float sigma;
};
std::vector<PlateRange> plate_ranges(const DeviceGrid& g, const PlateDef& P) {
    const int* b = P.box;
    std::vector<PlateRange> out;
    auto add = [&](int comp, int i0, int i1, int j0, int j1, int k0, int k1, float s) {
        PlateRange r{comp, {std::max(i0, 0), std::max(j0, 0), std::max(k0, 0)},
                     {std::min(i1, g.nx - 1), std::min(j1, g.ny - 1), std::min(k1, g.nz - 1)}, s};
        if (r.lo[0] <= r.hi[0] && r.lo[1] <= r.hi[1] && r.lo[2] <= r.hi[2]) out.push_back(r);
    };
    if (P.axis == 0) {
        add(1, b[0], b[0], b[1], b[4] - 1, b[2], b[5], P.sigma[0]);
        add(2, b[0], b[0], b[1], b[4], b[2], b[5] - 1, P.sigma[1]);
    } else if (P.axis == 1) {
        add(2, b[0], b[3], b[1], b[1], b[2], b[5] - 1, P.sigma[1]);
        add(0, b[0], b[3] - 1, b[1], b[1], b[2], b[5], P.sigma[0]);
    } else {
        add(0, b[0], b[3] - 1, b[1], b[4], b[2], b[2], P.sigma[0]);
        add(1, b[0], b[3], b[1], b[4] - 1, b[2], b[2], P.sigma[1]);
    }
    return out;
}

// Plate tables: edge ranges bucketed by plane (plate order kept within a plane, so the last plate
// wins as in the reference), and the list of nodes with a covered edge (node class kPlateNode).
int build_plates(fdtd_handle* h) {
    h->release(h->d_plates); h->release(h->d_plate_k); h->release(h->d_plate_nodes);
    h->d_plates = nullptr; h->d_plate_k = nullptr; h->d_plate_nodes = nullptr;
    h->n_plate_nodes = 0;
    if (h->plates.empty()) return FDTD_OK;
    const DeviceGrid& g = h->g;
    std::vector<std::vector<PlateEdges>> per_k(g.nz);
    std::vector<long long> nodes;
    for (const PlateDef& P : h->plates)
        for (const PlateRange& r : plate_ranges(g, P))
            for (int k = r.lo[2]; k <= r.hi[2]; ++k) {
                per_k[k].push_back(PlateEdges{r.comp, r.lo[0], r.hi[0], r.lo[1], r.hi[1], r.sigma});
                for (int j = r.lo[1]; j <= r.hi[1]; ++j)
                    for (int i = r.lo[0]; i <= r.hi[0]; ++i) nodes.push_back(((long long)k * g.ny + j) * g.nx + i);
            }
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    // lumped edges take their own coefficients from the cells' materials: no plate may cover one
    std::vector<long long> lumped_e[3];
    for (const LumpedDef& L : h->lumped)
        lumped_edges(L, [&](int i, int j, int k) { lumped_e[L.axis].push_back(((long long)k * g.ny + j) * g.nx + i); });
    for (auto& v : lumped_e) std::sort(v.begin(), v.end());
    for (const PlateDef& P : h->plates)
        for (const PlateRange& r : plate_ranges(g, P)) {
            const std::vector<long long>& le = lumped_e[r.comp];
            if (le.empty()) continue;
            for (int k = r.lo[2]; k <= r.hi[2]; ++k)
                for (int j = r.lo[1]; j <= r.hi[1]; ++j)
                    for (int i = r.lo[0]; i <= r.hi[0]; ++i)
                        if (std::binary_search(le.begin(), le.end(), ((long long)k * g.ny + j) * g.nx + i))
                            return fail(FDTD_ERR_INVALID, "a plate covers the edge of a lumped element");
        }
    std::vector<PlateEdges> flat;
    std::vector<int> koff(g.nz + 1, 0);
    for (int k = 0; k < g.nz; ++k) {
        flat.insert(flat.end(), per_k[k].begin(), per_k[k].end());
        koff[k + 1] = (int)flat.size();
    }
    std::vector<int4> list(nodes.size());
    for (size_t q = 0; q < nodes.size(); ++q) {
        const long long v = nodes[q];
        list[q] = make_int4((int)(v % g.nx), (int)((v / g.nx) % g.ny), (int)(v / ((long long)g.nx * g.ny)), 0);
    }
    CUDA_TRY(h->alloc((void**)&h->d_plates, sizeof(PlateEdges) * std::max<size_t>(flat.size(), 1)));
    CUDA_TRY(h->alloc((void**)&h->d_plate_k, sizeof(int) * (g.nz + 1)));
    CUDA_TRY(h->alloc((void**)&h->d_plate_nodes, sizeof(int4) * std::max<size_t>(list.size(), 1)));
    if (!flat.empty()) CUDA_TRY(cudaMemcpy(h->d_plates, flat.data(), sizeof(PlateEdges) * flat.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->d_plate_k, koff.data(), sizeof(int) * (g.nz + 1), cudaMemcpyHostToDevice));
    if (!list.empty()) CUDA_TRY(cudaMemcpy(h->d_plate_nodes, list.data(), sizeof(int4) * list.size(), cudaMemcpyHostToDevice));
    h->n_plate_nodes = (int)list.size();
    return FDTD_OK;
}

// Interface rows (kInterfaceNode and kGeneral nodes): gather the seven-cell keys, sort and unique
// them here, then write each node's coefficient row and the rows themselves. Runs after the node
// classes and plates are final.
int build_interface_rows(fdtd_handle* h) {
    const DeviceGrid& g = h->g;
    if (!h->rec) CUDA_TRY(h->alloc((void**)&h->rec, (size_t)vol(h) * sizeof(uint16_t)));
    if (!h->iface_table) {
        CUDA_TRY(h->alloc((void**)&h->iface_table, sizeof(unsigned long long) * kIfaceTableSize));
        CUDA_TRY(h->alloc((void**)&h->iface_keys, sizeof(unsigned long long) * kIfaceTableSize));
        CUDA_TRY(h->alloc((void**)&h->iface_slot_row, sizeof(int) * kIfaceTableSize));
        CUDA_TRY(h->alloc((void**)&h->iface_counters, sizeof(int) * 2));
    }
    // distinct keys on the device; only they come to the host (two small copies)
    CUDA_TRY(launch_iface_set(g, h->cls, h->mat, h->iface_table, h->iface_counters, h->iface_keys, h->stream));
    int counters[2] = {0, 0};
    CUDA_TRY(cudaMemcpyAsync(counters, h->iface_counters, sizeof(counters), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    const int n = std::min(counters[1], kIfaceTableSize);
    std::vector<unsigned long long> hk((size_t)n);
    if (n > 0) {
        CUDA_TRY(cudaMemcpyAsync(hk.data(), h->iface_keys, (size_t)n * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        std::sort(hk.begin(), hk.end());
        hk.erase(std::unique(hk.begin(), hk.end()), hk.end());
        if (hk.size() > (size_t)kMaxInterfaceRows) hk.resize((size_t)kMaxInterfaceRows);  // the rest stay general
        // pageable source: the copy has taken the data when the call returns
        CUDA_TRY(cudaMemcpyAsync(h->iface_keys, hk.data(), hk.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                                 h->stream));
    }
    const int n_rows = (int)hk.size();
    h->release(h->coef_rows);
    h->coef_rows = nullptr;
    h->n_iface_rows = 0;
    CUDA_TRY(h->alloc((void**)&h->coef_rows, sizeof(MatCoef) * (size_t)(kFirstInterfaceRow + n_rows)));
    CUDA_TRY(cudaMemcpyAsync(h->coef_rows, h->coef, sizeof(MatCoef) * (size_t)kFirstInterfaceRow, cudaMemcpyDeviceToDevice,
                             h->stream));
    CUDA_TRY(launch_iface_rows(g, h->cls, h->mat, h->iface_table, h->iface_keys, n_rows, h->iface_slot_row, h->rec,
                               h->stream));
    CUDA_TRY(launch_rec_general(g, h->d_lumped, h->n_lumped_edges, h->rec, h->stream));
    StepParams p{};  // the rows come from the material rows and properties only
    p.g = g;
    p.props = h->props;
    p.coef = h->coef;
    CUDA_TRY(launch_iface_coefs(p, h->iface_keys, n_rows, h->coef_rows, h->stream));
    h->n_iface_rows = n_rows;
    return FDTD_OK;
}

int build_probes(fdtd_handle* h) {
    h->release(h->d_probes); h->release(h->d_probe_k); h->release(h->d_probe_ids); h->release(h->ring);
    h->d_probes = nullptr; h->d_probe_k = nullptr; h->d_probe_ids = nullptr; h->ring = nullptr;
    const DeviceGrid& g = h->g;
    const size_t np = h->probes.size();
    std::vector<int> order(np);
    for (size_t q = 0; q < np; ++q) order[q] = (int)q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return h->probes[a].k < h->probes[b].k; });
    std::vector<Probe> sp;
    for (int q : order) sp.push_back(h->probes[q]);
    std::vector<int> koff(g.nz + 1, 0);
    for (const Probe& p : sp) koff[p.k + 1]++;
    for (int k = 0; k < g.nz; ++k) koff[k + 1] += koff[k];
    CUDA_TRY(h->alloc((void**)&h->d_probe_k, sizeof(int) * (g.nz + 1)));
    CUDA_TRY(cudaMemcpy(h->d_probe_k, koff.data(), sizeof(int) * (g.nz + 1), cudaMemcpyHostToDevice));
    CUDA_TRY(h->alloc((void**)&h->d_probes, sizeof(Probe) * std::max<size_t>(np, 1)));
    CUDA_TRY(h->alloc((void**)&h->d_probe_ids, sizeof(int) * std::max<size_t>(np, 1)));
    if (np) {
        CUDA_TRY(cudaMemcpy(h->d_probes, sp.data(), sizeof(Probe) * np, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(h->d_probe_ids, order.data(), sizeof(int) * np, cudaMemcpyHostToDevice));
    }
    CUDA_TRY(h->alloc((void**)&h->ring, sizeof(float) * (size_t)h->ring_cap * std::max<size_t>(np, 1)));
    h->dirty_probes = false;
    return FDTD_OK;
}

int ensure_prepared(fdtd_handle* h) {
    if (!h->dirty_materials && !h->dirty_lumped && !h->dirty_probes && !h->dirty_cpml && h->prepared) return FDTD_OK;
    if (h->dirty_materials || h->dirty_cpml || !h->prepared) {
        std::vector<MatProps> props(kMaxMaterials);
        for (int q = 0; q < kMaxMaterials; ++q) {
            fdtd_material_axes m =
                q < (int)h->materials.size() ? h->materials[q] : axes_of(fdtd_material{1.0f, kTiny, 1.0f, kTiny});
            if (q == kDesign && h->has_design) m = axes_of(h->design_base);  // eps_r comes per cell
            for (int a = 0; a < 3; ++a) props[q].a[a] = MatAxis{m.eps_r[a], m.sigma_e[a], m.mu_r[a], m.sigma_m[a]};
        }
        CUDA_TRY(cudaMemcpy(h->props, props.data(), sizeof(MatProps) * kMaxMaterials, cudaMemcpyHostToDevice));
        const int n_tab = h->has_design ? kMaxMaterials : (int)h->materials.size();
        CUDA_TRY(launch_material_tables(h->g, h->props, n_tab, h->coef, h->stream));
        if (!h->prepared || h->dirty_cpml) CUDA_TRY(launch_cpml_profiles(h->g, h->grid.pi, h->cpml_r0, h->prof, h->stream));
        h->dirty_cpml = false;
        CUDA_TRY(launch_bg_curl(h->g, h->coef, 0, h->d_kappa_ptrs, h->d_bg_ptrs, h->stream));
        h->dirty_materials = false;
        h->dirty_lumped = true;
    }
    if (h->dirty_lumped) {
        int rc = build_lumped(h);
        if (rc) return rc;
        // node classes depend on the material index and the lumped edges
        if (!h->cls) {
            CUDA_TRY(h->alloc((void**)&h->cls, (size_t)vol(h)));
            CUDA_TRY(cudaMemsetAsync(h->cls, kGeneral, (size_t)vol(h), h->stream));
        }
        CUDA_TRY(launch_node_class(h->g, h->mat, h->d_lumped, h->n_lumped_edges, h->has_design ? h->dbox : nullptr, h->cls,
                                   h->stream));
        rc = build_plates(h);
        if (rc) return rc;
        if (h->n_plate_nodes > 0) CUDA_TRY(launch_class_nodes(h->g, h->d_plate_nodes, h->n_plate_nodes, kPlateNode, h->cls, h->stream));
        rc = build_interface_rows(h);
        if (rc) return rc;
    }
    if (h->dirty_probes) {
        int rc = build_probes(h);
        if (rc) return rc;
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->prepared = true;
    return FDTD_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// fdtd_step_static_scratch: the fused sweep with its ping-pong target in a static device array.
//
// fdtd_step under FDTD_SCHEDULE_FUSED allocates a second field set, a second CPML set and the work
// list on its first call. Callers that cannot allocate while stepping (device memory reserved in
// full by their own pool; loops that must not let cudaMalloc / cudaFree synchronise the device)
// use this entry point instead: the same kernels alternate between the handle's buffers and a
// fixed array of FDTD_STEP_STATIC_SCRATCH_BYTES, and no device memory is allocated.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr size_t kStaticScratchBytes = FDTD_STEP_STATIC_SCRATCH_BYTES;
constexpr size_t kScratchAlign = 256;  // TMA needs 16-byte aligned bases; keep each piece on 256 B
constexpr int kMaxScratchDevices = 64;

// One per device and process; zero-initialised at module load, but no call relies on its contents.
static __device__ __align__(256) unsigned char g_step_scratch[kStaticScratchBytes];

std::mutex g_scratch_mu;
unsigned char* g_scratch_addr[kMaxScratchDevices] = {};
bool g_scratch_configured[kMaxScratchDevices] = {};

size_t align_up(size_t v) { return (v + kScratchAlign - 1) / kScratchAlign * kScratchAlign; }

// Offsets of the pieces of the scratch for handle h: 6 fields, 24 CPML arrays, work list.
struct ScratchLayout {
    size_t field[6];
    size_t psi[6][4];
    size_t items;
    size_t total;
};

ScratchLayout scratch_layout(const fdtd_handle* h, size_t n_items) {
    ScratchLayout L{};
    size_t off = 0;
    const size_t fb = align_up((size_t)vol(h) * sizeof(float));
    for (int c = 0; c < 6; ++c, off += fb) L.field[c] = off;
    for (int f = 0; f < 6; ++f) {
        const size_t pb = align_up((size_t)h->psi_elems[f] * sizeof(float));
        for (int q = 0; q < 4; ++q, off += pb) L.psi[f][q] = off;
    }
    L.items = off;
    off += align_up(n_items * sizeof(int4));
    L.total = off;
    return L;
}

// Address of the scratch on `dev` (the current device) and the sweep's shared-memory limit, set
// once per device.
int scratch_setup(int dev, unsigned char** base) {
    if (dev < 0 || dev >= kMaxScratchDevices) return fail(FDTD_ERR_STATE, "device ordinal outside the static scratch table");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* a = nullptr;
        CUDA_TRY(cudaGetSymbolAddress(&a, g_step_scratch));
        g_scratch_addr[dev] = (unsigned char*)a;
    }
    if (!g_scratch_configured[dev]) {
        CUDA_TRY(fused_configure());
        g_scratch_configured[dev] = true;
    }
    *base = g_scratch_addr[dev];
    return FDTD_OK;
}

}  // namespace

extern "C" int fdtd_step_static_scratch(fdtd_handle* h, int64_t n) {
    if (!h) return fail(FDTD_ERR_INVALID, "handle is NULL");
    if (n < 0) return fail(FDTD_ERR_INVALID, "negative step count");
    // preparation allocates (coefficient, lumped and probe tables): it must be done already
    if (!h->prepared || h->dirty_materials || h->dirty_lumped || h->dirty_probes)
        return fail(FDTD_ERR_STATE, "fdtd_step_static_scratch needs a prepared handle: call fdtd_prepare after the last "
                                    "change to materials, lumped elements or probes");
    int dev = -1;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev != h->device) return fail(FDTD_ERR_STATE, "the current device is not the handle's device");
    if (!h->static_planned) {  // planning, as for the fused schedule; host memory only
        FusedPlan plan;
        const PlanGrid pg = plan_grid(h->g);
        plan_fused(pg, plan_chunk(pg), h->has_design ? h->dbox : nullptr, plan);  // no CPML items: shell only
        const std::vector<PlanItem> all = flatten(plan, h->static_counts);
        if (h->static_items) CUDA_TRY(cudaFreeHost(h->static_items));
        h->static_items = nullptr;
        h->static_n_items = 0;
        if (!all.empty()) {
            CUDA_TRY(cudaHostAlloc((void**)&h->static_items, all.size() * sizeof(int4), cudaHostAllocDefault));
            std::memcpy(h->static_items, all.data(), all.size() * sizeof(int4));
        }
        h->static_n_items = all.size();
        h->static_planned = true;
    }
    const ScratchLayout L = scratch_layout(h, h->static_n_items);
    if (L.total > kStaticScratchBytes)
        return fail(FDTD_ERR_RANGE, "grid needs " + std::to_string(L.total) + " bytes of step scratch; the static scratch holds " +
                                        std::to_string(kStaticScratchBytes) + " (about a 64^3 grid with 10-cell CPML)");
    unsigned char* base = nullptr;
    int rc = scratch_setup(dev, &base);
    if (rc) return rc;
    if (n == 0) return FDTD_OK;

    void* enc = tensor_map_encoder();
    if (!enc) return fail(FDTD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const int a = h->cur;
    float* sf[6];
    for (int c = 0; c < 6; ++c) sf[c] = (float*)(base + L.field[c]);
    PsiSet sp{};
    for (int f = 0; f < 6; ++f) {
        sp.f[f].e[0] = h->psi_elems[f] ? (float*)(base + L.psi[f][0]) : nullptr;
        sp.f[f].e[1] = h->psi_elems[f] ? (float*)(base + L.psi[f][1]) : nullptr;
        sp.f[f].h[0] = h->psi_elems[f] ? (float*)(base + L.psi[f][2]) : nullptr;
        sp.f[f].h[1] = h->psi_elems[f] ? (float*)(base + L.psi[f][3]) : nullptr;
    }
    FusedMaps maps_h, maps_s;  // tensor maps (host structs) of the handle's buffer and the scratch
    {
        float* hh[3] = {h->field[a][3], h->field[a][4], h->field[a][5]};
        float* ee[3] = {h->field[a][0], h->field[a][1], h->field[a][2]};
        float* sh[3] = {sf[3], sf[4], sf[5]};
        float* se[3] = {sf[0], sf[1], sf[2]};
        if (encode_fused_maps(&maps_h, h->g, hh, ee, h->rec, enc) != 0 ||
            encode_fused_maps(&maps_s, h->g, sh, se, h->rec, enc) != 0)
            return fail(FDTD_ERR_CUDA, "tensor map encoding failed");
    }
    int4* d_items = (int4*)(base + L.items);
    const size_t n_items = h->static_n_items;
    if (n_items) CUDA_TRY(cudaMemcpyAsync(d_items, h->static_items, n_items * sizeof(int4), cudaMemcpyHostToDevice, h->stream));
    const FusedWork w = work_of(d_items, h->static_counts);
    // With an odd count the result ends in the scratch and is copied back whole, so the scratch's
    // CPML arrays start as copies of the handle's: the elements no step writes then agree. With an
    // even count the last step writes the handle's own buffers and the scratch needs no copy.
    for (int f = 0; f < 6 && (n & 1); ++f) {
        const size_t nb = (size_t)h->psi_elems[f] * sizeof(float);
        if (!nb) continue;
        float* src[4];
        psi_arrays(h, a, f, src);
        const float* dst[4] = {sp.f[f].e[0], sp.f[f].e[1], sp.f[f].h[0], sp.f[f].h[1]};
        for (int q = 0; q < 4; ++q) CUDA_TRY(cudaMemcpyAsync((void*)dst[q], src[q], nb, cudaMemcpyDeviceToDevice, h->stream));
    }
    const StepParams p = make_params(h);
    const FieldPtrs fh{h->field[a][0], h->field[a][1], h->field[a][2], h->field[a][3], h->field[a][4], h->field[a][5]};
    const FieldPtrs fs{sf[0], sf[1], sf[2], sf[3], sf[4], sf[5]};
    for (int64_t s = 0; s < n; ++s) {
        if ((s & 1) == 0) CUDA_TRY(launch_fused(maps_h, p, fh, fs, h->psi[a], sp, h->step, w, h->stream));
        else CUDA_TRY(launch_fused(maps_s, p, fs, fh, sp, h->psi[a], h->step, w, h->stream));
        ++h->step;
    }
    if (n & 1) {  // the last step wrote the scratch: copy the state back into the handle's buffers
        // only the nx columns of each row: the sweep never writes the row padding
        const DeviceGrid& g = h->g;
        for (int c = 0; c < 6; ++c)
            CUDA_TRY(cudaMemcpy2DAsync(h->field[a][c], (size_t)g.pitch * 4, sf[c], (size_t)g.pitch * 4, (size_t)g.nx * 4,
                                       (size_t)g.ny * g.nz, cudaMemcpyDeviceToDevice, h->stream));
        for (int f = 0; f < 6; ++f) {
            const size_t nb = (size_t)h->psi_elems[f] * sizeof(float);
            if (!nb) continue;
            float* dst[4];
            psi_arrays(h, a, f, dst);
            const float* src[4] = {sp.f[f].e[0], sp.f[f].e[1], sp.f[f].h[0], sp.f[f].h[1]};
            for (int q = 0; q < 4; ++q) CUDA_TRY(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyDeviceToDevice, h->stream));
        }
    }
    return FDTD_OK;
}

// ---------------------------------------------------------------------------------------------
// Design region and discrete adjoint (no reference counterpart).
// ---------------------------------------------------------------------------------------------
extern "C" int fdtd_set_design_region(fdtd_handle* h, const int32_t box[6], const fdtd_material* base, const float* eps_r) {
    if (!h || !box || !base || !eps_r) return fail(FDTD_ERR_INVALID, "NULL argument");
    const DeviceGrid& g = h->g;
    const int lo[3] = {std::max(g.pxn, 1), std::max(g.pyn, 1), std::max(g.pzn, 1)};
    const int hi[3] = {std::min(g.nx - 1 - g.pxp, g.nx - 2), std::min(g.ny - 1 - g.pyp, g.ny - 2),
                       std::min(g.nz - 1 - g.pzp, g.nz - 2)};
    // the E edges of the cells [b0, b3) lie on nodes b0..b3 of each axis: all must be interior nodes
    for (int a = 0; a < 3; ++a)
        if (box[a] >= box[a + 3] || box[a] < lo[a] || box[a + 3] > hi[a])
            return fail(FDTD_ERR_INVALID, "design box empty, or its edges reach the CPML slabs or the boundary planes");
    if (!(base->mu_r > 0.f) || !(base->sigma_e >= 0.f) || !(base->sigma_m > 0.f))
        return fail(FDTD_ERR_INVALID, "design base material: mu_r > 0, sigma_e >= 0, sigma_m > 0");
    if ((int)h->materials.size() > kDesign)
        return fail(FDTD_ERR_INVALID, "material index 255 is reserved for the design region: at most 255 materials");
    if (!h->plates.empty()) return fail(FDTD_ERR_STATE, "a design region cannot be combined with plates");
    for (const LumpedDef& L : h->lumped)
        if (L.axis != 2)
            return fail(FDTD_ERR_STATE, "a design region cannot be combined with x-directed lumped elements");
    for (const LumpedDef& L : h->lumped) {  // the cells of a lumped Ez edge (i,j): i-1..i, j-1..j
        const int* b = L.box;
        if (b[0] - 1 < box[3] && box[0] <= b[3] && b[1] - 1 < box[4] && box[1] <= b[4] && b[2] < box[5] && box[2] < b[5])
            return fail(FDTD_ERR_INVALID, "a lumped element touches the design region");
    }
    const size_t nd = (size_t)(box[3] - box[0]) * (box[4] - box[1]) * (box[5] - box[2]);
    for (size_t q = 0; q < nd; ++q)
        if (!(eps_r[q] > 0.f) || !std::isfinite(eps_r[q])) return fail(FDTD_ERR_INVALID, "design eps_r must be positive");
    const bool same = h->has_design && std::equal(box, box + 6, h->dbox);
    if (!same) {
        h->release(h->d_deps);
        h->d_deps = nullptr;
        CUDA_TRY(h->alloc((void**)&h->d_deps, nd * sizeof(float)));
        int b[6];
        for (int q = 0; q < 6; ++q) b[q] = box[q];
        CUDA_TRY(launch_paint(h->mat, g, b, (uint8_t)kDesign, h->stream));
        std::copy(box, box + 6, h->dbox);
    }
    CUDA_TRY(cudaMemcpyAsync(h->d_deps, eps_r, nd * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->design_base = *base;
    h->has_design = true;
    h->replan = true;            // fused work items
    h->static_planned = false;   // and those of fdtd_step_static_scratch
    h->dirty_materials = true;  // table entry 255, node classes
    h->adj.ready = false;
    return FDTD_OK;
}

namespace {

int adj_alloc(fdtd_handle* h, void** p, size_t n) {
    CUDA_TRY(h->alloc(p, n));
    h->adj.bufs.push_back(*p);
    return FDTD_OK;
}

long long edge_box_volume(const int* d) { return (long long)(d[3] - d[0] + 1) * (d[4] - d[1] + 1) * (d[5] - d[2] + 1); }

// Interval S of the box checkpoints inside a segment of K steps (0: none). The segment recompute
// needs only the design region's E, so it sweeps the cone of nodes that E depends on (see
// adj_recompute_step); a copy of the fields over the design edge box grown by S nodes, saved by
// the forward every S steps, restarts that cone with a reach below S. S is the largest value up
// to kAdjSubMax whose box holds interior nodes only (no CPML memory, no boundary plane), used
// only when it splits a segment.
constexpr int kAdjSubMax = 16;
int adj_sub_interval(const fdtd_handle* h, int K) {
    const DeviceGrid& g = h->g;
    const int* d = h->dbox;
    auto lo = [](int pn) { return std::max(pn, 1); };
    auto hi = [](int nn, int pp) { return std::min(nn - 1 - pp, nn - 2); };
    const int gap = std::min({kAdjSubMax, d[0] - lo(g.pxn), hi(g.nx, g.pxp) - d[3], d[1] - lo(g.pyn),
                              hi(g.ny, g.pyp) - d[4], d[2] - lo(g.pzn), hi(g.nz, g.pzp) - d[5]});
    return (K > 0 && gap >= 1 && gap < K) ? gap : 0;
}

// Buffers of an adjoint run of n steps with checkpoint interval K.
int adj_prepare(fdtd_handle* h, long long n, int K) {
    auto& A = h->adj;
    // a run of the same length, interval and design box reuses the buffers: freeing device or
    // pinned memory synchronises the whole device, which would serialise batched runs
    const long long key[8] = {n, K, h->dbox[0], h->dbox[1], h->dbox[2], h->dbox[3], h->dbox[4], h->dbox[5]};
    if (!A.bufs.empty() && A.pinned_samples && std::equal(key, key + 8, A.key)) {
        A.ready = false;
        return FDTD_OK;
    }
    for (void* p : A.bufs) h->release(p);
    A.bufs.clear();
    if (A.pinned_samples) cudaFreeHost(A.pinned_samples);
    if (A.pinned_grad) cudaFreeHost(A.pinned_grad);
    A.pinned_samples = nullptr;
    A.pinned_grad = nullptr;
    const cudaStream_t rev = A.rev;  // kept across runs
    cudaEvent_t ev[5];
    std::copy(A.ev, A.ev + 5, ev);
    A = fdtd_handle::Adjoint{};
    A.rev = rev;
    std::copy(ev, ev + 5, A.ev);
    const size_t V = (size_t)vol(h) * sizeof(float);
    int rc;
    for (int c = 0; c < 6; ++c) {
        if ((rc = adj_alloc(h, (void**)&A.st.l[c], V)) || (rc = adj_alloc(h, (void**)&A.st.ge[c], V)) ||
            (rc = adj_alloc(h, (void**)&A.st.gh[c], V)))
            return rc;
    }
    for (int f = 0; f < 6; ++f) {
        const size_t pn = (size_t)h->psi_elems[f] * sizeof(float);
        float* arr[4] = {nullptr, nullptr, nullptr, nullptr};
        for (int q = 0; q < 4 && pn; ++q)
            if ((rc = adj_alloc(h, (void**)&arr[q], pn))) return rc;
        A.psa.f[f].e[0] = arr[0]; A.psa.f[f].e[1] = arr[1]; A.psa.f[f].h[0] = arr[2]; A.psa.f[f].h[1] = arr[3];
    }
    const long long ne = edge_box_volume(h->dbox);
    // K > 0: two segments of snapshots, so that the backward recomputes one segment while it
    // reverses the next
    A.hist_slots = K > 0 ? 2 * ((long long)K + 1) : n + 1;
    A.ckpt_slots = K > 0 ? (n + K - 1) / K + 1 : 1;  // + the final state
    const size_t nd = (size_t)(h->dbox[3] - h->dbox[0]) * (h->dbox[4] - h->dbox[1]) * (h->dbox[5] - h->dbox[2]);
    if ((rc = adj_alloc(h, (void**)&A.samples, sizeof(float) * (size_t)std::max<long long>(n, 1))) ||
        (rc = adj_alloc(h, (void**)&A.hist, sizeof(float) * 3 * (size_t)ne * (size_t)A.hist_slots)) ||
        (rc = adj_alloc(h, (void**)&A.ckpt, (size_t)fdtd_state_bytes(h) * (size_t)A.ckpt_slots)) ||
        (rc = adj_alloc(h, (void**)&A.acc, sizeof(double) * 3 * (size_t)ne)) ||
        (rc = adj_alloc(h, (void**)&A.grad, sizeof(double) * nd)) ||
        (rc = adj_alloc(h, (void**)&A.no_probe_k, sizeof(int) * (size_t)(h->g.nz + 1))))
        return rc;
    CUDA_TRY(cudaMemsetAsync(A.no_probe_k, 0, sizeof(int) * (size_t)(h->g.nz + 1), h->stream));
    A.S = adj_sub_interval(h, K);
    if (A.S > 0) {
        const int S = A.S;
        const int* d = h->dbox;
        A.sub_box = NodeBox{d[0] - S, d[1] - S, d[2] - S, d[3] + 1 + S, d[4] + 1 + S, d[5] + 1 + S};
        A.sub_per_seg = (K - 1) / S;
        const size_t box = (size_t)(A.sub_box.x1 - A.sub_box.x0) * (A.sub_box.y1 - A.sub_box.y0) *
                           (A.sub_box.z1 - A.sub_box.z0);
        const size_t slots = (size_t)((n + K - 1) / K) * (size_t)A.sub_per_seg;
        if (adj_alloc(h, (void**)&A.sub, sizeof(float) * 6 * box * slots) != FDTD_OK) {
            cudaGetLastError();  // no room: the recompute sweeps the whole cone from the checkpoint
            A.S = 0;
            A.sub_per_seg = 0;
        }
    }
    CUDA_TRY(cudaMallocHost((void**)&A.pinned_samples, sizeof(float) * (size_t)std::max<long long>(n, 1)));
    CUDA_TRY(cudaMallocHost((void**)&A.pinned_grad, sizeof(double) * std::max<size_t>(nd, 1)));
    A.n = n;
    A.K = K;
    std::copy(key, key + 8, A.key);
    return FDTD_OK;
}

// Box checkpoint q (1 .. sub_per_seg: at step q * S of the segment) of segment sg.
float* adj_sub(fdtd_handle* h, long long sg, long long q) {
    const NodeBox& b = h->adj.sub_box;
    const size_t box = (size_t)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
    return h->adj.sub + (size_t)(sg * h->adj.sub_per_seg + q - 1) * 6 * box;
}
FieldPtrs cur_fields(fdtd_handle* h) {
    const int c = h->cur;
    return FieldPtrs{h->field[c][0], h->field[c][1], h->field[c][2], h->field[c][3], h->field[c][4], h->field[c][5]};
}
float* adj_slot(fdtd_handle* h, long long s) { return h->adj.hist + (size_t)s * 3 * (size_t)edge_box_volume(h->dbox); }
char* adj_ckpt(fdtd_handle* h, long long s) { return h->adj.ckpt + (size_t)s * (size_t)fdtd_state_bytes(h); }

// One forward step followed by the FoM sample (sample may be NULL) and an optional design snapshot.
int adj_forward_step(fdtd_handle* h, float* sample, float* snap) {
    int rc = fdtd_step(h, 1);
    if (rc) return rc;
    const int c = h->cur;
    CUDA_TRY(launch_after_step(h->field[c][0], h->field[c][1], h->field[c][2], h->g, h->adj.probe, sample, h->dbox, snap,
                               h->stream));
    return FDTD_OK;
}

// One step of a segment recompute (K > 0). The backward needs only the design region's E of each
// recomputed step, and E at the design edge box D after the segment's step t depends only on the
// segment's starting state within D grown by (segment length - t) nodes on every side: one step
// of the Yee update reads a node's neighbours one node away along each axis (E the lower H
// neighbours, H the upper E neighbours). So step t updates only that box (`reach` = length - t,
// clipped to the grid): the nodes inside take the same bits as in a whole-grid step, and those
// outside are stale but never read again within the segment. Probes sample nothing (pr has no
// probe planes): the ring keeps the forward's samples.
int adj_recompute_step(fdtd_handle* h, const StepParams& pr, long long reach, float* snap) {
    const DeviceGrid& g = h->g;
    const int* d = h->dbox;
    const int e = (int)std::min<long long>(reach, 1LL << 20);
    const NodeBox b{std::max(0, d[0] - e), std::max(0, d[1] - e), std::max(0, d[2] - e),
                    std::min(g.nx, d[3] + 1 + e), std::min(g.ny, d[4] + 1 + e), std::min(g.nz, d[5] + 1 + e)};
    const int c = h->cur;
    const FieldPtrs f{h->field[c][0], h->field[c][1], h->field[c][2], h->field[c][3], h->field[c][4], h->field[c][5]};
    StepParams q = pr;
    q.design_snap = snap;  // k_design_e writes the design region's E of the step
    CUDA_TRY(launch_two_pass_box(q, f, h->psi[c], b, h->step, h->stream));
    ++h->step;
    return FDTD_OK;
}

}  // namespace

namespace {

// The forward of an adjoint run, enqueued on the handle's stream without waiting: validation,
// buffers, checkpoints, the steps with their FoM samples and design snapshots, the samples' copy
// to pinned host memory. adj_forward_finish waits for it.
int adj_check(const fdtd_handle* h, int64_t n, int32_t checkpoint_every, int32_t pi, int32_t pj, int32_t pk) {
    if (!h->has_design) return fail(FDTD_ERR_STATE, "no design region (fdtd_set_design_region)");
    if (n < 1 || checkpoint_every < 0) return fail(FDTD_ERR_INVALID, "steps >= 1 and checkpoint interval >= 0 required");
    const DeviceGrid& g = h->g;
    if (pi < 1 || pi > g.nx - 2 || pj < 1 || pj > g.ny - 2 || pk < 0 || pk > g.nz - 2)
        return fail(FDTD_ERR_INVALID, "FoM probe must be an updated Ez edge");
    if (in_slab_host(pi, g.nx, g.pxn, g.pxp) || in_slab_host(pj, g.ny, g.pyn, g.pyp) || in_slab_host(pk, g.nz, g.pzn, g.pzp))
        return fail(FDTD_ERR_INVALID, "FoM probe inside the CPML");
    return FDTD_OK;
}

int adj_forward_enqueue(fdtd_handle* h, int64_t n, int32_t checkpoint_every, int32_t pi, int32_t pj, int32_t pk) {
    int rc = adj_check(h, n, checkpoint_every, pi, pj, pk);
    if (rc) return rc;
    const DeviceGrid& g = h->g;
    rc = ensure_prepared(h);
    if (rc) return rc;
    const int K = checkpoint_every;
    rc = adj_prepare(h, n, K);
    if (rc) return rc;
    auto& A = h->adj;
    A.start = h->step;
    A.probe = (long long)pk * g.plane + (long long)pj * g.pitch + pi;
    if (K == 0) {  // design E before the first step
        const int c = h->cur;
        CUDA_TRY(launch_after_step(h->field[c][0], h->field[c][1], h->field[c][2], g, A.probe, nullptr, h->dbox, adj_slot(h, 0),
                                   h->stream));
    }
    // one step per fdtd_step call never runs AUTO's trial: apply its direct choice (large grids
    // with mostly interior tiles take fused) before stepping
    if (h->schedule == FDTD_SCHEDULE_AUTO && h->auto_choice == FDTD_SCHEDULE_AUTO &&
        (long long)g.nx * g.ny * g.nz >= kAutoTrialCells)
        auto_direct(h);
    // two-pass steps take their records in k_design_e (no launch of their own): the E of the
    // design edge box is final there, and so is every other E
    const bool two_pass = !use_fused(h);
    StepParams pa = make_params(h);
    if (two_pass) {
        const int* d = h->dbox;
        const bool in_box = pi >= d[0] && pi <= d[3] && pj >= d[1] && pj <= d[4] && pk >= d[2] && pk <= d[5];
        pa.fom_node = in_box ? A.probe : -1;
        pa.fom_read = in_box ? -1 : A.probe;
    }
    for (long long s = 0; s < n; ++s) {
        if (K > 0 && s % K == 0) {
            if ((rc = state_copy(h, adj_ckpt(h, s / K), true))) return rc;
        } else if (A.S > 0 && (s % K) % A.S == 0) {
            CUDA_TRY(launch_box_state(cur_fields(h), g, A.sub_box, adj_sub(h, s / K, (s % K) / A.S), true, h->stream));
        }
        if (two_pass) {
            pa.fom_sample = A.samples + s;
            pa.design_snap = K == 0 ? adj_slot(h, s + 1) : nullptr;
            CUDA_TRY(launch_two_pass(pa, cur_fields(h), h->psi[h->cur], h->step, h->stream));
            ++h->step;
        } else if ((rc = adj_forward_step(h, A.samples + s, K == 0 ? adj_slot(h, s + 1) : nullptr))) {
            return rc;
        }
    }
    if ((rc = state_copy(h, adj_ckpt(h, A.ckpt_slots - 1), true))) return rc;  // final state
    CUDA_TRY(cudaMemcpyAsync(A.pinned_samples, A.samples, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    return FDTD_OK;
}

int adj_forward_finish(fdtd_handle* h, double* J) {
    auto& A = h->adj;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    A.host_samples.assign(A.pinned_samples, A.pinned_samples + A.n);
    double sum = 0.0;
    for (float v : A.host_samples) sum += (double)h->g.dt * (double)v * (double)v;
    *J = sum;
    A.ready = true;
    return FDTD_OK;
}

// The reverse sweep, enqueued without waiting (the reversal's own stream and events live in the
// handle): cleared adjoint state, the reverse steps (with segment recomputes for K > 0), the
// gradient into pinned host memory, the forward's final state restored. adj_backward_finish
// waits for it.
int adj_backward_enqueue(fdtd_handle* h) {
    auto& A = h->adj;
    if (!A.ready) return fail(FDTD_ERR_STATE, "no fdtd_adjoint_forward since the last change");
    const size_t V = (size_t)vol(h) * sizeof(float);
    for (int c = 0; c < 6; ++c) {
        CUDA_TRY(cudaMemsetAsync(A.st.l[c], 0, V, h->stream));
        CUDA_TRY(cudaMemsetAsync(A.st.ge[c], 0, V, h->stream));
        CUDA_TRY(cudaMemsetAsync(A.st.gh[c], 0, V, h->stream));
    }
    for (int f = 0; f < 6; ++f) {
        const size_t pn = (size_t)h->psi_elems[f] * sizeof(float);
        if (!pn) continue;
        CUDA_TRY(cudaMemsetAsync(A.psa.f[f].e[0], 0, pn, h->stream));
        CUDA_TRY(cudaMemsetAsync(A.psa.f[f].e[1], 0, pn, h->stream));
        CUDA_TRY(cudaMemsetAsync(A.psa.f[f].h[0], 0, pn, h->stream));
        CUDA_TRY(cudaMemsetAsync(A.psa.f[f].h[1], 0, pn, h->stream));
    }
    const long long ne = edge_box_volume(h->dbox);
    CUDA_TRY(cudaMemsetAsync(A.acc, 0, sizeof(double) * 3 * (size_t)ne, h->stream));
    const StepParams p = make_params(h);
    const float two_dt = 2.0f * h->g.dt;
    int rc;
    if (A.K == 0) {
        for (long long m = A.n - 1; m >= 0; --m) {
            const AdjStep st{A.probe, two_dt * A.host_samples[(size_t)m], A.acc, adj_slot(h, m), adj_slot(h, m + 1)};
            CUDA_TRY(launch_adj_step(p, A.st, A.psa, st, h->stream));
        }
    } else {
        // Segments are recomputed on the handle's stream (forward fields) and reversed on a second
        // stream (adjoint state), one segment apart: the recompute of segment sg - 1 runs while
        // segment sg is reversed. Snapshot buffers alternate by segment parity; events order a
        // reversal after its recompute and a recompute after the reversal that last read its
        // buffer.
        if (!A.rev) {
            CUDA_TRY(cudaStreamCreateWithFlags(&A.rev, cudaStreamNonBlocking));
            for (cudaEvent_t& e : A.ev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        StepParams pr = p;
        pr.probe_k = A.no_probe_k;
        const long long nseg = (A.n + A.K - 1) / A.K;
        const long long half = (long long)A.K + 1;
        auto slot = [&](long long sg, long long t) { return adj_slot(h, (sg & 1) * half + t); };
        cudaEvent_t* ev_rec = A.ev;
        cudaEvent_t* ev_rev = A.ev + 2;
        CUDA_TRY(cudaEventRecord(A.ev[4], h->stream));  // the adjoint state is cleared
        CUDA_TRY(cudaStreamWaitEvent(A.rev, A.ev[4], 0));
        auto recompute = [&](long long sg) -> int {
            int r = state_copy(h, adj_ckpt(h, sg), false);
            if (r) return r;
            h->step = A.start + sg * A.K;
            const long long len = std::min<long long>(A.K, A.n - sg * A.K);
            const int c = h->cur;
            CUDA_TRY(launch_after_step(h->field[c][0], h->field[c][1], h->field[c][2], h->g, A.probe, nullptr, h->dbox,
                                       slot(sg, 0), h->stream));
            for (long long t = 0; t < len; ++t) {
                if (A.S > 0 && t > 0 && t % A.S == 0)
                    CUDA_TRY(launch_box_state(cur_fields(h), h->g, A.sub_box, adj_sub(h, sg, t / A.S), false, h->stream));
                // the cone ends at the next box checkpoint (or the segment's end)
                const long long te = A.S > 0 ? std::min<long long>(len, (t / A.S + 1) * A.S) : len;
                if ((r = adj_recompute_step(h, pr, te - 1 - t, slot(sg, t + 1)))) return r;
            }
            CUDA_TRY(cudaEventRecord(ev_rec[sg & 1], h->stream));
            return FDTD_OK;
        };
        if ((rc = recompute(nseg - 1))) return rc;
        for (long long sg = nseg - 1; sg >= 0; --sg) {
            CUDA_TRY(cudaStreamWaitEvent(A.rev, ev_rec[sg & 1], 0));
            const long long len = std::min<long long>(A.K, A.n - sg * A.K);
            for (long long t = len - 1; t >= 0; --t) {
                const AdjStep st{A.probe, two_dt * A.host_samples[(size_t)(sg * A.K + t)], A.acc, slot(sg, t), slot(sg, t + 1)};
                CUDA_TRY(launch_adj_step(p, A.st, A.psa, st, A.rev));
            }
            CUDA_TRY(cudaEventRecord(ev_rev[sg & 1], A.rev));
            if (sg > 0) {
                // segment sg - 1 reuses the buffers segment sg + 1 was reversed from
                if (sg + 1 < nseg) CUDA_TRY(cudaStreamWaitEvent(h->stream, ev_rev[(sg + 1) & 1], 0));
                if ((rc = recompute(sg - 1))) return rc;
            }
        }
        CUDA_TRY(cudaEventRecord(A.ev[4], A.rev));
        CUDA_TRY(cudaStreamWaitEvent(h->stream, A.ev[4], 0));
    }
    CUDA_TRY(launch_grad_finalize(A.acc, h->dbox, A.grad, h->stream));
    const size_t nd = (size_t)(h->dbox[3] - h->dbox[0]) * (h->dbox[4] - h->dbox[1]) * (h->dbox[5] - h->dbox[2]);
    CUDA_TRY(cudaMemcpyAsync(A.pinned_grad, A.grad, sizeof(double) * nd, cudaMemcpyDeviceToHost, h->stream));
    // leave the handle where the forward left it
    if (A.K > 0) {
        if ((rc = state_copy(h, adj_ckpt(h, A.ckpt_slots - 1), false))) return rc;
        h->step = A.start + A.n;
    }
    return FDTD_OK;
}

int adj_backward_finish(fdtd_handle* h, double* grad) {
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    const size_t nd = (size_t)(h->dbox[3] - h->dbox[0]) * (h->dbox[4] - h->dbox[1]) * (h->dbox[5] - h->dbox[2]);
    std::memcpy(grad, h->adj.pinned_grad, sizeof(double) * nd);
    return FDTD_OK;
}

}  // namespace

extern "C" int fdtd_adjoint_forward(fdtd_handle* h, int64_t n, int32_t checkpoint_every, int32_t pi, int32_t pj, int32_t pk,
                                    double* J) {
    if (!h || !J) return fail(FDTD_ERR_INVALID, "NULL argument");
    int rc = adj_forward_enqueue(h, n, checkpoint_every, pi, pj, pk);
    return rc ? rc : adj_forward_finish(h, J);
}

extern "C" int fdtd_adjoint_backward(fdtd_handle* h, double* grad) {
    if (!h || !grad) return fail(FDTD_ERR_INVALID, "NULL argument");
    int rc = adj_backward_enqueue(h);
    return rc ? rc : adj_backward_finish(h, grad);
}

// Forward and backward of many handles: every handle's work is enqueued before any is waited for,
// so handles on different streams run concurrently; the results equal per-handle calls.
extern "C" int fdtd_batch_adjoint(fdtd_handle* const* handles, int32_t n, int64_t steps, int32_t checkpoint_every,
                                  const int32_t* probes, double* J, double* const* grads) {
    if (!handles || !probes || !J || !grads || n < 1) return fail(FDTD_ERR_INVALID, "NULL argument or no handles");
    for (int q = 0; q < n; ++q) {
        if (!handles[q] || !grads[q]) return fail(FDTD_ERR_INVALID, "NULL handle or gradient");
        for (int r = 0; r < q; ++r)
            if (handles[r] == handles[q]) return fail(FDTD_ERR_INVALID, "a handle appears twice");
    }
    int rc;
    for (int q = 0; q < n; ++q)  // nothing is enqueued unless every handle's arguments hold
        if ((rc = adj_check(handles[q], steps, checkpoint_every, probes[3 * q], probes[3 * q + 1], probes[3 * q + 2])))
            return rc;
    for (int q = 0; q < n; ++q)
        if ((rc = adj_forward_enqueue(handles[q], steps, checkpoint_every, probes[3 * q], probes[3 * q + 1], probes[3 * q + 2])))
            return rc;
    for (int q = 0; q < n; ++q)
        if ((rc = adj_forward_finish(handles[q], J + q))) return rc;
    for (int q = 0; q < n; ++q)
        if ((rc = adj_backward_enqueue(handles[q]))) return rc;
    for (int q = 0; q < n; ++q)
        if ((rc = adj_backward_finish(handles[q], grads[q]))) return rc;
    return FDTD_OK;
}

// ---------------------------------------------------------------------------------------------
// Batched persistent launch (no reference counterpart).
// ---------------------------------------------------------------------------------------------
struct fdtd_batch {
    std::vector<fdtd_handle*> hs;
    int device = 0;
    cudaStream_t stream = nullptr;      // launch stream (graph capture needs a non-default one)
    cudaStream_t own_stream = nullptr;
    std::vector<BatchInstance> inst;    // host copy, refreshed before each launch
    BatchInstance* d_inst = nullptr;
    int* d_order = nullptr;
    int* d_queue = nullptr;
    int cluster = 4, threads = 256, n_clusters = 0;  // cluster 0: flat per-step form; -1: chains
    int4* d_items = nullptr;            // flat form: {instance, x0, y0, k} per 32 x 8 block
    int n_items = 0;
    struct Graph {
        long long steps;
        int cfg[3];
        cudaGraph_t graph;
        cudaGraphExec_t exec;
    };
    std::vector<Graph> graphs;          // captured launches by step count and configuration
    // chain form: one stream per instance while capturing, the events that fork and join them,
    // and a signature of the descriptors the captured graphs bake in
    std::vector<cudaStream_t> chain_streams;
    std::vector<cudaEvent_t> chain_events;  // [0]: fork, [1 + q]: join of instance q
    unsigned long long chain_sig = 0;
};

namespace {

void batch_drop_graph(fdtd_batch* b) {
    for (auto& G : b->graphs) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        if (G.graph) cudaGraphDestroy(G.graph);
    }
    b->graphs.clear();
}

// Instance descriptors from the handles' current in-place buffers and steps.
int batch_refresh(fdtd_batch* b) {
    for (size_t q = 0; q < b->hs.size(); ++q) {
        fdtd_handle* h = b->hs[q];
        int rc = ensure_prepared(h);
        if (rc) return rc;
        if (h->stream != b->stream) CUDA_TRY(cudaStreamSynchronize(h->stream));  // the handle's own work first
        const int a = h->cur;
        BatchInstance& I = b->inst[q];
        I.p = make_params(h);
        I.f = FieldPtrs{h->field[a][0], h->field[a][1], h->field[a][2], h->field[a][3], h->field[a][4], h->field[a][5]};
        I.ps = h->psi[a];
        I.step = h->step;
    }
    CUDA_TRY(cudaMemcpyAsync(b->d_inst, b->inst.data(), sizeof(BatchInstance) * b->inst.size(), cudaMemcpyHostToDevice,
                             b->stream));
    return FDTD_OK;
}

int batch_set_config(fdtd_batch* b, int cluster, int threads) {
    if (cluster == -1) {  // chains: each instance's own two-pass kernels, instances concurrent
        if (threads != 256) return fail(FDTD_ERR_INVALID, "the chain form (cluster -1) runs 256 threads per CTA");
        b->cluster = -1;
        b->threads = 256;
        b->n_clusters = 0;
        return FDTD_OK;
    }
    if (cluster == 0) {  // flat per-step kernels: 256 threads per CTA
        if (threads != 256) return fail(FDTD_ERR_INVALID, "the flat form (cluster 0) runs 256 threads per CTA");
        b->cluster = 0;
        b->threads = 256;
        b->n_clusters = 0;
        return FDTD_OK;
    }
    if (!batch_threads_supported(threads) || (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8))
        return fail(FDTD_ERR_INVALID, "cluster size 0 (flat), 1, 2, 4 or 8 and 128, 256 or 512 threads per CTA");
    int n = 0;
    CUDA_TRY(batch_max_clusters(cluster, threads, &n));
    if (n < 1) return fail(FDTD_ERR_CUDA, "no cluster of this shape fits on the device");
    b->cluster = cluster;
    b->threads = threads;
    b->n_clusters = std::min<int>(n, (int)b->hs.size());
    return FDTD_OK;
}

// The captured launch of `steps` steps under the current configuration (captured on first use).
int batch_graph(fdtd_batch* b, long long steps, cudaGraphExec_t* out) {
    const int cfg[3] = {b->cluster, b->threads, b->n_clusters};
    for (auto& G : b->graphs)
        if (G.steps == steps && std::equal(cfg, cfg + 3, G.cfg)) {
            *out = G.exec;
            return FDTD_OK;
        }
    if (b->graphs.size() >= 4) batch_drop_graph(b);
    const int n = (int)b->hs.size();
    if (b->cluster == -1 && b->chain_streams.empty()) {
        b->chain_streams.assign(n, nullptr);
        b->chain_events.assign(n + 1, nullptr);
        for (int q = 0; q < n; ++q) CUDA_TRY(cudaStreamCreateWithFlags(&b->chain_streams[q], cudaStreamNonBlocking));
        for (int q = 0; q <= n; ++q) CUDA_TRY(cudaEventCreateWithFlags(&b->chain_events[q], cudaEventDisableTiming));
    }
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    if (b->cluster == -1) {
        // fork one chain per instance, `steps` two-pass steps each, join, advance the counters
        e = cudaEventRecord(b->chain_events[0], b->stream);
        for (int q = 0; q < n && e == cudaSuccess; ++q) {
            const BatchInstance& I = b->inst[q];
            cudaStream_t cs = b->chain_streams[q];
            e = cudaStreamWaitEvent(cs, b->chain_events[0], 0);
            for (long long t = 0; t < steps && e == cudaSuccess; ++t)
                e = launch_two_pass_rel(I.p, I.f, I.ps, &b->d_inst[q].step, (int)t, cs);
            if (e == cudaSuccess) e = cudaEventRecord(b->chain_events[1 + q], cs);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->chain_events[1 + q], 0);
        }
        if (e == cudaSuccess) e = launch_batch_advance(b->d_inst, n, (int)steps, b->stream);
    } else if (b->cluster == 0) {
        e = launch_batch_flat(b->d_inst, n, b->d_items, b->n_items, steps, b->stream);
    } else {
        e = launch_batch(b->d_inst, b->d_order, n, b->d_queue, steps, b->cluster, b->threads, b->n_clusters, b->stream);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(FDTD_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    fdtd_batch::Graph G{steps, {cfg[0], cfg[1], cfg[2]}, g, nullptr};
    if (cudaGraphInstantiate(&G.exec, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(FDTD_ERR_CUDA, "batch graph instantiation");
    }
    b->graphs.push_back(G);
    *out = G.exec;
    return FDTD_OK;
}

// Run `steps` steps on every instance (refresh, graph launches), then advance the step counters.
// The persistent form is one launch of `steps` steps; the flat and chain forms replay a graph of
// kFlatChunk steps and one of the remainder. The chain form's graphs bake the descriptors in, so
// they are captured again when a descriptor changes (a handle stepped alone under the fused
// schedule, tables rebuilt).
constexpr long long kFlatChunk = 32;
unsigned long long descriptor_signature(const fdtd_batch* b) {
    unsigned long long h = 1469598103934665603ULL;  // FNV-1a over the descriptors without their steps
    for (const BatchInstance& I : b->inst) {
        const unsigned char* c = reinterpret_cast<const unsigned char*>(&I);
        for (size_t q = 0; q < offsetof(BatchInstance, step); ++q) h = (h ^ c[q]) * 1099511628211ULL;
    }
    return h;
}
int batch_run(fdtd_batch* b, long long steps) {
    int rc = batch_refresh(b);
    if (rc) return rc;
    if (b->cluster == -1) {
        const unsigned long long sig = descriptor_signature(b);
        if (sig != b->chain_sig) {
            batch_drop_graph(b);
            b->chain_sig = sig;
        }
    }
    cudaGraphExec_t ex = nullptr;
    if (b->cluster <= 0) {
        const long long chunk = std::min(steps, kFlatChunk), full = steps / chunk, rem = steps % chunk;
        if ((rc = batch_graph(b, chunk, &ex))) return rc;
        for (long long q = 0; q < full; ++q) CUDA_TRY(cudaGraphLaunch(ex, b->stream));
        if (rem) {
            if ((rc = batch_graph(b, rem, &ex))) return rc;
            CUDA_TRY(cudaGraphLaunch(ex, b->stream));
        }
    } else {
        if ((rc = batch_graph(b, steps, &ex))) return rc;
        CUDA_TRY(cudaGraphLaunch(ex, b->stream));
    }
    for (fdtd_handle* h : b->hs) h->step += steps;
    return FDTD_OK;
}

}  // namespace

extern "C" int fdtd_batch_create(fdtd_handle* const* handles, int32_t n, fdtd_batch** out) {
    if (!handles || !out || n < 1) return fail(FDTD_ERR_INVALID, "NULL argument or empty batch");
    *out = nullptr;
    int dev = -1;
    CUDA_TRY(cudaGetDevice(&dev));
    for (int q = 0; q < n; ++q) {
        if (!handles[q]) return fail(FDTD_ERR_INVALID, "NULL handle in the batch");
        if (handles[q]->device != dev) return fail(FDTD_ERR_INVALID, "batch handles must live on the current device");
        if (handles[q]->has_design) return fail(FDTD_ERR_INVALID, "handles with a design region cannot join a batch");
        if (!handles[q]->plates.empty()) return fail(FDTD_ERR_INVALID, "handles with plates cannot join a batch");
        for (int r = 0; r < q; ++r)
            if (handles[r] == handles[q]) return fail(FDTD_ERR_INVALID, "a handle appears twice in the batch");
    }
    fdtd_batch* b = new fdtd_batch();
    b->hs.assign(handles, handles + n);
    b->device = dev;
    b->inst.resize(n);
    auto cleanup = [&](int rc) { fdtd_batch_destroy(b); return rc; };
    if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_CUDA, "batch stream"));
    b->stream = b->own_stream;
    if (cudaMalloc((void**)&b->d_inst, sizeof(BatchInstance) * n) != cudaSuccess ||
        cudaMalloc((void**)&b->d_order, sizeof(int) * n) != cudaSuccess || cudaMalloc((void**)&b->d_queue, sizeof(int)) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_OOM, "batch tables"));
    // longest first: clusters that finish early pick up the short instances
    std::vector<int> order(n);
    for (int q = 0; q < n; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return vol(b->hs[x]) > vol(b->hs[y]); });
    if (cudaMemcpy(b->d_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_CUDA, "batch order upload"));
    // flat form: every 32 x 8 block of every plane of every instance
    std::vector<int4> items;
    for (int q = 0; q < n; ++q) {
        const DeviceGrid& g = b->hs[q]->g;
        if (g.plane * (long long)(g.nz + 1) >= (1LL << 31))
            return cleanup(fail(FDTD_ERR_INVALID, "batch instances must hold fewer than 2^31 nodes"));
        for (int k = 0; k < g.nz; ++k)
            for (int y0 = 0; y0 < g.ny; y0 += 8)
                for (int x0 = 0; x0 < g.nx; x0 += 32) items.push_back(make_int4(q, x0, y0, k));
    }
    if (items.size() > (size_t)INT32_MAX) return cleanup(fail(FDTD_ERR_INVALID, "batch too large for the flat form"));
    b->n_items = (int)items.size();
    if (cudaMalloc((void**)&b->d_items, sizeof(int4) * std::max<size_t>(items.size(), 1)) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_OOM, "batch work list"));
    if (cudaMemcpy(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup(fail(FDTD_ERR_CUDA, "batch work list upload"));
    int rc = batch_set_config(b, -1, 256);
    if (rc) return cleanup(rc);
    *out = b;
    return FDTD_OK;
}

extern "C" int fdtd_batch_destroy(fdtd_batch* b) {
    if (!b) return FDTD_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_drop_graph(b);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    for (cudaStream_t cs : b->chain_streams)
        if (cs) cudaStreamDestroy(cs);
    for (cudaEvent_t ev : b->chain_events)
        if (ev) cudaEventDestroy(ev);
    cudaFree(b->d_inst);
    cudaFree(b->d_order);
    cudaFree(b->d_queue);
    cudaFree(b->d_items);
    delete b;
    return FDTD_OK;
}

extern "C" int fdtd_batch_set_stream(fdtd_batch* b, void* stream) {
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (!stream) return fail(FDTD_ERR_INVALID, "the batch needs a created stream (graph capture)");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->stream = (cudaStream_t)stream;
    batch_drop_graph(b);
    return FDTD_OK;
}

extern "C" int fdtd_batch_set_config(fdtd_batch* b, int32_t cluster, int32_t threads) {
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    return batch_set_config(b, cluster, threads);
}

extern "C" int fdtd_batch_get_config(const fdtd_batch* b, int32_t* cluster, int32_t* threads, int32_t* n_clusters) {
    if (!b || !cluster || !threads || !n_clusters) return fail(FDTD_ERR_INVALID, "NULL argument");
    *cluster = b->cluster;
    *threads = b->threads;
    *n_clusters = b->n_clusters;
    return FDTD_OK;
}

extern "C" int fdtd_batch_step(fdtd_batch* b, int64_t steps) {
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (steps < 0) return fail(FDTD_ERR_INVALID, "negative step count");
    if (steps == 0) return FDTD_OK;
    return batch_run(b, steps);
}

extern "C" int fdtd_batch_synchronize(fdtd_batch* b) {
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (fdtd_handle* h : b->hs) {
        int st = 0;
        CUDA_TRY(cudaMemcpy(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost));
        if (st) return fail(FDTD_ERR_DEVICE, "device status word " + std::to_string(st));
    }
    return FDTD_OK;
}

extern "C" int fdtd_batch_tune(fdtd_batch* b, int64_t steps, double* best_ms) {
    if (!b) return fail(FDTD_ERR_INVALID, "batch is NULL");
    if (steps < 1) return fail(FDTD_ERR_INVALID, "tuning needs at least one step");
    // every candidate runs from the same state: save all instances, restore after each trial
    const size_t nh = b->hs.size();
    std::vector<void*> saved(nh, nullptr);
    std::vector<long long> steps0(nh);
    std::vector<cudaStream_t> streams(nh);
    for (size_t q = 0; q < nh; ++q) streams[q] = b->hs[q]->stream;
    auto restore_all = [&]() {
        for (void* p : saved) cudaFree(p);
        for (size_t q = 0; q < nh; ++q) b->hs[q]->stream = streams[q];
    };
    for (size_t q = 0; q < nh; ++q) {
        fdtd_handle* h = b->hs[q];
        int rc = ensure_prepared(h);
        if (!rc && h->stream != b->stream && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = fail(FDTD_ERR_CUDA, "sync");
        if (!rc && cudaMalloc(&saved[q], (size_t)fdtd_state_bytes(h)) != cudaSuccess) rc = fail(FDTD_ERR_OOM, "tuning state copies");
        h->stream = b->stream;  // the state copies go on the batch stream during tuning
        if (!rc) rc = state_copy(h, saved[q], true);
        if (rc) { restore_all(); return rc; }
        steps0[q] = h->step;
    }
    const int clusters[6] = {-1, 0, 1, 2, 4, 8}, threads[3] = {128, 256, 512};
    double best = 1e300;
    int best_c = b->cluster, best_t = b->threads;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = FDTD_OK;
    for (int c : clusters) {
        for (int t : threads) {
            if (c <= 0 && t != 256) continue;
            if (batch_set_config(b, c, t) != FDTD_OK) continue;  // shape does not fit: skip it
            // a first run captures the candidate's graphs, the second is timed; states restored after each
            float ms = 0.f;
            for (int rep = 0; rep < 2 && !rc; ++rep) {
                cudaEventRecord(e0, b->stream);
                if ((rc = batch_run(b, steps))) break;
                cudaEventRecord(e1, b->stream);
                if (cudaEventSynchronize(e1) != cudaSuccess) { rc = fail(FDTD_ERR_CUDA, "tuning run failed"); break; }
                cudaEventElapsedTime(&ms, e0, e1);
                for (size_t q = 0; q < nh && !rc; ++q) {
                    rc = state_copy(b->hs[q], saved[q], false);
                    b->hs[q]->step = steps0[q];
                }
            }
            if (rc) break;
            if (ms < best) { best = ms; best_c = c; best_t = t; }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(b->stream);
    restore_all();
    if (rc) return rc;
    rc = batch_set_config(b, best_c, best_t);
    if (best_ms) *best_ms = best;
    return rc;
}

// ---------------------------------------------------------------------------------------------
// Port voltage and current (voltMgpu, currMgpu, fdtdrav.h:2185-2488).
// ---------------------------------------------------------------------------------------------
namespace {

// The current loop of currMgpu for direction `axis` (0 x, 1 y, 2 z; cases 1, 2, 3 of
// fdtdrav.h:2318-2480) on the current box c, as four groups of H probes in summation order, and
// the cell sizes a1, a2 of I = a1 s1 + a2 s2 - a1 s3 - a2 s4.
//   x: s1 Hy(ie-1, j, ks-1), s2 Hz(ie-1, je, k), s3 Hy(ie-1, j, ke), s4 Hz(ie-1, js-1, k); a1 dy, a2 dz
//   y: s1 Hz(is-1, je-1, k), s2 Hx(i, je-1, ke), s3 Hz(ie, je-1, k), s4 Hx(i, je-1, ks-1); a1 dz, a2 dx
//   z: s1 Hy(ie, j, ke-1), s2 Hx(i, js-1, ke-1), s3 Hy(is-1, j, ke-1), s4 Hx(i, je, ke-1); a1 dy, a2 dx
// with i in [is, ie], j in [js, je], k in [ks, ke].
void port_groups(int axis, const int* c, std::vector<Probe> g[4]) {
    for (int q = 0; q < 4; ++q) g[q].clear();
    if (axis == 0) {
        for (int j = c[1]; j <= c[4]; ++j) g[0].push_back(Probe{FDTD_HY, c[3] - 1, j, c[2] - 1});
        for (int k = c[2]; k <= c[5]; ++k) g[1].push_back(Probe{FDTD_HZ, c[3] - 1, c[4], k});
        for (int j = c[1]; j <= c[4]; ++j) g[2].push_back(Probe{FDTD_HY, c[3] - 1, j, c[5]});
        for (int k = c[2]; k <= c[5]; ++k) g[3].push_back(Probe{FDTD_HZ, c[3] - 1, c[1] - 1, k});
    } else if (axis == 1) {
        for (int k = c[2]; k <= c[5]; ++k) g[0].push_back(Probe{FDTD_HZ, c[0] - 1, c[4] - 1, k});
        for (int i = c[0]; i <= c[3]; ++i) g[1].push_back(Probe{FDTD_HX, i, c[4] - 1, c[5]});
        for (int k = c[2]; k <= c[5]; ++k) g[2].push_back(Probe{FDTD_HZ, c[3], c[4] - 1, k});
        for (int i = c[0]; i <= c[3]; ++i) g[3].push_back(Probe{FDTD_HX, i, c[4] - 1, c[2] - 1});
    } else {
        const int kc = c[5] - 1;
        for (int j = c[1]; j <= c[4]; ++j) g[0].push_back(Probe{FDTD_HY, c[3], j, kc});
        for (int i = c[0]; i <= c[3]; ++i) g[1].push_back(Probe{FDTD_HX, i, c[1] - 1, kc});
        for (int j = c[1]; j <= c[4]; ++j) g[2].push_back(Probe{FDTD_HY, c[0] - 1, j, kc});
        for (int i = c[0]; i <= c[3]; ++i) g[3].push_back(Probe{FDTD_HX, i, c[4], kc});
    }
}

}  // namespace

extern "C" int fdtd_add_port(fdtd_handle* h, int32_t voltage_axis, const int32_t vbox[6], int32_t current_axis,
                             const int32_t ibox[6], int32_t* id_out) {
    if (!h || !vbox || !ibox) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (voltage_axis < 0 || voltage_axis > 2) return fail(FDTD_ERR_INVALID, "voltage axis must be 0, 1 or 2");
    if (current_axis < 0 || current_axis > 2) return fail(FDTD_ERR_INVALID, "current axis must be 0, 1 or 2");
    if (h->step > 0) return fail(FDTD_ERR_STATE, "ports must be added before the first step");
    const DeviceGrid& g = h->g;
    const int* v = vbox;
    const int* c = ibox;
    // the summed ranges: half-open along the voltage axis, closed across it
    const int va = voltage_axis;
    const int vi1 = va == 0 ? v[3] - 1 : v[3], vj1 = va == 1 ? v[4] - 1 : v[4], vk1 = va == 2 ? v[5] - 1 : v[5];
    if (v[0] < 0 || v[1] < 0 || v[2] < 0 || vi1 >= g.nx || vj1 >= g.ny || vk1 >= g.nz || v[0] > vi1 || v[1] > vj1 ||
        v[2] > vk1)
        return fail(FDTD_ERR_INVALID, "voltage box outside the grid or empty (half-open along the voltage axis)");
    if (c[0] > c[3] || c[1] > c[4] || c[2] > c[5] || (current_axis == 2 && c[5] < 1))
        return fail(FDTD_ERR_INVALID, "current box empty or reversed");
    std::vector<Probe> grp[4];
    port_groups(current_axis, c, grp);
    for (int q = 0; q < 4; ++q)
        for (const Probe& pr : grp[q])
            if (pr.i < 0 || pr.i >= g.nx || pr.j < 0 || pr.j >= g.ny || pr.k < 0 || pr.k >= g.nz)
                return fail(FDTD_ERR_INVALID, "the current loop of the box leaves the grid");
    PortDef P{};
    std::copy(v, v + 6, P.vbox);
    std::copy(c, c + 6, P.ibox);
    P.current_axis = current_axis;
    P.voltage_axis = voltage_axis;
    P.first = (int)h->probes.size();
    for (int k = v[2]; k <= vk1; ++k)
        for (int j = v[1]; j <= vj1; ++j)
            for (int i = v[0]; i <= vi1; ++i) h->probes.push_back(Probe{FDTD_EZ, i, j, k});
    P.n_v = (int)h->probes.size() - P.first;
    for (int q = 0; q < 4; ++q) {
        h->probes.insert(h->probes.end(), grp[q].begin(), grp[q].end());
        P.n[q] = (int)grp[q].size();
    }
    h->ports.push_back(P);
    h->dirty_probes = true;
    if (id_out) *id_out = (int32_t)h->ports.size() - 1;
    return FDTD_OK;
}

extern "C" int fdtd_read_port(fdtd_handle* h, int32_t id, int64_t first, int64_t n, int32_t time_average,
                              float* voltage, float* current) {
    if (!h || (n > 0 && (!voltage || !current))) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (id < 0 || id >= (int)h->ports.size()) return fail(FDTD_ERR_INVALID, "no such port");
    if (n == 0) return FDTD_OK;
    const int np = (int)h->probes.size();
    std::vector<float> rows((size_t)n * np);
    int rc = fdtd_read_probes(h, first, n, rows.data());
    if (rc) return rc;
    const PortDef& P = h->ports[id];
    const float dx = h->g.dx, dy = h->g.dy, dz = h->g.dz;
    const float a1 = P.current_axis == 1 ? dz : dy, a2 = P.current_axis == 0 ? dz : dx;
    // voltMgpu cases 1 / 2 / 3 (fdtdrav.h:2214-2290), with float box bounds
    const float is = (float)P.vbox[0], js = (float)P.vbox[1], ks = (float)P.vbox[2];
    const float ie = (float)P.vbox[3], je = (float)P.vbox[4], ke = (float)P.vbox[5];
    const float csuf = P.voltage_axis == 0   ? (-dx) / ((je - js + 1) * (ke - ks + 1))
                       : P.voltage_axis == 1 ? (-dy) / ((ke - ks + 1) * (ie - is + 1))
                                             : (-dz) / ((ie - is + 1) * (je - js + 1));
    for (int64_t t = 0; t < n; ++t) {
        const float* r = rows.data() + (size_t)t * np + P.first;
        float volt = 0.f;
        for (int q = 0; q < P.n_v; ++q) volt = volt + r[q];
        voltage[t] = volt * csuf;
        const float* h4 = r + P.n_v;
        float sum[4];
        for (int q = 0; q < 4; ++q) {
            float acc = 0.f;
            for (int e = 0; e < P.n[q]; ++e) acc = acc + h4[e];
            sum[q] = acc;
            h4 += P.n[q];
        }
        // a1 s1 + a2 s2 - a1 s3 - a2 s4 as the reference's compiled expressions contract it: one
        // product fused with the other as the addend (the first fused in the x loop, the second in
        // the y and z loops), then the two subtractions as FMAs
        const float lead = P.current_axis == 0 ? std::fmaf(a1, sum[0], a2 * sum[1]) : std::fmaf(a2, sum[1], a1 * sum[0]);
        current[t] = std::fmaf(-a2, sum[3], std::fmaf(-a1, sum[2], lead));
    }
    if (time_average && n > 1) {
        // correcI averages in place, one thread per step: I(t) = (I(t) + I(t+1)) / 2 from the
        // unaveraged neighbour, and the last step (I(t) + I(t-1)) / 2 from the already averaged
        // one (its branch diverges from its neighbour's inside the warp and runs after it)
        for (int64_t t = 0; t + 1 < n; ++t) current[t] = (current[t] + current[t + 1]) / 2;
        current[n - 1] = (current[n - 1] + current[n - 2]) / 2;
    }
    return FDTD_OK;
}

extern "C" int fdtd_port_spectrum(fdtd_handle* h, int32_t id, int64_t first, int64_t n, float z0_re, float z0_im,
                                  float* v_spectrum, float* i_spectrum, float* s11, float* zin) {
    if (!h) return fail(FDTD_ERR_INVALID, "NULL argument");
    if (n < 2 || n > INT32_MAX) return fail(FDTD_ERR_INVALID, "the spectrum needs 2 .. 2^31-1 steps");
    if (!(z0_re > 0.f)) return fail(FDTD_ERR_INVALID, "Re z0 must be positive");
    std::vector<float> v((size_t)n), c((size_t)n);
    int rc = fdtd_read_port(h, id, first, n, 1, v.data(), c.data());
    if (rc) return rc;
    std::string err;
    rc = port_spectra(h->stream, (int)n, v.data(), c.data(), z0_re, z0_im, v_spectrum, i_spectrum, s11, zin, &err);
    return rc ? fail(rc, err) : FDTD_OK;
}

extern "C" int fdtd_port_zin(int64_t n_bins, const float* v_spectrum, const float* i_spectrum, float z0_re,
                             float z0_im, float* s11, float* zin) {
    if (n_bins < 1 || n_bins > INT32_MAX / 4) return fail(FDTD_ERR_INVALID, "n_bins must be 1 .. 2^29-1");
    if (!v_spectrum || !i_spectrum) return fail(FDTD_ERR_INVALID, "NULL spectrum");
    if (!(z0_re > 0.f)) return fail(FDTD_ERR_INVALID, "Re z0 must be positive");
    std::string err;
    const int rc = port_zin(nullptr, (int)n_bins, v_spectrum, i_spectrum, z0_re, z0_im, s11, zin, &err);
    return rc ? fail(rc, err) : FDTD_OK;
}
