// One annealing step driven from native code: the same launch sequence and host decisions as
// the Python engine's run_layer (gate layer with BP-gauged truncation, then loopy BP to
// tolerance), with the two device-to-host reads of a step (truncation column maxima, BP loop
// state) done here.  A caller binding it through ctypes releases the interpreter lock for the
// whole step, so host threads driving concurrent jobs do not serialise on it.
//
// Mirrors src/bqa/state.py:315-321 (run_layer), :230-247 (_simple_update), :97-124 (_run_bp).
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "internal.h"

extern "C" {
int32_t bqa_ext_msgs(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                     void* ext_out, double ztime, void* stream);
int32_t bqa_ext_msgs_split(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                           void* pm, int32_t edges, const double* edge_j, double ztime, void* ext_out, void* stream);
int32_t bqa_env_factor(const void* mats, int32_t count, int32_t n, int32_t dtype, double eps, void* lu, void* ul,
                       int32_t* status, void* stream);
int32_t bqa_bond_canon(const void* lu, const void* ul, int32_t edges, int32_t n, int32_t dtype, double eps, void* canon,
                       void* lmbds, void* colmax, int32_t* status, void* stream);
int32_t bqa_lmbds_truncate(void* lmbds, int32_t stride, int32_t rows, int32_t dim, int32_t dtype, void* stream);
int32_t bqa_apply_update(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dim, int32_t dtype,
                         const void* canon, const void* lmbds, int32_t lam_stride, double ztime, double xtime,
                         void* stream);
int32_t bqa_msgs_from_lmbds(const void* lmbds, int32_t lam_stride, int32_t edges, int32_t dim, int32_t dtype,
                            void* msgs, void* stream);
int32_t bqa_bp_sweep(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, void* msgs_a,
                     void* msgs_b, void* dist_parts, const int32_t* loop_state, void* stream);
int32_t bqa_bp_sweep_split(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, void* msgs_a,
                           void* msgs_b, void* pm, int32_t edges, void* dist_parts, const int32_t* loop_state,
                           void* stream);
int32_t bqa_bp_finalize(void* msgs_a, void* msgs_b, int64_t msg_elems, int32_t dtype, void* dist_parts,
                        int32_t* loop_state, double eps, double damping, int32_t max_iters, void* stream);
int32_t bqa_ext_combine(const void* pm, int32_t edges, int32_t chi, int32_t dtype, const double* edge_j, double ztime,
                        void* ext_out, void* stream);
int32_t bqa_bp_sweep_plan(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype,
                          const int32_t* variants, void* msgs_a, void* msgs_b, void* pm, int32_t edges,
                          void* dist_parts, const int32_t* loop_state, void* stream);
}

namespace bqa {

static int cuda_rc(cudaError_t e, const char* what) {
    return e == cudaSuccess ? BQA_OK : set_error(BQA_ERR_CUDA, "bqa_run_layer: %s: %s", what, cudaGetErrorString(e));
}

static int store_dim(const bqa_job* j, int chi) {
    return (j->pad_bonds && chi > 4 && chi <= 16 && chi % 4) ? chi + 4 - chi % 4 : chi;
}

static int gate_layer(bqa_job* j, double xtime, double ztime, bqa_layer_info* info, cudaStream_t st) {
    const int chi = j->chis, n = 2 * chi, dt = j->dtype, E = j->edges;
    void* s = reinterpret_cast<void*>(st);
    void* msgs = j->msgs[j->mcur];
    int rc;
    if (j->split_sweeps && j->blocks_valid)
        // the converged BP run left the open-bond blocks of these messages in lu
        rc = bqa_ext_combine(j->lu, E, chi, dt, j->edge_j, ztime, j->ext, s);
    else if (j->split_sweeps)
        rc = bqa_ext_msgs_split(j->classes, j->n_classes, chi, dt, msgs, j->lu, E, j->edge_j, ztime, j->ext, s);
    else
        rc = bqa_ext_msgs(j->classes, j->n_classes, chi, dt, msgs, j->ext, ztime, s);
    j->blocks_valid = 0;   // lu is overwritten by the environment factors below
    if (rc) return rc;
    if ((rc = bqa_env_factor(j->ext, E, n, dt, j->pinv_eps, j->lu, j->ul, j->status, s))) return rc;
    const size_t bits = dt == BQA_C64 ? 4 : 8;
    if ((rc = cuda_rc(cudaMemsetAsync(j->colmax, 0, bits * (size_t)j->colmax_elems, st), "colmax"))) return rc;
    void* canon = j->ext;   // the extended messages are consumed; canonicalisers reuse their storage
    if ((rc = bqa_bond_canon(j->lu, j->ul, E, n, dt, j->pinv_eps, canon, j->lmbds, j->colmax, j->status, s))) return rc;
    // global truncation (src/bqa/backends.py:297-303): one small device-to-host read
    unsigned char host[64 * 8];
    int32_t status = 0;
    if ((rc = cuda_rc(cudaMemcpyAsync(host, j->colmax, bits * n, cudaMemcpyDeviceToHost, st), "colmax read"))) return rc;
    if ((rc = cuda_rc(cudaMemcpyAsync(&status, j->status, sizeof(int32_t), cudaMemcpyDeviceToHost, st), "status"))) return rc;
    if ((rc = cuda_rc(cudaStreamSynchronize(st), "sync"))) return rc;
    if (status) {
        info->svd_not_converged = 1;
        if ((rc = cuda_rc(cudaMemsetAsync(j->status, 0, sizeof(int32_t), st), "status reset"))) return rc;
    }
    std::vector<double> max_l(n);
    for (int i = 0; i < n; ++i) {
        if (dt == BQA_C64) { float f; std::memcpy(&f, host + 4 * i, 4); max_l[i] = f; }
        else { double d; std::memcpy(&d, host + 8 * i, 8); max_l[i] = d; }
    }
    int below = 0;
    for (int i = 0; i < n; ++i) below += max_l[i] < j->pinv_eps;
    const int rank = n - below;
    const int dim = rank < j->max_bond_dim ? rank : j->max_bond_dim;
    double err2 = 0;
    for (int i = dim; i < n; ++i) err2 += max_l[i] * max_l[i];
    info->trunc_err = std::sqrt(err2);
    const int dims = store_dim(j, dim);
    if (dims != dim && (rc = bqa_lmbds_truncate(j->lmbds, n, E / 2, dim, dt, s))) return rc;
    if ((rc = bqa_apply_update(j->classes, j->n_classes, chi, dims, dt, canon, j->lmbds, n, ztime, xtime, s))) return rc;
    // the updated tensors are current: swap each class's buffers
    for (int c = 0; c < j->n_classes; ++c) {
        void* t = j->classes[c].tensor;
        j->classes[c].tensor = j->classes[c].tensor_out;
        j->classes[c].tensor_out = t;
    }
    j->tcur = 1 - j->tcur;
    j->chi = dim;
    j->chis = dims;
    j->lam_stride = n;
    info->bond_dim = dim;
    return bqa_msgs_from_lmbds(j->lmbds, n, E, dims, dt, j->msgs[j->mcur], s);
}

// Whether the job's BP sweeps run in two stages (open-bond blocks in lu, then messages).
static bool job_two_stage(const bqa_job* j) {
    if (j->sweep_variants) {
        const int32_t form = j->sweep_variants[(size_t)j->chis * (j->n_classes + 1)];
        return form == 0 ? j->split_sweeps != 0 : form == 1;
    }
    return j->split_sweeps != 0;
}

// One sweep of the job's BP loop: the tuned per-class kernels when the job carries a plan.
static int job_sweep(bqa_job* j, void* a, void* b, void* s) {
    if (j->sweep_variants) {
        const int32_t* row = j->sweep_variants + (size_t)j->chis * (j->n_classes + 1);
        const bool two_stage = row[0] == 0 ? j->split_sweeps != 0 : row[0] == 1;
        return bqa_bp_sweep_plan(j->classes, j->n_classes, j->chis, j->dtype, row + 1, a, b,
                                 two_stage ? j->lu : nullptr, j->edges, j->dist_parts, j->loop_state, s);
    }
    if (j->split_sweeps)
        return bqa_bp_sweep_split(j->classes, j->n_classes, j->chis, j->dtype, a, b, j->lu, j->edges, j->dist_parts,
                                  j->loop_state, s);
    return bqa_bp_sweep(j->classes, j->n_classes, j->chis, j->dtype, a, b, j->dist_parts, j->loop_state, s);
}

// The host side of a finished BP run from its final loop state: which buffer holds the kept
// messages, whether lu holds their open-bond blocks, and the run's figures.
static void bp_conclude(bqa_job* j, const int32_t* ls, bqa_layer_info* info) {
    if (ls[2]) j->mcur = 1 - j->mcur;
    // converged: the kept messages are the last sweep's input, whose blocks that sweep left in lu
    j->blocks_valid = (!ls[3] && job_two_stage(j)) ? 1 : 0;
    info->sweeps = ls[1];
    info->bp_exhausted = ls[3];
    float best;
    std::memcpy(&best, &ls[6], 4);
    info->best_dist = best;
}

static int bp_reset(bqa_job* j, cudaStream_t st) {
    int rc = cuda_rc(cudaMemsetAsync(j->loop_state, 0, 8 * sizeof(int32_t), st), "loop state");
    if (!rc) rc = cuda_rc(cudaMemsetAsync(j->dist_parts, 0, 2 * sizeof(int64_t), st), "dist");
    return rc;
}

static int run_bp(bqa_job* j, bqa_layer_info* info, cudaStream_t st) {
    if (j->max_bp_iters < 1) return set_error(BQA_ERR_ARG, "max_bp_iter_number must be >= 1 to run BP");
    void* s = reinterpret_cast<void*>(st);
    void* a = j->msgs[j->mcur];
    void* b = j->msgs[1 - j->mcur];
    int rc;
    if ((rc = bp_reset(j, st))) return rc;
    const int64_t elems = (int64_t)j->edges * j->chis * j->chis;
    const int every = j->bp_check_every > 0 ? j->bp_check_every : 1;
    int launched = 0;
    int32_t ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    while (true) {
        const int group = (j->max_bp_iters - launched) < every ? (j->max_bp_iters - launched) : every;
        for (int g = 0; g < group; ++g) {
            if ((rc = job_sweep(j, a, b, s))) return rc;
            if ((rc = bqa_bp_finalize(a, b, elems, j->dtype, j->dist_parts, j->loop_state, j->bp_eps, j->damping,
                                      j->max_bp_iters, s)))
                return rc;
            ++launched;
        }
        if ((rc = cuda_rc(cudaMemcpyAsync(ls, j->loop_state, sizeof(ls), cudaMemcpyDeviceToHost, st), "loop read")))
            return rc;
        if ((rc = cuda_rc(cudaStreamSynchronize(st), "sync"))) return rc;
        if (ls[0]) break;
        if (launched >= j->max_bp_iters)
            return set_error(BQA_ERR_UNSUPPORTED, "BP loop state did not finish after the iteration cap");
    }
    bp_conclude(j, ls, info);
    return BQA_OK;
}

}  // namespace bqa

using namespace bqa;

extern "C" int32_t bqa_run_layer(bqa_job* job, double xtime, double ztime, bqa_layer_info* info, void* stream) {
    if (!job || !info || !job->classes || job->n_classes < 0 || job->edges < 2 || job->chis < 1 ||
        2 * job->chis > job->colmax_elems || 2 * job->chis > 64)
        return set_error(BQA_ERR_ARG, "bqa_run_layer: bad argument");
    std::memset(info, 0, sizeof(*info));
    cudaStream_t st = as_stream(stream);
    int rc = gate_layer(job, xtime, ztime, info, st);
    if (rc) return rc;
    return run_bp(job, info, st);
}

// ---- BP to tolerance as one CUDA graph ----------------------------------------------------
//
// The device-driven BP loop launches the same kernels with the same arguments every sweep
// (which message buffer is read, whether the run is done and whether to damp all live in
// loop_state on the device), so a whole run -- zero the loop state, then sweep + decision +
// damping while the decision kernel has not marked the run done, then copy the loop state to
// the host -- is captured once per (buffers, bond dim, loop parameters) as a graph with a
// WHILE node.  A BP run is then one graph launch and one host read, instead of 3-4 launches
// per sweep, a host read every bp_check_every sweeps and up to bp_check_every - 1 sweeps
// queued after convergence that return at once.  Same kernels in the same order as run_bp:
// the state after a step is bit-identical.

namespace bqa {

// Repeats the WHILE body while the run is not done.  loop_state[7] counts the body passes;
// the loop also ends after max_iters passes whatever the decision says, so it cannot run on.
__global__ void bp_graph_cond_kernel(cudaGraphConditionalHandle handle, int32_t* ls, int max_iters) {
    const int passes = ls[7] + 1;
    ls[7] = passes;
    cudaGraphSetConditional(handle, (ls[0] == 0 && passes < max_iters) ? 1u : 0u);
}

struct GraphEntry {
    std::vector<uint64_t> key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

}  // namespace bqa

struct bqa_graph_cache {
    int device = 0;
    cudaStream_t capture[2] = {nullptr, nullptr};   // private streams: capture cannot use the legacy stream
    int32_t* host_ls = nullptr;                      // pinned: target of the graph's loop-state copy
    std::vector<bqa::GraphEntry> entries;            // oldest first
};

namespace bqa {

constexpr size_t kGraphCacheEntries = 16;

static void release(GraphEntry& e) {
    if (e.exec) cudaGraphExecDestroy(e.exec);
    if (e.graph) cudaGraphDestroy(e.graph);
    e.exec = nullptr;
    e.graph = nullptr;
}

static uint64_t bits_of(double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return u;
}

// Everything a captured BP run bakes into its launches.
static std::vector<uint64_t> bp_graph_key(const bqa_job* j) {
    std::vector<uint64_t> k = {(uint64_t)j->dtype, (uint64_t)j->chis, (uint64_t)j->mcur, (uint64_t)j->edges,
                               (uint64_t)j->split_sweeps, (uint64_t)j->max_bp_iters, bits_of(j->bp_eps),
                               bits_of(j->damping), (uint64_t)(uintptr_t)j->msgs[0], (uint64_t)(uintptr_t)j->msgs[1],
                               (uint64_t)(uintptr_t)j->lu, (uint64_t)(uintptr_t)j->dist_parts,
                               (uint64_t)(uintptr_t)j->loop_state, (uint64_t)j->n_classes};
    if (j->sweep_variants)
        for (int c = 0; c <= j->n_classes; ++c)
            k.push_back((uint64_t)(1 + j->sweep_variants[(size_t)j->chis * (j->n_classes + 1) + c]));
    for (int c = 0; c < j->n_classes; ++c) {
        const bqa_class& x = j->classes[c];
        const void* p[] = {x.node_ids, x.in_pos, x.out_pos, x.lmbd_pos, x.edge_ampl, x.node_ampl, x.tensor, x.scratch};
        k.push_back((uint64_t)x.degree);
        k.push_back((uint64_t)x.count);
        k.push_back((uint64_t)x.scratch_elems);
        for (const void* q : p) k.push_back((uint64_t)(uintptr_t)q);
    }
    return k;
}

// One sweep, the decision and the damping, then the loop condition: the WHILE body.
static int bp_body(bqa_job* j, cudaGraphConditionalHandle h, cudaStream_t st) {
    void* s = reinterpret_cast<void*>(st);
    void* a = j->msgs[j->mcur];
    void* b = j->msgs[1 - j->mcur];
    int rc = job_sweep(j, a, b, s);
    if (rc) return rc;
    const int64_t elems = (int64_t)j->edges * j->chis * j->chis;
    if ((rc = bqa_bp_finalize(a, b, elems, j->dtype, j->dist_parts, j->loop_state, j->bp_eps, j->damping,
                              j->max_bp_iters, s)))
        return rc;
    bp_graph_cond_kernel<<<1, 1, 0, st>>>(h, j->loop_state, j->max_bp_iters);
    return check_launch("bp_graph_cond");
}

static int capture_bp_graph(bqa_job* j, bqa_graph_cache* cache, GraphEntry* out) {
    cudaStream_t s0 = cache->capture[0], s1 = cache->capture[1];
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) return cuda_rc(e, "cudaGraphCreate");
    int rc = BQA_OK;
    bool cap0 = false, cap1 = false;
    do {
        cudaGraphConditionalHandle h;
        // default 1 at every launch: the body runs at least once (max_bp_iters >= 1)
        if ((rc = cuda_rc(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault), "handle"))) break;
        if ((rc = cuda_rc(cudaStreamBeginCaptureToGraph(s0, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                          "capture")))
            break;
        cap0 = true;
        if ((rc = cuda_rc(cudaMemsetAsync(j->loop_state, 0, 8 * sizeof(int32_t), s0), "loop state"))) break;
        if ((rc = cuda_rc(cudaMemsetAsync(j->dist_parts, 0, 2 * sizeof(int64_t), s0), "dist"))) break;
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* edata = nullptr;
        size_t ndeps = 0;
        if ((rc = cuda_rc(cudaStreamGetCaptureInfo(s0, &cs, nullptr, nullptr, &deps, &edata, &ndeps), "capture info")))
            break;
        cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        if ((rc = cuda_rc(cudaGraphAddNode(&node, g, deps, edata, ndeps, &p), "while node"))) break;
        if ((rc = cuda_rc(cudaStreamUpdateCaptureDependencies(s0, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
                          "capture dependencies")))
            break;
        cudaGraph_t body = p.conditional.phGraph_out[0];
        if ((rc = cuda_rc(cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                          "body capture")))
            break;
        cap1 = true;
        rc = bp_body(j, h, s1);
        cudaGraph_t tmp = nullptr;
        cap1 = false;
        const int rc_end = cuda_rc(cudaStreamEndCapture(s1, &tmp), "body capture end");
        if (rc || (rc = rc_end)) break;
        if ((rc = cuda_rc(cudaMemcpyAsync(cache->host_ls, j->loop_state, 8 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          s0),
                          "loop read")))
            break;
    } while (false);
    if (cap1) {
        cudaGraph_t tmp = nullptr;
        cudaStreamEndCapture(s1, &tmp);
    }
    if (cap0) {
        cudaGraph_t tmp = nullptr;
        const int rc_end = cuda_rc(cudaStreamEndCapture(s0, &tmp), "capture end");
        if (!rc) rc = rc_end;
    }
    cudaGetLastError();   // a failed capture leaves its error pending; it is reported through rc
    if (rc) {
        cudaGraphDestroy(g);
        return rc;
    }
    cudaGraphExec_t exec = nullptr;
    if ((rc = cuda_rc(cudaGraphInstantiate(&exec, g, 0), "cudaGraphInstantiate"))) {
        cudaGraphDestroy(g);
        return rc;
    }
    out->graph = g;
    out->exec = exec;
    return BQA_OK;
}

static int run_bp_graph(bqa_job* j, bqa_graph_cache* cache, bqa_layer_info* info, cudaStream_t st) {
    if (j->max_bp_iters < 1) return set_error(BQA_ERR_ARG, "max_bp_iter_number must be >= 1 to run BP");
    int dev = 0;
    int rc;
    if ((rc = cuda_rc(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
    if (dev != cache->device) return set_error(BQA_ERR_ARG, "bqa graph cache belongs to device %d, not %d",
                                               cache->device, dev);
    std::vector<uint64_t> key = bp_graph_key(j);
    GraphEntry* hit = nullptr;
    for (auto& e : cache->entries)
        if (e.key == key) hit = &e;
    if (!hit) {
        GraphEntry fresh;
        fresh.key = std::move(key);
        if ((rc = capture_bp_graph(j, cache, &fresh))) return rc;
        if (cache->entries.size() >= kGraphCacheEntries) {
            release(cache->entries.front());
            cache->entries.erase(cache->entries.begin());
        }
        cache->entries.push_back(std::move(fresh));
        hit = &cache->entries.back();
    }
    if ((rc = cuda_rc(cudaGraphLaunch(hit->exec, st), "cudaGraphLaunch"))) return rc;
    if ((rc = cuda_rc(cudaStreamSynchronize(st), "sync"))) return rc;
    int32_t ls[8];
    std::memcpy(ls, cache->host_ls, sizeof(ls));
    if (!ls[0]) return set_error(BQA_ERR_UNSUPPORTED, "BP graph ended without a decision after %d sweeps", ls[1]);
    bp_conclude(j, ls, info);
    return BQA_OK;
}

static int check_job(const bqa_job* job) {
    if (!job || !job->classes || job->n_classes < 0 || job->edges < 2 || job->chis < 1 ||
        2 * job->chis > job->colmax_elems || 2 * job->chis > 64)
        return set_error(BQA_ERR_ARG, "bad job");
    return BQA_OK;
}

}  // namespace bqa

extern "C" int32_t bqa_graph_cache_create(bqa_graph_cache** out) {
    if (!out) return set_error(BQA_ERR_ARG, "bqa_graph_cache_create: null output");
    *out = nullptr;
    auto* c = new (std::nothrow) bqa_graph_cache();
    if (!c) return set_error(BQA_ERR_ARG, "bqa_graph_cache_create: out of host memory");
    int rc = cuda_rc(cudaGetDevice(&c->device), "cudaGetDevice");
    for (int i = 0; i < 2 && !rc; ++i)
        rc = cuda_rc(cudaStreamCreateWithFlags(&c->capture[i], cudaStreamNonBlocking), "cudaStreamCreate");
    if (!rc) rc = cuda_rc(cudaHostAlloc((void**)&c->host_ls, 8 * sizeof(int32_t), cudaHostAllocDefault), "cudaHostAlloc");
    if (rc) {
        bqa_graph_cache_destroy(c);
        return rc;
    }
    *out = c;
    return BQA_OK;
}

extern "C" int32_t bqa_graph_cache_destroy(bqa_graph_cache* cache) {
    if (!cache) return BQA_OK;
    for (auto& e : cache->entries) release(e);
    for (cudaStream_t s : cache->capture)
        if (s) cudaStreamDestroy(s);
    if (cache->host_ls) cudaFreeHost(cache->host_ls);
    delete cache;
    return BQA_OK;
}

extern "C" int32_t bqa_run_bp_graph(bqa_job* job, bqa_graph_cache* cache, bqa_layer_info* info, void* stream) {
    if (!cache || !info) return set_error(BQA_ERR_ARG, "bqa_run_bp_graph: bad argument");
    int rc = check_job(job);
    if (rc) return rc;
    std::memset(info, 0, sizeof(*info));
    info->bond_dim = job->chi;
    return run_bp_graph(job, cache, info, as_stream(stream));
}

extern "C" int32_t bqa_run_layer_graph(bqa_job* job, bqa_graph_cache* cache, double xtime, double ztime,
                                       bqa_layer_info* info, void* stream) {
    if (!cache || !info) return set_error(BQA_ERR_ARG, "bqa_run_layer_graph: bad argument");
    int rc = check_job(job);
    if (rc) return rc;
    std::memset(info, 0, sizeof(*info));
    cudaStream_t st = as_stream(stream);
    if ((rc = gate_layer(job, xtime, ztime, info, st))) return rc;
    return run_bp_graph(job, cache, info, st);
}

// ---- packed BP runs: the sweeps of several jobs in shared launches ---------------------------
//
// A job server keeps many jobs resident; after each job's gate layer (bqa_gate_layer, on the
// job's own stream) the jobs waiting for BP are swept together: every sweep issues each node
// kernel once for all their classes of that kernel, one combine for all their two-stage
// sweeps and one decision kernel for all their loop states (pack_execute).  Each job keeps
// its own loop state, so it stops, damps or swaps buffers exactly as in a run of its own, and
// its messages are the same bits; the caller takes a job out once its loop state says done
// (bqa_bp_end) and may add newly waiting jobs between calls (bqa_bp_begin).

namespace bqa {

constexpr int kMaxPackedJobs = 64;

struct LoopStates {
    const int32_t* ls[kMaxPackedJobs];
    int n;
};

__global__ void gather_loop_states_kernel(const __grid_constant__ LoopStates t, int32_t* out) {
    const int i = threadIdx.x;
    if (i < 8 * t.n) out[i] = t.ls[i >> 3][i & 7];
}

// restores the thread's launch mode when a collection ends, also on an early return
struct CollectGuard {
    explicit CollectGuard(PackList* l) { pack_collect(l); }
    ~CollectGuard() { pack_collect(nullptr); }
};

}  // namespace bqa

extern "C" int32_t bqa_gate_layer(bqa_job* job, double xtime, double ztime, bqa_layer_info* info, void* stream) {
    if (!info) return set_error(BQA_ERR_ARG, "bqa_gate_layer: bad argument");
    int rc = check_job(job);
    if (rc) return rc;
    std::memset(info, 0, sizeof(*info));
    return gate_layer(job, xtime, ztime, info, as_stream(stream));
}

extern "C" int32_t bqa_bp_begin(bqa_job* job, void* stream) {
    int rc = check_job(job);
    if (rc) return rc;
    if (job->max_bp_iters < 1) return set_error(BQA_ERR_ARG, "max_bp_iter_number must be >= 1 to run BP");
    return bp_reset(job, as_stream(stream));
}

extern "C" int32_t bqa_bp_packed(bqa_job* const* jobs, int32_t n_jobs, int32_t sweeps, int32_t* loop_states,
                                 int32_t* host_loop_states, void* stream) {
    if (!jobs || n_jobs < 1 || n_jobs > kMaxPackedJobs || sweeps < 1 || !loop_states || !host_loop_states)
        return set_error(BQA_ERR_ARG, "bqa_bp_packed: bad argument (1 <= n_jobs <= %d, sweeps >= 1)", kMaxPackedJobs);
    for (int i = 0; i < n_jobs; ++i) {
        int rc = check_job(jobs[i]);
        if (rc) return rc;
        if (jobs[i]->dtype != jobs[0]->dtype) return set_error(BQA_ERR_ARG, "bqa_bp_packed: jobs of different dtypes");
    }
    cudaStream_t st = as_stream(stream);
    void* s = stream;
    PackList list;
    {
        CollectGuard guard(&list);
        for (int i = 0; i < n_jobs; ++i) {
            bqa_job* j = jobs[i];
            void* a = j->msgs[j->mcur];
            void* b = j->msgs[1 - j->mcur];
            int rc = job_sweep(j, a, b, s);
            if (!rc)
                rc = bqa_bp_finalize(a, b, (int64_t)j->edges * j->chis * j->chis, j->dtype, j->dist_parts,
                                     j->loop_state, j->bp_eps, j->damping, j->max_bp_iters, s);
            if (rc) return rc;
        }
    }
    int rc;
    for (int k = 0; k < sweeps; ++k)
        if ((rc = pack_execute(list, st))) return rc;
    LoopStates t;
    t.n = n_jobs;
    for (int i = 0; i < n_jobs; ++i) t.ls[i] = jobs[i]->loop_state;
    gather_loop_states_kernel<<<1, 8 * kMaxPackedJobs, 0, st>>>(t, loop_states);
    if ((rc = check_launch("gather loop states"))) return rc;
    if ((rc = cuda_rc(cudaMemcpyAsync(host_loop_states, loop_states, 8 * sizeof(int32_t) * n_jobs,
                                      cudaMemcpyDeviceToHost, st),
                      "loop states read")))
        return rc;
    return cuda_rc(cudaStreamSynchronize(st), "sync");
}

extern "C" int32_t bqa_bp_end(bqa_job* job, const int32_t* loop_state, bqa_layer_info* info) {
    if (!job || !loop_state || !info) return set_error(BQA_ERR_ARG, "bqa_bp_end: bad argument");
    if (!loop_state[0]) return set_error(BQA_ERR_ARG, "bqa_bp_end: the BP run is not done (%d sweeps)", loop_state[1]);
    bp_conclude(job, loop_state, info);
    return BQA_OK;
}
