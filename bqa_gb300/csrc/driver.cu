// One annealing step driven from native code: the same launch sequence and host decisions as
// the Python engine's run_layer (gate layer with BP-gauged truncation, then loopy BP to
// tolerance), with the two device-to-host reads of a step (truncation column maxima, BP loop
// state) done here.  A caller binding it through ctypes releases the interpreter lock for the
// whole step, so host threads driving concurrent jobs do not serialise on it.
//
// Mirrors src/bqa/state.py:315-321 (run_layer), :230-247 (_simple_update), :97-124 (_run_bp).
#include <cmath>
#include <cstring>
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
    if (j->split_sweeps)
        rc = bqa_ext_msgs_split(j->classes, j->n_classes, chi, dt, msgs, j->lu, E, j->edge_j, ztime, j->ext, s);
    else
        rc = bqa_ext_msgs(j->classes, j->n_classes, chi, dt, msgs, j->ext, ztime, s);
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

static int run_bp(bqa_job* j, bqa_layer_info* info, cudaStream_t st) {
    if (j->max_bp_iters < 1) return set_error(BQA_ERR_ARG, "max_bp_iter_number must be >= 1 to run BP");
    void* s = reinterpret_cast<void*>(st);
    void* a = j->msgs[j->mcur];
    void* b = j->msgs[1 - j->mcur];
    int rc;
    if ((rc = cuda_rc(cudaMemsetAsync(j->loop_state, 0, 8 * sizeof(int32_t), st), "loop state"))) return rc;
    if ((rc = cuda_rc(cudaMemsetAsync(j->dist_parts, 0, 2 * sizeof(int64_t), st), "dist"))) return rc;
    const int64_t elems = (int64_t)j->edges * j->chis * j->chis;
    const int every = j->bp_check_every > 0 ? j->bp_check_every : 1;
    int launched = 0;
    int32_t ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    while (true) {
        const int group = (j->max_bp_iters - launched) < every ? (j->max_bp_iters - launched) : every;
        for (int g = 0; g < group; ++g) {
            if (j->split_sweeps)
                rc = bqa_bp_sweep_split(j->classes, j->n_classes, j->chis, j->dtype, a, b, j->lu, j->edges,
                                        j->dist_parts, j->loop_state, s);
            else
                rc = bqa_bp_sweep(j->classes, j->n_classes, j->chis, j->dtype, a, b, j->dist_parts, j->loop_state, s);
            if (rc) return rc;
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
    if (ls[2]) j->mcur = 1 - j->mcur;
    info->sweeps = ls[1];
    info->bp_exhausted = ls[3];
    float best;
    std::memcpy(&best, &ls[6], 4);
    info->best_dist = best;
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
