/*
 * bqa_gb300 -- C ABI of the GB300 (sm_103a) annealing backend.
 *
 * The reference (LuchnikovI/bqa v0.1.6) is pure Python and has no FFI; its plugin point
 * is the backend registry plus the ``Tensor`` ABC (src/bqa/backends.py:24-572), driven by
 * the state VM in src/bqa/state.py.  These entry points are the coarse operations that VM
 * performs per annealing step, each fused over all nodes of a degree class; every one
 * cites the reference code it replaces.
 *
 * Conventions
 *  - All pointers are DEVICE pointers unless a parameter says "host".
 *  - ``dtype`` selects the arithmetic: BQA_C64 = complex64 stored as interleaved float
 *    pairs (``float2``), real side buffers float; BQA_C128 = complex128 (``double2``),
 *    real side buffers double -- the reference's BQA_PRECISION=single / double
 *    (src/bqa/utils.py:10-30).
 *  - Index maps are int32, node-major: ``in_pos[i*d + k]`` is the message slot of the
 *    edge nbr_k -> node i of the class (the reference keeps the same values k-major,
 *    src/bqa/config/config_canonicalization.py:62-131).
 *  - A node tensor of degree d at bond dim chi is ``[2][chi]...[chi]`` (last bond
 *    fastest); a class stores its B tensors back to back.  Messages are ``[E][chi][chi]``.
 *  - ``stream`` is a cudaStream_t (0 = legacy default stream).  Calls are asynchronous
 *    on that stream and never synchronise the device.
 *  - Every entry point returns a status (BQA_OK = 0).  No entry point aborts, and every
 *    device-side iteration is capped; a cap that is hit is reported through a device
 *    status word, never by spinning.
 *  - Scratch buffers are allocated by the caller and passed in; the library calls no
 *    allocator (bqa_canonicalize_noalloc keeps its scratch in a static device array).
 */
#ifndef BQA_GB300_H
#define BQA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    BQA_OK = 0,
    BQA_ERR_ARG = 1,          /* bad argument (null pointer, negative size, ...) */
    BQA_ERR_UNSUPPORTED = 2,  /* size outside what the kernels are built for */
    BQA_ERR_CUDA = 3          /* a CUDA runtime call failed; see bqa_last_error() */
};

enum { BQA_C64 = 0, BQA_C128 = 1 };

/* message-kernel form of one degree class in a BP sweep (bqa_bp_sweep_plan) */
enum {
    BQA_VARIANT_DEFAULT = 0,  /* the kernel bqa_bp_sweep / bqa_bp_sweep_split launch */
    BQA_VARIANT_TILED = 1,    /* register-tiled: half-node (two-stage sweep) or whole-node (one stage) */
    BQA_VARIANT_GENERIC = 2,  /* generic shared-memory kernel (global-memory form beyond shared memory) */
    BQA_VARIANT_TENSOR = 3,   /* FP32-accurate tensor-core (tcgen05) half-node kernel: bond products
                                 and closing contractions in 2xFP16 (BQA_GB300_TC_KIND=products or
                                 tf32 at library load: 2xFP16 or 3xTF32 products with the closing
                                 contractions on the CUDA cores); two-stage complex64 sweeps of
                                 degree 3 at bond dim 16 */
    BQA_VARIANT_TENSOR_BF16 = 4, /* half-node kernel with BF16 tensor-core products AND closing
                                    contractions (FP32 accumulation; messages ~1e-3 relative),
                                    same shapes as TENSOR */
    BQA_VARIANT_MIXED = 5     /* precision follows the BP loop: with a loop state, a sweep after the
                                 first whose last distance (loop_state[5]) exceeds the switch
                                 (2^-5, or BQA_GB300_MIXED_SWITCH at library load) runs the BF16
                                 kernel, every other sweep the default FP32-accurate half-node
                                 kernel (2xFP16 tensor cores unless BQA_GB300_TC=0);
                                 same shapes as TENSOR */
};

/* device status word bits (written by kernels into a caller int32) */
enum {
    BQA_STATUS_SVD_NOT_CONVERGED = 1, /* a Jacobi SVD hit its sweep cap */
    BQA_STATUS_LAYOUT_EDGE = 2,       /* an edge endpoint outside [0, n), a self-loop, or slot p + E/2
                                         not the reversal of slot p */
    BQA_STATUS_LAYOUT_DEGREE = 4      /* a node's degree exceeds max_degree */
};

/* One degree class: the B nodes of degree d (reference ``Layout``,
 * src/bqa/config/config_canonicalization.py:25-32). */
typedef struct bqa_class {
    int32_t degree;            /* d >= 0 */
    int32_t count;             /* B, number of nodes in the class */
    const int32_t* node_ids;   /* [B]    global node id of each tensor */
    const int32_t* in_pos;     /* [B][d] slot of message nbr_k -> node */
    const int32_t* out_pos;    /* [B][d] slot of message node -> nbr_k */
    const int32_t* lmbd_pos;   /* [B][d] lambda slot of the edge (= out_pos % (E/2)) */
    const double* edge_ampl;   /* [B][d] coupling J of the edge */
    const double* node_ampl;   /* [B]    field h of the node */
    void* tensor;              /* [B][2][chi^d] complex, current tensors */
    void* tensor_out;          /* [B][2][dim^d] complex, written by bqa_apply_update */
    void* scratch;             /* complex work space for node tensors beyond shared memory (or NULL) */
    int64_t scratch_elems;     /* its size in complex elements; see bqa_node_scratch_elems */
} bqa_class;

/* One annealing job's device state and parameters, for bqa_run_layer.  Buffers as for the
 * entry points below; the fields marked "state" are read and updated by each step. */
typedef struct bqa_job {
    int32_t dtype;             /* BQA_C64 / BQA_C128 */
    int32_t n_classes;
    bqa_class* classes;        /* tensor = current buffer, tensor_out = the other (swapped by a step) */
    int32_t edges;             /* E directed edges */
    int32_t max_bond_dim;
    int32_t max_bp_iters;      /* reference max_bp_iter_number (>= 1) */
    int32_t bp_check_every;    /* BP sweeps launched between host reads of the loop state */
    int32_t pad_bonds;         /* bond dims > 4 stored rounded up to a multiple of 4 */
    int32_t split_sweeps;      /* BP sweeps and extended messages in two stages (pm in lu) */
    int32_t colmax_elems;      /* entries of colmax (>= 2 chi) */
    int32_t chi, chis;         /* state: logical and storage bond dim */
    int32_t lam_stride;        /* state: row stride of lmbds */
    int32_t mcur, tcur;        /* state: current message buffer, tensor ping-pong parity */
    double bp_eps, pinv_eps, damping;
    void* msgs[2];             /* [E][chis][chis] each */
    void* ext;                 /* [E][2chi][2chi]: extended messages, then canonicalisers */
    void* lu;                  /* [E][2chi][2chi]; also the blocks of the two-stage passes */
    void* ul;                  /* [E][2chi][2chi] */
    void* lmbds;               /* [E/2][2chi] real */
    void* colmax;              /* [colmax_elems] real bit patterns */
    void* dist_parts;          /* 2 x int64 */
    int32_t* loop_state;       /* 8 x int32 */
    int32_t* status;           /* 1 x int32 */
    const double* edge_j;      /* [E/2] couplings (two-stage extended messages) */
    const int32_t* sweep_variants; /* host [33][n_classes + 1] or NULL (sweeps as split_sweeps says).  Row chis
                                      plans the BP sweeps at storage bond dim chis (bqa_bp_sweep_plan): entry 0
                                      the form (0: as split_sweeps, 1: two-stage, 2: one-stage), entry 1 + c
                                      class c's BQA_VARIANT_*.  Extended messages keep split_sweeps. */
    int32_t blocks_valid;      /* state: lu holds the open-bond blocks of the current messages and tensors
                                  (set by a BP run that converged with two-stage sweeps; the next gate
                                  layer then forms its extended messages with bqa_ext_combine alone and
                                  clears it).  Set it to 0 after changing tensors or messages. */
} bqa_job;

/* What one step did. */
typedef struct bqa_layer_info {
    int32_t bond_dim;          /* bond dim after the truncation */
    int32_t sweeps;            /* BP sweeps run */
    int32_t bp_exhausted;      /* the BP loop hit max_bp_iters */
    int32_t svd_not_converged; /* a Jacobi SVD hit its sweep cap (status word reset) */
    double trunc_err;          /* per-edge truncation error bound */
    double best_dist;          /* last BP distance when exhausted */
} bqa_layer_info;

/*
 * One annealing step (src/bqa/state.py:315-321): the gate layer with BP-gauged truncation
 * (bqa_ext_msgs[_split], bqa_env_factor, bqa_bond_canon, the global truncation decision,
 * bqa_lmbds_truncate, bqa_apply_update, bqa_msgs_from_lmbds) and loopy BP to tolerance
 * (bqa_bp_sweep[_split] + bqa_bp_finalize in groups, the loop state read every
 * bp_check_every sweeps), the same launches and decisions a host would make calling those
 * entry points.  Blocks the calling thread at the two reads of a step.
 */
int32_t bqa_run_layer(bqa_job* job, double xtime, double ztime, bqa_layer_info* info, void* stream);

/*
 * Captured CUDA graphs of BP runs, one cache per job (opaque).  The BP loop of
 * src/bqa/state.py:97-124 launches the same kernels with the same arguments every sweep (the
 * loop state lives on the device), so a whole run -- zero the loop state, sweep + decision +
 * damping under a WHILE node that repeats until the decision kernel marks the run done (at the
 * latest after max_bp_iters sweeps), copy the loop state to the host -- is captured once per
 * (buffers, bond dim, current message buffer, loop parameters) and replayed as ONE graph launch
 * and one host read per BP run.  Create the cache with the job's device current; it owns two
 * non-blocking capture streams, a pinned 32-byte host buffer and up to 16 executable graphs
 * (oldest evicted).  One host thread at a time per cache.
 */
typedef struct bqa_graph_cache bqa_graph_cache;
int32_t bqa_graph_cache_create(bqa_graph_cache** out /* host */);
int32_t bqa_graph_cache_destroy(bqa_graph_cache* cache);

/*
 * bqa_run_layer with its BP run replayed from the cache (captured on first use): the gate
 * layer is launched as in bqa_run_layer (its gate angles change every step), then the BP run
 * is one graph launch.  Same kernels in the same order as bqa_run_layer, minus the sweeps it
 * queues after convergence (those return at once), so the state after the step is
 * bit-identical.  Blocks the calling thread at the two reads of a step.
 */
int32_t bqa_run_layer_graph(bqa_job* job, bqa_graph_cache* cache, double xtime, double ztime, bqa_layer_info* info,
                            void* stream);

/* The BP run alone (src/bqa/state.py:97-124) from the cache; info->sweeps, bp_exhausted and
 * best_dist are filled in, bond_dim is the job's current bond dim. */
int32_t bqa_run_bp_graph(bqa_job* job, bqa_graph_cache* cache, bqa_layer_info* info, void* stream);

/*
 * Packed BP runs: the BP loops of several resident jobs (src/bqa/state.py:97-124, whose per
 * degree-class sweep is the loop at :105-112) in shared launches, for a server that keeps many
 * jobs on one GPU.
 *
 * bqa_gate_layer: the gate layer of bqa_run_layer alone (extended messages, truncation,
 * tensor update, messages from the new lambdas); blocks at its one read (column maxima).
 * bqa_bp_begin: zero the job's loop state and convergence maxima on `stream` (the start of a
 * BP run).  bqa_bp_packed: `sweeps` sweeps of every listed job (1 <= n_jobs <= 64, one dtype);
 * each sweep launches each node kernel ONCE for the classes of all the jobs that use it (the
 * register-tiled half-node kernels, the generic kernel per (degree, bond dim); kernels with
 * per-class scratch or tensor memory one class at a time), one combine for all two-stage
 * jobs and one decision kernel for all loop states, then damping where a job damps.  A job
 * whose loop state says done returns at once from the later sweeps.  Afterwards the jobs'
 * loop states are gathered into loop_states (device, 8 * n_jobs int32) and copied to
 * host_loop_states (8 * n_jobs int32, job i at 8 i); the call blocks until then.
 * bqa_bp_end (host only): conclude a job's BP run whose loop state (host copy, 8 int32) says
 * done: current message buffer, reusable open-bond blocks, info->sweeps / bp_exhausted /
 * best_dist.  A job's state after bqa_gate_layer + bqa_bp_begin + bqa_bp_packed until done +
 * bqa_bp_end is bit-identical to bqa_run_layer's: every CTA computes what it computes in the
 * job's own launches.  Each job's gate layer must be complete (its stream synchronised)
 * before its first packed sweep, and the packed stream's work before the job's next step.
 */
int32_t bqa_gate_layer(bqa_job* job, double xtime, double ztime, bqa_layer_info* info, void* stream);
int32_t bqa_bp_begin(bqa_job* job, void* stream);
int32_t bqa_bp_packed(bqa_job* const* jobs /* host array */, int32_t n_jobs, int32_t sweeps,
                      int32_t* loop_states /* device */, int32_t* host_loop_states, void* stream);
int32_t bqa_bp_end(bqa_job* job, const int32_t* loop_state /* host */, bqa_layer_info* info);

/* ABI version of this header (bumped on any signature change). */
int32_t bqa_abi_version(void);

/* Kernel launches this library has issued in the process so far, all threads together (a
 * launch captured into a CUDA graph counts once, at capture; graph replays do not count). */
int64_t bqa_launch_count(void);

/*
 * Complex elements of scratch one CTA needs to process a class of degree `degree` at bond
 * dim chi (updates to dims <= chi) when its node tensors exceed shared memory, 0 when they
 * fit.  Such a class runs on min(count, scratch_elems / this) CTAs, each walking its share of
 * the nodes with the work tensors in its slice of bqa_class.scratch (the reference handles
 * any degree; this is the path for large chi^d, e.g. degree 5-6 at chi 8).
 */
int64_t bqa_node_scratch_elems(int32_t degree, int32_t chi, int32_t dtype);

/* Text of the last error raised on the calling host thread (static storage). */
const char* bqa_last_error(void);

/* Largest bond dimension the kernels accept for degree d at dtype (0: unsupported). */
int32_t bqa_max_bond_dim(int32_t degree, int32_t dtype);

/*
 * One BP sweep over all classes (src/bqa/state.py:105-113 with
 * Tensor.pass_msgs, src/bqa/backends.py:381-408): for every node and bond k, the message
 * node -> nbr_k is the trace-normalised contraction of conj(T) with T after every other
 * incoming message has been applied.  Every message slot of the output buffer is written,
 * and max|new-old|^2, max|new+old|^2 are folded into dist_parts (2 reals as unsigned bits:
 * uint32[2] for BQA_C64, uint64[2] for BQA_C128; zero them before the first sweep,
 * bqa_bp_finalize re-zeroes them).
 * With loop_state == NULL the sweep reads msgs_a and writes msgs_b.  Otherwise
 * (device-driven loop, see bqa_bp_finalize) it returns at once when loop_state[0] (done)
 * is set, and reads buffer loop_state[2] (0: msgs_a, 1: msgs_b) and writes the other.
 */
int32_t bqa_bp_sweep(const bqa_class* classes /* host array */, int32_t n_classes, int32_t chi, int32_t dtype,
                     void* msgs_a, void* msgs_b, void* dist_parts, const int32_t* loop_state, void* stream);

/*
 * The same sweep as bqa_bp_sweep, in two stages through a caller scratch pm[E][2][chi][chi]:
 * every node writes its phys-resolved open-bond blocks P_0, P_1 of every bond (complex64
 * nodes of degree 2-4 at chi % 4 == 0 run one CTA per (node, physical index), in half the
 * shared memory), then one kernel forms msg = (P_0 + P_1)/tr per slot and the convergence
 * maxima.  Same inputs, outputs and loop_state behaviour as bqa_bp_sweep.  A degree-3
 * half-node CTA whose incoming messages are all exactly diagonal (the first sweep after
 * bqa_msgs_from_lmbds) applies them as bond scalings: the values the dense products give.
 */
int32_t bqa_bp_sweep_split(const bqa_class* classes /* host array */, int32_t n_classes, int32_t chi, int32_t dtype,
                           void* msgs_a, void* msgs_b, void* pm, int32_t edges, void* dist_parts,
                           const int32_t* loop_state, void* stream);

/*
 * One BP sweep with the message kernel of every class chosen by the caller: variants[c]
 * (host int32 [n_classes], BQA_VARIANT_*) for classes[c]; pm != NULL runs the two-stage form
 * of bqa_bp_sweep_split (TILED = half-node kernels, GENERIC = generic open-bond blocks, then one
 * combine pass over all `edges` slots), pm == NULL the one-stage form of bqa_bp_sweep (TILED =
 * whole-node kernels).  TILED is BQA_ERR_UNSUPPORTED where no register-tiled kernel exists
 * (complex64, degree 2-4, chi in {4, 8, 12, 16} minus (2, 4) and (4, 12+)); at degree 3, bond dim
 * 16 it is the CUDA-core half-node kernel.  TENSOR is the tensor-core half-node kernel (two-stage,
 * complex64, degree 3, bond dim 16 only; BQA_ERR_UNSUPPORTED elsewhere), which is also what
 * DEFAULT launches there unless BQA_GB300_TC=0 was set when the library loaded.  GENERIC may carry
 * the CTA size of the shared-memory generic kernel as warps per node in bits 8-15
 * (GENERIC | (w << 8), 1 <= w <= 32; 0 keeps the kernel's own choice: one thread per fibre, at
 * most 8 warps, or 32 for nodes whose shared memory leaves room for at most two CTAs per SM at
 * bond dims <= 8); above 8 warps only at bond dims <= 8 (BQA_ERR_UNSUPPORTED otherwise), and the
 * CTA size does not
 * change the messages (every output is formed by one thread in a fixed order).  Classes whose
 * nodes exceed shared memory keep the global-memory kernel's 256 threads.  variants == NULL is
 * bqa_bp_sweep_split (pm != NULL) or bqa_bp_sweep.  The choices are the search space of the
 * host-side autotuner (bqa_gb300/autotune.py); every variant computes the same messages up to
 * rounding.  Generic-kernel classes of one CTA size go out in one launch where that costs no
 * class an extra wave (BQA_GB300_MERGE_CLASSES=0 at library load: one launch per class; the
 * messages are the same bits).  Same loop_state and dist_parts behaviour as bqa_bp_sweep.
 */
int32_t bqa_bp_sweep_plan(const bqa_class* classes /* host array */, int32_t n_classes, int32_t chi, int32_t dtype,
                          const int32_t* variants /* host */, void* msgs_a, void* msgs_b, void* pm, int32_t edges,
                          void* dist_parts, const int32_t* loop_state, void* stream);

/*
 * Tensor-core kernel health (no reference counterpart): *out (host) = the number of CTAs of the
 * tensor-core kernels whose bounded wait for their MMAs ran out since the library loaded (or
 * since the last reset), 0 in correct operation; such a CTA's output blocks from that
 * half-node on are not valid (left unwritten, or written from incomplete accumulators by the
 * 2xFP16 kernel, which finishes the half-node before it stops), so a non-zero count voids the
 * sweep.
 * reset != 0 zeroes the counter after reading it.  Blocks the calling thread until `stream`
 * has drained.
 */
int32_t bqa_tc_faults(int32_t* out /* host */, int32_t reset, void* stream);

/*
 * BP convergence decision and damping after one sweep (src/bqa/state.py:113-124,
 * Tensor.get_dist src/bqa/backends.py:492-495, damping src/bqa/backends.py:761-764).
 * loop_state is int32[8] = {done, sweeps, cur, exhausted, damp_pending, dist (float bits),
 * best dist (float bits), unused}; zero it (and dist_parts) before the first sweep of a
 * BP run.  When dist < eps the run is done and the current buffer (the sweep's INPUT) is
 * kept; otherwise the current buffer becomes damping*current + (1-damping)*new (a buffer
 * flip when damping == 0).  After sweep max_iters without convergence the run is done
 * with ``exhausted`` set and ``cur`` pointing at the raw output of the last sweep (the
 * reference keeps that buffer too).  Does nothing once done is set.
 */
int32_t bqa_bp_finalize(void* msgs_a, void* msgs_b, int64_t msg_elems, int32_t dtype, void* dist_parts,
                        int32_t* loop_state, double eps, double damping, int32_t max_iters, void* stream);

/*
 * Extended messages of the ZZ-gate layer (src/bqa/state.py:127-139 with the conditional-Z
 * bond extension src/bqa/backends.py:393-404,519-526): for every node and bond k the
 * 2chi x 2chi message of the tensor whose bond k carries half of exp(-i J_k ztime Z Z).
 * Writes ext_out[E][2chi][2chi].
 */
int32_t bqa_ext_msgs(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                     void* ext_out, double ztime, void* stream);

/*
 * bqa_ext_msgs in two stages, the way bqa_bp_sweep_split runs a sweep: the half-node kernels
 * write P_0 and P_1 of every open bond to pm ([edges][2][chi][chi] scratch), then one pass per
 * slot forms the extended message from them with the coupling edge_j[slot % (edges/2)]
 * (edge_j: device double [edges/2], the J of each undirected edge).  Same output as
 * bqa_ext_msgs.
 */
int32_t bqa_ext_msgs_split(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                           void* pm, int32_t edges, const double* edge_j, double ztime, void* ext_out, void* stream);

/*
 * The second stage of bqa_ext_msgs_split alone: extended messages from open-bond blocks
 * pm[edges][2][chi][chi] that are already in place.  A BP run that stopped on convergence
 * keeps its last sweep's input messages (src/bqa/state.py:118-120), and a two-stage sweep
 * leaves in pm the blocks of exactly those messages and the current tensors, so the next
 * step's extended messages need only this pass (bqa_job.blocks_valid).
 */
int32_t bqa_ext_combine(const void* pm, int32_t edges, int32_t chi, int32_t dtype, const double* edge_j, double ztime,
                        void* ext_out, void* stream);

/*
 * Environment factors of every (extended) message m = U S Vh, singular values <= eps
 * dropped (src/bqa/backends.py:483-490,709-727): lu = sqrt(S) Vh and ul = U pinv(sqrt(S)),
 * both [count][n][n], n <= 32.  One-sided Jacobi SVD per matrix in the dtype's precision;
 * a matrix that hits the sweep cap sets BQA_STATUS_SVD_NOT_CONVERGED in *status.
 */
int32_t bqa_env_factor(const void* mats, int32_t count, int32_t n, int32_t dtype, double eps, void* lu, void* ul,
                       int32_t* status, void* stream);

/*
 * Bond canonicalisation (src/bqa/state.py:171-200): for every undirected edge p < E/2,
 * ker = lu[p] lu[p+E/2]^T = us s vhs (masked at eps), lambdas = s/|s| (descending) into
 * lmbds[p][0..n-1] (real), canonicalisers ul[p] us -> canon[p+E/2] and ul[p+E/2] vhs^T ->
 * canon[p], and the max over edges of each lambda column folded into colmax[0..n-1]
 * (real bits, uint32 for BQA_C64, uint64 for BQA_C128; caller zeroes;
 * src/bqa/backends.py:297-303).  edges must be even (BQA_ERR_ARG otherwise): slot p + E/2 is the
 * reversal of slot p.
 */
int32_t bqa_bond_canon(const void* lu, const void* ul, int32_t edges, int32_t n, int32_t dtype, double eps, void* canon,
                       void* lmbds, void* colmax, int32_t* status, void* stream);

/*
 * Tensor update of one annealing step after truncation to bond dim ``dim``: per node,
 * every bond k gets half of its ZZ gate and its canonicaliser (first dim columns of
 * canon[in_pos[k]], src/bqa/backends.py:416-432), then Rz(h ztime) and Rx(xtime)
 * (src/bqa/state.py:142-156), sqrt(lambda) on every bond and per-node L2 normalisation
 * (symmetric gauge, src/bqa/state.py:219-227).  Reads tensor, writes tensor_out.
 * lmbds is real [E/2][lam_stride] with the kept values in the first dim columns.
 */
int32_t bqa_apply_update(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dim, int32_t dtype,
                         const void* canon, const void* lmbds, int32_t lam_stride, double ztime, double xtime,
                         void* stream);

/*
 * Zero the spectrum columns [dim, stride) of every row of lmbds[rows][stride] (real): the
 * columns a truncation to bond dim `dim` removes (src/bqa/backends.py:289-303), when the
 * tensors are stored at a larger, zero-padded bond dimension.
 */
int32_t bqa_lmbds_truncate(void* lmbds, int32_t stride, int32_t rows, int32_t dim, int32_t dtype, void* stream);

/* msgs[e] = diag(lmbds[e % (E/2)][0..dim-1]) / trace (src/bqa/state.py:56-57). */
int32_t bqa_msgs_from_lmbds(const void* lmbds, int32_t lam_stride, int32_t edges, int32_t dim, int32_t dtype,
                            void* msgs, void* stream);

/*
 * Per-node 2x2 marginals (src/bqa/state.py:77-94, src/bqa/backends.py:440-448), written
 * to rho[node_id][2][2].  Degree-0 nodes get psi psi^dagger.
 */
int32_t bqa_densities(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs,
                      void* rho, void* stream);

/*
 * Phys-resolved open-bond blocks P_s of every directed edge slot (unnormalised), written
 * to pm[E][2][chi][chi]; input of bqa_edge_zz.  No reference counterpart (the reference
 * computes no two-site quantity); the definition is oracle/bqa_oracle.py:psplit_msgs.
 */
int32_t bqa_psplit(const bqa_class* classes, int32_t n_classes, int32_t chi, int32_t dtype, const void* msgs, void* pm,
                   void* stream);

/* BP two-site <Z_u Z_v> of every undirected edge p < E/2 from pm, into zz[p] (float64). */
int32_t bqa_edge_zz(const void* pm, int32_t edges, int32_t chi, int32_t dtype, double* zz, void* stream);

/*
 * Projective measurement of m nodes of one class (src/bqa/backends.py:730-734): for each
 * j < m, the outcome-(1 - outcomes[j]) half of node positions[j] is zeroed; then the
 * whole class buffer (count * node_elems complex) is divided by its L2 norm.
 * positions/outcomes are device int32[m]; norm2_scratch is a device double.
 */
int32_t bqa_project_nodes(void* tensors, int32_t count, int32_t node_elems, int32_t dtype, const int32_t* positions,
                          const int32_t* outcomes, int32_t m, double* norm2_scratch, void* stream);

/*
 * bqa_env_factor followed by bqa_bond_canon with no caller scratch.  No counterpart in the
 * reference: it serves callers that cannot allocate device memory (a host whose device heap
 * belongs to an external pool allocator, or a pipeline that must avoid the device-wide
 * synchronisation of cudaMalloc/cudaFree).  The factors lu and ul live in a 64 MiB static
 * device array inside the library, held by every GPU that loads it until process exit, so
 * 2 * edges * n^2 * sizeof(complex) must not exceed 64 MiB (BQA_ERR_UNSUPPORTED otherwise;
 * e.g. 65,536 edges at n = 8 or 4,096 at n = 32 in complex64).  Inputs: ext_msgs[edges][n][n].
 * Outputs as bqa_bond_canon (canon, lmbds, status bits OR-ed in); colmax is zeroed here
 * before it is filled.  The first call on a device looks up the array's device address, so
 * make it before any stream capture; that address is cached per device ordinal and does not
 * survive cudaDeviceReset.  Calls share the array: calls that overlap on the GPU race.  edges
 * must be even (BQA_ERR_ARG otherwise).  When the return code is not BQA_OK, every output
 * (canon, lmbds, colmax, status) is undefined: the call may have cleared or partly written them.
 */
int32_t bqa_canonicalize_noalloc(const void* ext_msgs, int32_t edges, int32_t n, int32_t dtype, double eps,
                                 void* canon, void* lmbds, void* colmax, int32_t* status, void* stream);

/*
 * Degree-class compilation on the device, first stage (replaces the per-node loop of
 * _make_degree_to_layout, src/bqa/config/config_canonicalization.py:62-131).
 * edges: int32 [E][2] (src, dst) in message-slot order, E even, slot p + E/2 the reversal of
 * slot p (the reference's edge dict: user edges, then their reversals).  Outputs
 * (caller-allocated device int32): deg[n]; start[n] = exclusive scan of deg; order[E] = the
 * slots grouped by source node, increasing slot inside a group (bond k of node v is
 * order[start[v] + k]); class_first[max_degree + 1] = lowest node id of each degree (only
 * meaningful where class_count > 0); class_count[max_degree + 1].  fill[n] is scratch.
 * Bad edges set BQA_STATUS_LAYOUT_EDGE and nodes of degree > max_degree
 * BQA_STATUS_LAYOUT_DEGREE in *status; the outputs are then undefined.  The host orders the
 * classes by class_first (first appearance over node ids, as the reference's dict does).
 */
int32_t bqa_layout_degrees(const int32_t* edges, int32_t E, int32_t n, int32_t max_degree, int32_t* deg,
                           int32_t* start, int32_t* order, int32_t* fill, int32_t* class_first,
                           int32_t* class_count, int32_t* status, void* stream);

/*
 * Second stage, one call per degree class (reference ``Layout`` fields,
 * src/bqa/config/config_canonicalization.py:25-32,82-131): node_ids[count] = the nodes of
 * this degree in increasing id; position[v] = index of v in its class (written for this
 * class's nodes); node-major [count][degree] maps out_pos (slot node -> nbr_k), in_pos
 * ((out + E/2) % E), lmbd_pos (out % (E/2)), edge_ampl (slot_ampl[out], the coupling J);
 * node_ampl[count] = node_field[v].  in_pos, lmbd_pos, edge_ampl, node_ampl may be NULL.
 */
int32_t bqa_layout_class(int32_t degree, int32_t count, const int32_t* deg, const int32_t* start,
                         const int32_t* order, int32_t n, int32_t E, const double* slot_ampl,
                         const double* node_field, int32_t* node_ids, int32_t* position, int32_t* in_pos,
                         int32_t* out_pos, int32_t* lmbd_pos, double* edge_ampl, double* node_ampl, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BQA_GB300_H */
