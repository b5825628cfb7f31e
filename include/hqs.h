/*
 * hqs.h - C ABI of the GB300 state-vector engine (libhqs.so).
 *
 * Drop-in boundary for the C++ engine behind HiQ's SimulatorMPI ProjectQ
 * backend. The reference binds the engine to Python with pybind11
 * (_cppsim_mpi.cpp:61-83); this library exposes the same operations as plain
 * C functions over an opaque handle, and hiqsimulator_gb300/_cppsim_mpi is a
 * pybind11 module with the reference's class and method names built on top
 * of it. Every function returns HQS_OK or an error code; the message of the
 * last error on a handle is hqs_sim_last_error(). Errors that the reference
 * raises as std::runtime_error (RuntimeError in Python) return
 * HQS_ERR_RUNTIME with the reference's message.
 *
 * Layout: a state of n qubits is 2^n complex amplitudes in position order
 * (bit p of the index is the qubit at position p), complex128 values as
 * interleaved (re, im) doubles like std::complex<double>. Matrices are
 * dim x dim, row-major, interleaved complex128. Bit j of a matrix index acts
 * on qubit ids[j].
 *
 * Threading: a handle is used by one host thread at a time (the reference
 * runs MPI_THREAD_FUNNELED, SimulatorMPI.cpp:73). Different handles are
 * independent and may run concurrently; each owns a CUDA stream.
 */
#ifndef HQS_H
#define HQS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HQS_OK 0
#define HQS_ERR_RUNTIME 1  /* reference std::runtime_error */
#define HQS_ERR_INVALID 2  /* bad argument (null pointer, short buffer, bad enum) */
#define HQS_ERR_CUDA 3     /* CUDA failure; message names the call */
#define HQS_ERR_MEMORY 4   /* host or device allocation failed */

#define HQS_C128 0 /* complex128 state */
#define HQS_C64 1  /* complex64 state */

#define HQS_ARITH_AUTO 0 /* c128 -> TC, c64 -> TC64 */
#define HQS_ARITH_F64 1  /* native FP64 */
#define HQS_ARITH_DF 2   /* double-float (2 x FP32), ~48-bit */
#define HQS_ARITH_F32 3  /* FP32 (complex64 states) */
#define HQS_ARITH_TC 4   /* complex128: dense 3-5 qubit gates as exact fp16 digit products on the
                            tensor cores (six digits per real; tensor-memory pass from 12 qubits),
                            everything else double-float */
#define HQS_ARITH_TF32 5 /* complex64: dense 3-5 qubit gates as 3xTF32 products on the tensor
                            cores (hi*hi + hi*lo + lo*hi, FP32 accumulate), everything else FP32.
                            The tensor cores' accumulation rounds toward zero; each k-step's
                            products are summed apart and added with round-to-nearest, which
                            leaves a norm loss of about 7e-8 per dense 5-qubit gate (measured). */
#define HQS_ARITH_TC64 6 /* complex64: dense 3-5 qubit gates as exact fp16 digit products on the
                            tensor cores (3 state x 4 gate digits in the tensor-memory pass from
                            12 qubits, exact levels: no truncation bias; two digits below 12 qubits
                            and in serving batches), everything else FP32. hqs_sim / hqs_server
                            map HQS_ARITH_TC with HQS_C64 to this. */

typedef struct hqs_sim hqs_sim;

/* Message of the last failed call on this thread that had no handle
 * (hqs_sim_create, kernel-level calls). */
const char* hqs_last_error(void);
/* Library version string. */
const char* hqs_version(void);

/* ------------------------------------------------------------------------
 * Engine-level API: one entry per method of _cppsim_mpi.SimulatorMPI.
 * ------------------------------------------------------------------------ */

/* SimulatorMPI(seed, max_local, max_cluster_size): _cppsim_mpi.cpp:64,
 * SimulatorMPI.cpp:66-104. precision: HQS_C128 / HQS_C64; arith: HQS_ARITH_*. */
int hqs_sim_create(uint64_t seed, int64_t max_local, int64_t max_cluster_size, int precision, int arith,
                   hqs_sim** out);
void hqs_sim_destroy(hqs_sim* sim);
const char* hqs_sim_last_error(const hqs_sim* sim);

/* allocate_qubit: _cppsim_mpi.cpp:71, SimulatorMPI.cpp:184-216. */
int hqs_sim_allocate_qubit(hqs_sim* sim, int64_t id);
/* allocate_qureg(ids, init): _cppsim_mpi.cpp:70, SimulatorMPI.cpp:218-251. */
int hqs_sim_allocate_qureg(hqs_sim* sim, const int64_t* ids, size_t n, double init_re, double init_im);
/* deallocate_qubit: _cppsim_mpi.cpp:72, SimulatorMPI.cpp:369-426. */
int hqs_sim_deallocate_qubit(hqs_sim* sim, int64_t id);
/* apply_controlled_gate(matrix, ids, ctrls): _cppsim_mpi.cpp:74, SimulatorMPI.cpp:710-815.
 * m: dim*dim interleaved complex128, row-major; dim == 2^nids. Queues only. */
int hqs_sim_apply_controlled_gate(hqs_sim* sim, const double* m, size_t dim, const int64_t* ids, size_t nids,
                                  const int64_t* ctrls, size_t nctrls);
/* run(): _cppsim_mpi.cpp:78, SimulatorMPI.cpp:441-541. Fuses the queued gates
 * and schedules the fused gate on the device (asynchronously). */
int hqs_sim_run(hqs_sim* sim);
/* measure_qubits(ids): _cppsim_mpi.cpp:73, SimulatorMPI.cpp:897-1008. out[i] = 0/1. */
int hqs_sim_measure_qubits(hqs_sim* sim, const int64_t* ids, size_t n, uint8_t* out);
/* get_probability(bits, ids): _cppsim_mpi.cpp:77, SimulatorMPI.cpp:561-600. */
int hqs_sim_get_probability(hqs_sim* sim, const uint8_t* bits, size_t nbits, const int64_t* ids, size_t nids,
                            double* out);
/* get_amplitude(bits, ids): _cppsim_mpi.cpp:76, SimulatorMPI.cpp:602-650. out: (re, im). */
int hqs_sim_get_amplitude(hqs_sim* sim, const uint8_t* bits, size_t nbits, const int64_t* ids, size_t nids,
                          double* out);
/* collapse_wavefunction(ids, values): _cppsim_mpi.cpp:81, SimulatorMPI.cpp:1010-1058. */
int hqs_sim_collapse_wavefunction(hqs_sim* sim, const int64_t* ids, size_t nids, const uint8_t* values,
                                  size_t nvalues);
/* entropy(): _cppsim_mpi.cpp:79, SimulatorMPI.cpp:681-694. */
int hqs_sim_entropy(hqs_sim* sim, double* out);
/* number of allocated qubits (size of the id lists below). */
int hqs_sim_num_qubits(const hqs_sim* sim, size_t* out);
/* get_qubits_ids / get_local_qubits_ids / get_global_qubits_ids:
 * _cppsim_mpi.cpp:65-68, SimulatorMPI.cpp:652-679. out: position order; *n
 * receives the count (the global list is always empty on one device). */
int hqs_sim_get_qubits_ids(const hqs_sim* sim, int64_t* out, size_t cap, size_t* n);
int hqs_sim_get_local_qubits_ids(const hqs_sim* sim, int64_t* out, size_t cap, size_t* n);
int hqs_sim_get_global_qubits_ids(const hqs_sim* sim, int64_t* out, size_t cap, size_t* n);
/* set_qubits_perm(ids): _cppsim_mpi.cpp:68, SimulatorMPI.cpp:661-667 (relabels, no data movement). */
int hqs_sim_set_qubits_perm(hqs_sim* sim, const int64_t* ids, size_t n);
/* swap_qubits(pairs): _cppsim_mpi.cpp:69, SimulatorMPI.cpp:1060-1138. Pairs are
 * (global id, local id); one device has no global qubits, so a non-empty list
 * fails exactly like the reference's lookup. */
int hqs_sim_swap_qubits(hqs_sim* sim, const int64_t* pairs, size_t n);
/* cheat_local(): _cppsim_mpi.cpp:80, SimulatorMPI.cpp:543-559. Copies the 2^n
 * amplitudes (position order, interleaved complex128) into out (cap amplitudes). */
int hqs_sim_cheat_local(hqs_sim* sim, double* out, size_t cap);
/* emulate_math: _cppsim_mpi.cpp:75, SimulatorMPI.hpp:218-225: always fails
 * with "SimulatorMPI::emulate_math() is not supported". */
int hqs_sim_emulate_math(hqs_sim* sim);

/* Pauli operators, encoded as nterms terms; term t has the factors
 * [term_off[t], term_off[t+1]) of (qubit index into ids, 'X'|'Y'|'Z') and the
 * complex coefficient (coefs[2t], coefs[2t+1]). These are the calls the Python
 * backend makes at hiq/projectq/backends/_sim/_simulator_mpi.py:182-183 and
 * :222-223 that the reference engine never bound. */
int hqs_sim_get_expectation_value(hqs_sim* sim, size_t nterms, const size_t* term_off, const int64_t* factor_index,
                                  const char* factor_pauli, const double* coefs, const int64_t* ids, size_t nids,
                                  double* out);
/* Several expectation values in one call (extension; no reference
 * counterpart): operator o is the terms [op_off[o], op_off[o + 1]) of the
 * term arrays laid out as for hqs_sim_get_expectation_value (term t has
 * factors [term_off[t], term_off[t + 1]) and coefficient coefs[2t] + i
 * coefs[2t + 1]); out[o] receives its value. The distinct Z strings of the
 * operators made only of Z factors share one read of the state per 64
 * strings; other operators take one hqs_sim_get_expectation_value each. */
int hqs_sim_get_expectation_values(hqs_sim* sim, size_t nops, const size_t* op_off, const size_t* term_off,
                                   const int64_t* factor_index, const char* factor_pauli, const double* coefs,
                                   const int64_t* ids, size_t nids, double* out);
int hqs_sim_apply_qubit_operator(hqs_sim* sim, size_t nterms, const size_t* term_off, const int64_t* factor_index,
                                 const char* factor_pauli, const double* coefs, const int64_t* ids, size_t nids);
/* set_wavefunction(wf, ids): called at _simulator_mpi.py:305-306. wf: len
 * interleaved complex128 amplitudes; ids: every allocated qubit, in the order
 * the simulator adopts (ids[j] -> position j). */
int hqs_sim_set_wavefunction(hqs_sim* sim, const double* wf, size_t len, const int64_t* ids, size_t nids);

/* --- extensions (no reference counterpart) --- */
/* Launch every pending fused gate and wait for the device. */
int hqs_sim_synchronize(hqs_sim* sim);
/* shots full-register samples without collapse, one draw each from the
 * simulator's RNG; out[s] = sampled basis index in position order. */
int hqs_sim_sample(hqs_sim* sim, uint64_t shots, uint64_t* out);
/* Move qubits ids[i] to positions[i] with one in-place bit-permutation sweep
 * (at most 12 positions change). */
int hqs_sim_move_qubits(hqs_sim* sim, const int64_t* ids, const int* positions, size_t n);
/* Fused-pass planner limits: tile bits (<= 12), gates per pass (<= 24),
 * pending fused gates before an automatic launch. 0 keeps a value. */
int hqs_sim_set_pass_limits(hqs_sim* sim, int max_tile_bits, int max_ops, int defer);
/* Counters: gates, runs, passes, pass_ops, bytes_moved, flushes. */
int hqs_sim_stats(const hqs_sim* sim, uint64_t out[6]);
/* Precision and arithmetic of the handle. */
int hqs_sim_info(const hqs_sim* sim, int* precision, int* arith);
/* Zero-copy view of the state (the device-side counterpart of cheat_local,
 * SimulatorMPI.cpp:543-559): launches every pending fused gate, waits for the
 * device, and returns the device address of the 2^n amplitudes in position
 * order (interleaved complex128, or interleaved complex64 for HQS_C64), their
 * count and the CUDA device ordinal. The address stays valid until the handle
 * is destroyed or a call allocates or deallocates a qubit, applies a qubit
 * operator or sets the wavefunction; later passes change the contents in
 * place. Device writes through the view must be complete before the next
 * call on the handle (the handle's stream does not wait for other streams). */
int hqs_sim_state_view(hqs_sim* sim, void** state, uint64_t* amplitudes, int* device);
/* Device timing on the handle's stream: start records an event after every
 * pending fused gate is launched; stop records a second one, waits for it and
 * returns the elapsed milliseconds. */
int hqs_sim_timer_start(hqs_sim* sim);
int hqs_sim_timer_stop(hqs_sim* sim, float* ms);
/* Per-launch timing of the apply passes: while on, CUDA events bracket every
 * pass launch; hqs_sim_pass_timing waits for them and returns the number of
 * launches, their algorithmic HBM bytes and summed device milliseconds since
 * the previous call. */
int hqs_sim_set_pass_timing(hqs_sim* sim, int on);
int hqs_sim_pass_timing(hqs_sim* sim, uint64_t* launches, uint64_t* bytes, double* ms);
/* The launches behind the last hqs_sim_pass_timing call, in launch order:
 * kernel (HQS_KERNEL_PASS: the tiled pass kernel; HQS_KERNEL_UMMA: the
 * tensor-memory pass), gate ops applied, TMA copies per tile and target
 * positions of a tensor-memory pass, algorithmic HBM bytes and device
 * milliseconds. Up to cap records are written; *count receives the total. */
#define HQS_KERNEL_PASS 0
#define HQS_KERNEL_UMMA 1
typedef struct {
    int32_t kernel;
    int32_t nops;
    int32_t copies;        /* HQS_KERNEL_UMMA: TMA copies per tile (else 0) */
    int32_t pad;
    uint64_t target_mask;  /* HQS_KERNEL_UMMA: the dense gate's five (padded) target positions */
    uint64_t bytes;
    double ms;
} hqs_pass_record;
int hqs_sim_pass_log(hqs_sim* sim, hqs_pass_record* out, size_t cap, size_t* count);

/* Greedy fusion schedule (the rule of HiQ's GreedyScheduler + ClusterScheduler,
 * hiq/projectq/cengines/_greedyscheduler.py:119-137,
 * src/scheduler/cluster_scheduler.cpp:41-99): gate g has targets
 * tgt[toff[g]..toff[g+1]) and controls ctl[coff[g]..coff[g+1]); every gate is
 * treated as non-diagonal. order[] receives gate indices in emission order and
 * cluster_end[c] the end of cluster c in order[]; *nclusters the count. */
int hqs_greedy_schedule(int ngates, const int64_t* tgt, const int* toff, const int64_t* ctl, const int* coff,
                        int nlocals, const int64_t* locals, int cluster_size, int* order, int* cluster_end,
                        int* nclusters);

/* Host FP64 gate fusion (fusion_mpi.hpp:85-226, SimulatorMPI.cpp:710-815), no
 * device: gate g is a dim[g] x dim[g] row-major complex128 matrix (the
 * matrices concatenated in m as interleaved doubles) on targets
 * ids[ioff[g]..ioff[g+1]) with controls ctrls[coff[g]..coff[g+1]); each is
 * tested for exact diagonality and inserted in order, then the queue is fused
 * into one gate: out_m (2^n_ids x 2^n_ids, cap_m complex values), its qubit
 * ids ascending (matrix bit l <-> out_ids[l]), the controls every gate shared
 * (ascending) and whether it is diagonal. At most 12 fused qubits. */
int hqs_fuse(size_t ngates, const double* m, const size_t* dim, const int64_t* ids, const size_t* ioff,
             const int64_t* ctrls, const size_t* coff, double* out_m, size_t cap_m, int64_t* out_ids,
             size_t cap_ids, size_t* n_ids, int64_t* out_ctrls, size_t cap_ctrls, size_t* n_ctrls, int* out_diag);

/* ------------------------------------------------------------------------
 * Batched circuit server (no reference counterpart): many independent
 * circuits resident in HBM, admitted in arrival order against a byte budget
 * (2^n x bytes per amplitude) and advanced together, one fused pass per
 * circuit per round in a single batched launch.
 * ------------------------------------------------------------------------ */
typedef struct hqs_server hqs_server;

#define HQS_RESULT_AMPLITUDE0 0  /* <0...0|psi> */
#define HQS_RESULT_SAMPLE 1      /* one full-register sample for the given uniform draw */
#define HQS_RESULT_EXPECTATION 2 /* sum_t Re(c_t <psi|P_t|psi>) */

typedef struct {
    uint64_t id;
    int kind;
    double value_re, value_im; /* amplitude, or the expectation in value_re */
    uint64_t sample;           /* basis index for HQS_RESULT_SAMPLE */
    double submit_s, admit_s, done_s;
    uint32_t passes;
} hqs_server_result;

/* precision HQS_C128 / HQS_C64; arith as for hqs_sim_create; budget_bytes:
 * HBM for resident states; max_active: resident circuits at most;
 * cluster_size: gates are fused while their qubits fit (<= 5). */
int hqs_server_create(int precision, int arith, uint64_t budget_bytes, int max_active, int cluster_size,
                      hqs_server** out);
void hqs_server_destroy(hqs_server* srv);
const char* hqs_server_last_error(const hqs_server* srv);
/* Queue a circuit on n qubits: gate g has ntgt[g] targets and nctl[g]
 * controls (qubit indices 0..n-1, concatenated in tgt / ctl) and a
 * 2^ntgt x 2^ntgt row-major complex128 matrix (concatenated in mats). For
 * HQS_RESULT_EXPECTATION, nterms Pauli terms are given as x / y / z bit masks
 * over qubit indices and complex coefficients. */
int hqs_server_submit(hqs_server* srv, int n, int ngates, const int* ntgt, const int* tgt, const int* nctl,
                      const int* ctl, const double* mats, int kind, double rnd, size_t nterms, const uint64_t* px,
                      const uint64_t* py, const uint64_t* pz, const double* coefs, uint64_t* id_out);
/* One round; completed results go to out (cap entries), their count to *n. */
int hqs_server_step(hqs_server* srv, hqs_server_result* out, size_t cap, size_t* n);
/* queued, resident, bytes in use, rounds, launches */
int hqs_server_info(const hqs_server* srv, uint64_t out[5]);
/* Host seconds spent in step() since creation: out[0] batching (items and
 * matrix staging), out[1] waiting for a staging buffer to be free, out[2]
 * launches, out[3] results of finished circuits, out[4] admissions, out[5]
 * all of step(). No reference counterpart (diagnostics of the server). */
int hqs_server_timing(const hqs_server* srv, double out[6]);

/* ------------------------------------------------------------------------
 * Kernel-level API on device memory (one fused gate / reduction per call).
 * state: device pointer to 2^n amplitudes (complex128 for HQS_ARITH_F64/DF/TC,
 * complex64 for HQS_ARITH_F32/TF32/TC64). stream: a cudaStream_t or NULL. Calls are
 * asynchronous except those returning a value to the host.
 * ------------------------------------------------------------------------ */
typedef struct hqs_ws hqs_ws;
int hqs_ws_create(hqs_ws** out);
void hqs_ws_destroy(hqs_ws* ws);
/* Apply nops fused gates in order (kernelK / kernelK_diag1 of
 * src/simulator-mpi/kernels/nointrin/, dispatched as in SimulatorMPI.cpp:470-524).
 * Gate i: k[i] targets at positions pos[5*i .. 5*i+k[i]) (matrix bit j <->
 * pos[5*i+j]), control mask ctrl[i], diag[i] != 0 for a diagonal gate. Its
 * matrix starts at mats (interleaved complex128) after the previous gates':
 * 4^k entries for a dense gate, 2^k (the diagonal) for a diagonal one, 1 for
 * k == 0. Gates are grouped into tiled passes of at most max_tile_bits tile
 * bits and max_ops gates (0 = defaults). *bytes_out (optional) receives the
 * algorithmic HBM bytes, *passes_out (optional) the number of sweeps. */
/* How hqs_apply_gates would group the same gates into passes, computed on
 * the host (no GPU, no matrices needed). No reference counterpart (the
 * reference runs one sweep per fused gate). *npasses receives the count;
 * the first cap passes are described in out. */
typedef struct {
    uint32_t first_op, nops;   /* the pass applies gates [first_op, first_op + nops) */
    uint32_t q, w;             /* tile bits; tile positions 0..w-1 are the contiguous low run */
    uint32_t prefetch;         /* 0 none, 1 staging buffer, 2 every gate in place, second tile buffer */
    uint32_t tc_ops;           /* gates on the tensor cores */
    uint64_t tile_mask;        /* state positions in the tile */
    uint64_t fixed_mask;       /* control positions outside the tile every gate shares */
    uint64_t smem_bytes, pool_bytes, sweep_bytes;
} hqs_pass_info;
int hqs_plan_passes(int n, int arith, int nops, const int* k, const int* pos, const uint64_t* ctrl, const int* diag,
                    int max_tile_bits, int max_ops, hqs_pass_info* out, size_t cap, size_t* npasses);

/* The launches hqs_apply_gates makes for the same gates, computed on the host
 * (no GPU): with HQS_ARITH_TC (complex128) or HQS_ARITH_TC64 (complex64) on
 * states of 12 or more qubits, every dense gate on 3-5 qubits gets a
 * tensor-memory pass (tcgen05 tensor cores, TMA tile copies) together with
 * the diagonal / scalar gates around it; the rest are
 * tiled passes as in hqs_plan_passes. No reference counterpart (the reference
 * runs one sweep per fused gate, SimulatorMPI.cpp:441-541). *nlaunches
 * receives the count; the first cap launches are described in out. */
typedef struct {
    uint32_t first_op, nops;   /* the launch applies gates [first_op, first_op + nops) */
    uint32_t umma;             /* 1: tensor-memory pass */
    uint32_t tc_op;            /* tensor-memory pass: index (within the launch) of the dense gate */
    uint64_t tile_mask;        /* state positions in the tile */
    uint64_t target_mask;      /* tensor-memory pass: the five target positions (padded) */
    uint64_t fixed_mask;       /* control positions outside the tile every gate shares */
    uint32_t rank, nextra;     /* tensor-memory pass: TMA tensor rank, tile bits fetched as separate copies */
    uint32_t box_bytes;        /* tensor-memory pass: bytes of one TMA box */
    int32_t dim_kind[5], dim_pos[5], dim_bits[5];  /* TMA dimensions: 1 box run + gap above it, 2 the same
                                                      with extra tile bits (last); first position; positions */
    int32_t dim_box[5];        /* of each dimension's positions, the box run at its bottom */
    uint64_t pool_bytes, sweep_bytes;
} hqs_launch_info;
int hqs_plan_launches(int n, int arith, int nops, const int* k, const int* pos, const uint64_t* ctrl, const int* diag,
                      int max_tile_bits, int max_ops, hqs_launch_info* out, size_t cap, size_t* nlaunches);

int hqs_apply_gates(hqs_ws* ws, void* state, int n, int arith, int nops, const int* k, const int* pos,
                    const uint64_t* ctrl, const int* diag, const double* mats, int max_tile_bits, int max_ops,
                    uint64_t* bytes_out, uint64_t* passes_out);
/* Sum of |a_i|^2 over (i & mask) == val (getProbability_internal, SimulatorMPI.cpp:841-870). */
int hqs_probability(hqs_ws* ws, const void* state, int n, int arith, uint64_t mask, uint64_t val, double* out);
/* nblocks block sums of |a|^2 (calcLocalApproxDistribution before the prefix
 * sum, SimulatorMPI.cpp:817-839); out: host array of nblocks doubles. */
int hqs_block_sums(hqs_ws* ws, const void* state, int n, int arith, uint64_t nblocks, double* out);
/* Zero (i & mask) != val, scale the rest by scale (normalize, SimulatorMPI.cpp:872-895). */
int hqs_collapse(hqs_ws* ws, void* state, int n, int arith, uint64_t mask, uint64_t val, double scale);
/* In-place bit permutation: state bit newpos[j] receives old bit oldpos[j] (m <= 12). */
int hqs_permute_bits(hqs_ws* ws, void* state, int n, int arith, int m, const uint8_t* oldpos, const uint8_t* newpos);
/* Remove bit pos keeping the half where it equals keep (DeallocateLocalQubit
 * compaction, SimulatorMPI.cpp:303-318), in place. */
int hqs_drop_bit(hqs_ws* ws, void* state, int n, int arith, int pos, int keep);
/* Probability sum for callers that cannot allocate device memory (no
 * counterpart in the reference). Same result as hqs_probability, but every
 * scratch byte lives in a fixed 32 KiB __device__ array inside libhqs.so and
 * the sum is written to the caller's device pointer d_out on `stream` (a
 * cudaStream_t, NULL for the legacy default stream), asynchronously; nothing
 * is allocated, freed or synchronized. For code that runs under a foreign
 * memory pool or inside recorded launch sequences, where cudaMalloc is not
 * allowed. Limit: states of at most 2^40 amplitudes (n <= 40); larger
 * requests fail with HQS_ERR_INVALID before any launch. All calls on a device
 * share the array, so calls that overlap on the GPU race; the first call on a
 * device looks the array up and should come before any stream capture, and
 * the entry point must not be used on a device after cudaDeviceReset. */
int hqs_probability_noalloc(const void* state, int n, int arith, uint64_t mask, uint64_t val, double* d_out,
                            void* stream);
/* Wait for the workspace's stream. */
int hqs_ws_synchronize(hqs_ws* ws);
/* Device timing of the workspace's stream: start records an event; stop
 * records a second one, waits for it and returns the elapsed milliseconds. */
int hqs_ws_timer_start(hqs_ws* ws);
int hqs_ws_timer_stop(hqs_ws* ws, float* ms);

#ifdef __cplusplus
}
#endif

#endif /* HQS_H */
