/*
 * mbqc_gb300.h -- C ABI of the GB300 windowed-MBQC sweep library
 * (libmbqc_gb300.so).
 *
 * The library replaces the compute path behind mentpy's
 * ``PatternSimulator(circuit, backend="numpy-sv" | "numpy-dm")``:
 *
 *   mentpy/simulators/np_simulator_sv.py:227-297   NumpySimulatorSV.run
 *   mentpy/simulators/np_simulator_dm.py:218-283   NumpySimulatorDM.run
 *
 * Conventions
 *   - Every function returns MBQC_OK (0) or a negative MBQC_E_* code; no C++
 *     exception crosses the ABI.  mbqc_last_error() gives the message of the
 *     calling thread's last failure.
 *   - Device buffers are owned by the caller and passed as plain pointers;
 *     complex numbers are interleaved (re, im) pairs: "complex64" means pairs
 *     of float, "complex128" pairs of double.  Strides count elements
 *     (complex elements for state arrays, doubles for angle arrays).
 *   - ``stream`` is a cudaStream_t (NULL = the legacy default stream); all
 *     work is stream-ordered and asynchronous with respect to the host.
 *   - A plan is immutable after creation and may be used concurrently from
 *     several host threads and streams.
 *   - Amplitude index conventions follow mentpy: the first qubit of a list is
 *     the most significant bit of the state index (np.kron order).
 */
#ifndef MBQC_GB300_H
#define MBQC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MBQC_ABI_VERSION 2

#define MBQC_OK 0
#define MBQC_E_INVALID (-1)     /* bad argument / plan mismatch          */
#define MBQC_E_CUDA (-2)        /* CUDA runtime error                     */
#define MBQC_E_UNSUPPORTED (-3) /* window or plane outside the kernels    */
#define MBQC_E_NOMEM (-4)       /* allocation failed                      */

/* per-run status word written by the kernels */
#define MBQC_RUN_OK 0
#define MBQC_RUN_ZERO_NORM 1 /* projected state vanished: output is NaN, as the
                                reference's 0/0 normalisation gives          */
#define MBQC_RUN_NAN 2       /* NaN/Inf met (density matrix: the reference
                                raises ValueError, np_simulator_dm.py:179-182) */

/* flags for the forward entry points */
#define MBQC_F_REF_PHASE 1u /* statevector output carries the global phase the
                               reference's summing partial trace leaves
                               (state_ops.py:69,73): prod_k (v0+v1)/|v0+v1| */

#define MBQC_F_HOST_INPUTS 2u /* angles and input states are page-locked host
                                 memory read in place (mbqc_mapped_pointer):
                                 the register-resident statevector kernel
                                 loads them uncached (ld.global.cv), so every
                                 launch fetches them over the CPU-GPU link */

#define MBQC_F_DM_EXPECTATION 4u /* density matrix, mode="expectation": Z steps
                                     trace the qubit out unprojected and
                                     report prob1/(prob0+prob1) in probs */

#define MBQC_F_INPUTS_READY 8u /* mbqc_sv_forward: the caller guarantees that
                                  no earlier work on the stream writes this
                                  call's angles or input states (they were
                                  filled by the host, or before the loop).
                                  The kernel then reads them and runs its
                                  sweep while that work finishes, and waits
                                  for it only before its first write; the
                                  default waits before reading them. */

#define MBQC_F_DM_FULL_MATRIX 16u /* density matrix: keep the full 2^w x 2^w rho
                                     (windows <= 7) instead of the factored
                                     form; the same results to float rounding */

#define MBQC_F_STREAM_TMA 32u /* mbqc_sv_forward_stream: stage the tiles of the
                                 mixed passes with TMA bulk copies (one per
                                 256-byte row, completing on an mbarrier)
                                 instead of 16-byte asynchronous copies; the
                                 same results bit for bit */

/* measurement planes of a plan step */
#define MBQC_PLANE_XY 0
#define MBQC_PLANE_X 1
#define MBQC_PLANE_Y 2
#define MBQC_PLANE_XZ 3
#define MBQC_PLANE_YZ 4
#define MBQC_PLANE_Z 5   /* density matrix only: outcome drawn, or with
                            MBQC_F_DM_EXPECTATION recorded as prob1/(prob0+prob1)
                            without projection (np_simulator_dm.py:327-344)   */

/* step_mask bit: no qubit enters after this step (the window shrinks) */
#define MBQC_STEP_DEAD 0x80000000u

typedef void *mbqc_stream_t; /* cudaStream_t */
typedef struct mbqc_plan mbqc_plan;

/*
 * One compiled window plan (host memory, copied by mbqc_plan_create).
 * Replaces the window bookkeeping of NumpySimulatorSV.__init__ /
 * NumpySimulatorDM.__init__ (np_simulator_sv.py:38-128,
 * np_simulator_dm.py:33-115) and the per-step node lookups of
 * ``measure`` (np_simulator_sv.py:164-225).  Window slot of schedule
 * position j is physical index bit (j mod window); the qubit measured at
 * step k sits on bit (k mod window) and the qubit entering after it reuses
 * that bit.
 */
typedef struct mbqc_circuit_desc {
  int32_t window;                 /* w, 1..30                                   */
  int32_t n_steps;                /* M = number of measured nodes               */
  int32_t n_in;                   /* input qubits                               */
  int32_t n_out;                  /* output qubits                              */
  int32_t n_angles;               /* length of one angle vector                 */
  const int32_t *in_bits;         /* [n_in]   physical bit of input qubit i     */
  const int32_t *out_bits;        /* [n_out]  physical bit of output qubit j    */
  const uint32_t *init_cz;        /* [window] CZ partners (higher bits) of bit q
                                     inside the first window                    */
  const uint32_t *step_mask;      /* [n_steps] CZ partners of the entering qubit,
                                     or MBQC_STEP_DEAD                          */
  const int32_t *step_angle;      /* [n_steps] angle-vector index, -1 = fixed   */
  const int32_t *step_plane;      /* [n_steps] MBQC_PLANE_*                     */
  const double *step_fixed_angle; /* [n_steps] angle used when step_angle = -1  */
} mbqc_circuit_desc;

/*
 * An open graph with its measurements, for the native plan compiler.
 * Node i of the arrays is label nodes[i]; the array order is the graph's node
 * order (networkx insertion order), which decides ties of the measurement
 * order as in MBQCircuit.calculate_order (mbqcircuit.py:390-422).
 */
typedef struct mbqc_graph_desc {
  int32_t n_nodes;
  const int32_t *nodes;           /* [n_nodes] labels in graph order            */
  int32_t n_edges;
  const int32_t *edges;           /* [n_edges][2] labels                        */
  int32_t n_inputs;
  const int32_t *inputs;          /* [n_inputs] labels, input order             */
  int32_t n_outputs;
  const int32_t *outputs;         /* [n_outputs] labels, output order           */
  const int32_t *plane;           /* [n_nodes] MBQC_PLANE_*, -1 = no measurement
                                     (exactly the outputs)                      */
  const int32_t *trainable;       /* [n_nodes] 1 = angle from the angle vector  */
  const double *angle;            /* [n_nodes] angle of the fixed measurements  */
  int32_t n_trainable;            /* length of trainable_order, or 0            */
  const int32_t *trainable_order; /* labels in angle-vector order, or NULL:
                                     graph order of the trainable nodes         */
  int32_t window_size;            /* 0 or 1: inputs + 1 (the simulators' default) */
  int32_t kind;                   /* 0 statevector, 1 density matrix            */
} mbqc_graph_desc;

/* Output of the native plan compiler: caller-owned arrays, each with room
 * for n_nodes entries (init_cz: 32); the scalars are filled in. */
typedef struct mbqc_plan_tables {
  int32_t window, n_steps, n_in, n_out, n_angles, n_nodes;
  int32_t *in_bits;
  uint32_t *init_cz;
  uint32_t *step_mask;
  int32_t *step_angle;
  int32_t *step_plane;
  double *step_fixed_angle;
  int32_t *out_bits;
  int32_t *out_nodes;             /* output labels in the returned order        */
  int32_t *schedule;              /* measurement order (all nodes, labels)      */
} mbqc_plan_tables;

/*
 * Native plan compiler (host only, no device call): causal-flow layers
 * (flow.py:115-188), measurement order (mbqcircuit.py:390-422) and the
 * window tables of the simulators' constructors (np_simulator_sv.py:61-128,
 * 207-223, 278-297; np_simulator_dm.py:47-115, 267-283).  Returns
 * MBQC_E_UNSUPPORTED for what it leaves to the Python compiler: graphs
 * without a causal flow, measured outputs, a flow search that depends on
 * Python's set iteration order (a candidate shared by two frontier nodes).
 */
int mbqc_compile_graph(const mbqc_graph_desc *graph, mbqc_plan_tables *tables);

/*
 * Many open graphs in flat arrays (graph i owns entries [off[i], off[i+1])
 * of each array; edges in pairs), every trainable angle in graph order.
 */
typedef struct mbqc_graph_batch {
  int32_t n_graphs;
  const int64_t *node_off;        /* [n_graphs + 1]                             */
  const int32_t *nodes;           /* labels in graph order                      */
  const int32_t *plane;           /* per node, as in mbqc_graph_desc            */
  const int32_t *trainable;       /* per node                                   */
  const double *angle;            /* per node                                   */
  const int64_t *edge_off;        /* [n_graphs + 1], in edges (pairs)           */
  const int32_t *edges;
  const int64_t *in_off;          /* [n_graphs + 1]                             */
  const int32_t *inputs;
  const int64_t *out_off;         /* [n_graphs + 1]                             */
  const int32_t *outputs;
  int32_t window_size;            /* as in mbqc_graph_desc                      */
  int32_t kind;                   /* 0 statevector, 1 density matrix            */
} mbqc_graph_batch;

/*
 * Compile a batch of open graphs natively and upload them as one plan table
 * (circuit i = graph i), for uneven batches of thousands of circuits.
 * info [n_graphs][5] (or NULL) receives window, n_steps, n_in, n_out,
 * n_angles per graph.  plan NULL: compile only (host, no device call).
 * Fails on the first graph that mbqc_compile_graph declines, naming it.
 */
int mbqc_plan_create_from_graphs(const mbqc_graph_batch *batch, mbqc_plan **plan, int32_t *info);

/*
 * A statevector batch bound once and launched many times (serving loops):
 * mbqc_sv_call_create takes the arguments of mbqc_sv_forward (f64 = 0) or
 * of mbqc_sv_forward_f64 (f64 = 1, variant ignored), checks them, builds the
 * kernel's parameter block and chooses the kernel and its launch geometry;
 * mbqc_sv_call_launch then makes only the launch, on ``stream``, reading the
 * buffers' current contents.  The plan and the bound buffers must outlive
 * the call (it keeps their addresses).  Launches only read the call, so one
 * call may be launched from several threads or streams; launches that
 * overlap write the same output buffers.  Register kernel windows only
 * (w <= 10; wider windows go through mbqc_sv_forward_stream).
 */
typedef struct mbqc_sv_call mbqc_sv_call;
int mbqc_sv_call_create(const mbqc_plan *plan, int64_t batch, const double *angles, int64_t angle_stride,
                        const void *psi_in, int64_t in_stride, void *psi_out, uint32_t flags, int32_t variant,
                        double *logprob, int32_t *status, int32_t f64, mbqc_sv_call **call);
int mbqc_sv_call_launch(const mbqc_sv_call *call, mbqc_stream_t stream);
void mbqc_sv_call_destroy(mbqc_sv_call *call);

/*
 * Flow byproduct tables for sampled outcomes (device memory): on outcome 1
 * of step k, an X acts on the node measured at step x_step[k] (or -1) and on
 * the output-index bits x_out[k]; a Z acts on the steps z_idx[z_off[k] ..
 * z_off[k+1]) (all later than k) and on the output-index bits z_out[k]
 * (output j is bit n_out-1-j).  x_step, x_out, z_out have one entry per
 * step, z_off n_steps + 1.  Built from the causal flow as in mentpy's
 * PennyLane backend (pennylane_simulator.py:144-153): X on flow(i), Z on the
 * neighbours of flow(i) measured after i.
 */
typedef struct mbqc_byproducts {
  const int32_t *x_step;
  const int32_t *z_off;
  const int32_t *z_idx;
  const uint32_t *x_out;
  const uint32_t *z_out;
} mbqc_byproducts;

/*
 * Statevector sweep with drawn outcomes (force0=False, the PennyLane
 * backend's semantics) for windows <= 20 and any number of steps whose Pauli
 * frame (2 bits a step) fits in shared memory (about 900,000): each outcome
 * is drawn from the branch weights with SplitMix64 of (seed, run, step); the
 * byproducts become a Pauli frame (a pending X flips the next measurement
 * angle's sign, a Z adds pi; the frame left on the outputs is applied to the
 * returned state).  psi_out [batch, 2^n_out] normalised, global phase
 * unspecified; outcomes [batch, outcome_stride] int8 or NULL.  Windows 15
 * to 20 keep the window in a caller workspace of the size
 * mbqc_sv_sampled_workspace reports (0 bytes for windows <= 14, where
 * workspace may be NULL).
 */
int mbqc_sv_sampled_workspace(const mbqc_plan *plan, int64_t batch, size_t *bytes);
int mbqc_sv_forward_sampled(const mbqc_plan *plan, int64_t batch, const double *angles,
                            int64_t angle_stride, const float *psi_in, int64_t in_stride,
                            float *psi_out, uint64_t seed, const mbqc_byproducts *byproducts,
                            int8_t *outcomes, int64_t outcome_stride, int32_t *status,
                            void *workspace, size_t workspace_bytes, mbqc_stream_t stream);

/* ABI version and the last error message of the calling thread. */
int mbqc_abi_version(void);
const char *mbqc_last_error(void);

/*
 * Upload ``n_circuits`` plans into one device-resident plan table.  Runs of
 * a batched density-matrix call pick their circuit by index (the
 * ``run_circuit`` argument of mbqc_dm_forward / mbqc_dm_adjoint); the
 * statevector entry points run circuit 0.
 * Replaces the per-simulator setup of PatternSimulator.__init__
 * (pattern_simulator.py:38-70).
 */
int mbqc_plan_create(const mbqc_circuit_desc *circuits, int32_t n_circuits,
                     mbqc_plan **plan);
int mbqc_plan_destroy(mbqc_plan *plan);

/*
 * Batched statevector sweep, complex64 amplitudes with FP64 norm reduction.
 * Replaces ``NumpySimulatorSV.reset(input_state); run(angles,
 * output_form="sv")`` (np_simulator_sv.py:227-297, 299-320) for ``batch``
 * independent runs of circuit 0 of ``plan``:
 *   angles   [batch, angle_stride] double (run b uses angles + b*angle_stride)
 *   psi_in   [batch or 1, 2^n_in] complex64 (in_stride 0 broadcasts row 0;
 *            need not be normalised)
 *   psi_out  [batch, 2^n_out] complex64, normalised, in the reference's output
 *            qubit order
 *   logprob  [batch] double or NULL: ln of the probability of the all-zero
 *            outcome branch, sum_k ln prob0_k
 *   status   [batch] int32 or NULL: MBQC_RUN_*
 *   variant  -1 = tuned default, else log2(lanes per run) of the register
 *            kernel (windows <= 10)
 * The kernel is launched as a programmatic dependent of the previous work on
 * ``stream`` (environment MBQC_PDL=0: a plain launch): before that work
 * completes it reads only the plan, unless ``flags`` holds
 * MBQC_F_INPUTS_READY, and it writes nothing.
 */
int mbqc_sv_forward(const mbqc_plan *plan, int64_t batch, const double *angles,
                    int64_t angle_stride, const float *psi_in, int64_t in_stride,
                    float *psi_out, uint32_t flags, int32_t variant,
                    double *logprob, int32_t *status, mbqc_stream_t stream);

/*
 * Wide windows (8..30; the register kernel covers <= 10): the same sweep with
 * each run's 2^w window streamed through ``workspace`` in passes of up to ten
 * fused steps (five for windows 8 and 9).  Same arguments and results as
 * mbqc_sv_forward plus the workspace, sized by mbqc_sv_stream_workspace
 * (batch * 2^w * 8 bytes plus per-run bookkeeping and epilogue partials).  The reference cannot run these windows: its dense
 * 2^w x 2^w operators (gates.py:62-72,127-143) need 256 GiB at w = 17.
 */
int mbqc_sv_stream_workspace(const mbqc_plan *plan, int64_t batch, size_t *bytes);
int mbqc_sv_forward_stream(const mbqc_plan *plan, int64_t batch, const double *angles,
                           int64_t angle_stride, const float *psi_in, int64_t in_stride,
                           float *psi_out, uint32_t flags, double *logprob, int32_t *status,
                           void *workspace, size_t workspace_bytes, mbqc_stream_t stream);

/* Same sweep in complex128 (FP64 check mode). */
int mbqc_sv_forward_f64(const mbqc_plan *plan, int64_t batch,
                        const double *angles, int64_t angle_stride,
                        const double *psi_in, int64_t in_stride,
                        double *psi_out, uint32_t flags, double *logprob,
                        int32_t *status, mbqc_stream_t stream);

/*
 * Batched density-matrix sweep, windows <= 8 (in shared memory: the full
 * rho for windows <= 7, or, for plans whose last step shrinks the window,
 * rho in factored form -- the (w-1)-qubit matrix of the bits other than the
 * last entering qubit's slot, whose |+> and CZs are applied implicitly).
 * Replaces ``NumpySimulatorDM.reset(input_state); run(angles)``
 * (np_simulator_dm.py:218-305) for ``batch`` runs.  All runs of one call
 * share the window size ``window``.  run_circuit NULL: ``batch`` runs of
 * circuit 0, per-run arrays indexed by run.  run_circuit given: ``batch``
 * entries, entry b simulates circuit c = run_circuit[b] of the plan table and
 * every per-run array below is indexed by c (one run per circuit: the uneven
 * batch of many different circuits, one call per window size).
 *   angles    [batch, angle_stride] double
 *   psi_in    [batch or 1, in_stride] complex64 pure input states (in_stride 0
 *             broadcasts row 0; unnormalised inputs are kept as the reference
 *             keeps them: the first outcome test sees |psi|^2)
 *   rho_out   [batch, out_stride] complex64: rho over the quantum outputs in
 *             the reference's order, 2^n_out x 2^n_out row-major
 *   noise     depolarising strength q in [0, 1]: every qubit passes once
 *             through the depolarising channel, just before it is measured
 *             (outputs: after the sweep) -- PennyLane's placement
 *             (pennylane_simulator.py:123-126) seen through the window; 0 =
 *             the reference numpy path
 *   outcomes  [batch, outcome_stride] int8 or NULL: outcome of every step, 1
 *             iff prob0 < 1e-4 (np_simulator_dm.py:335-338)
 *   probs     [batch, outcome_stride] double or NULL: prob0 of every step
 *   status    [batch] or NULL: MBQC_RUN_NAN where the reference raises
 *             ValueError (np_simulator_dm.py:179-182)
 */
int mbqc_dm_forward(const mbqc_plan *plan, int64_t batch, int32_t window,
                    const int32_t *run_circuit, const double *angles, int64_t angle_stride,
                    const float *psi_in, int64_t in_stride, float *rho_out, int64_t out_stride,
                    double noise, int8_t *outcomes, double *probs, int64_t outcome_stride,
                    int32_t *status, mbqc_stream_t stream);

/*
 * Uneven batch of density-matrix circuits in ONE persistent launch: circuit
 * c (c < n_circuits) of ``plan`` runs once per call, every per-run array
 * indexed by c, as mbqc_dm_forward with run_circuit = all circuits.  Replaces
 * one NumpySimulatorDM.run (np_simulator_dm.py:218-346) per circuit.
 * Windows 2..8 whose last step shrinks the window (the plan compiler's
 * schedules), density matrices in factored form (a (w-1)-qubit matrix in
 * shared memory per run).
 *
 * mbqc_dm_batch_create sorts the circuits into tiles (runs of one window
 * that one 256-thread block executes together, tile_tpr[w] threads per run;
 * tile_tpr NULL or 0 entries = defaults; valid shapes: w 2..4: 32, w 5: 32
 * or 64, w 6: 32, 64 or 128, w 7: 64, 128 or 256, w 8: 256), orders them
 * longest first and uploads the schedule (device memory owned by the batch).
 * blocks_per_sm 0 = as many as fit.  mbqc_dm_batch_forward launches one
 * kernel whose resident blocks claim tiles with an atomic counter until the
 * list is exhausted (no block waits on another; the launch resets the
 * counter for the next one, so it can be captured in a CUDA graph).  Calls
 * on one batch must not overlap on the GPU (they share the counter).
 * mbqc_dm_batch_info: info[0] tiles, [1] blocks, [2] shared memory per
 * block, [3 + w - 2] threads per run of window w (w = 2..8).
 * mbqc_dm_batch_create_ex: the circuits of window w with at least
 * long_steps[w] steps (0 = none) take the tile shape long_tpr[w] (0 = the
 * window's shape): the longest runs, which end the batch, with more threads.
 */
typedef struct mbqc_dm_batch mbqc_dm_batch;
int mbqc_dm_batch_create_ex(const mbqc_plan *plan, int32_t n_circuits, const int32_t *tile_tpr,
                            const int32_t *long_tpr, const int32_t *long_steps, int32_t blocks_per_sm,
                            mbqc_dm_batch **batch);
int mbqc_dm_batch_create(const mbqc_plan *plan, int32_t n_circuits, const int32_t *tile_tpr,
                         int32_t blocks_per_sm, mbqc_dm_batch **batch);
int mbqc_dm_batch_destroy(mbqc_dm_batch *batch);
int mbqc_dm_batch_info(const mbqc_dm_batch *batch, int32_t *info);
int mbqc_dm_batch_forward(const mbqc_dm_batch *batch, const double *angles, int64_t angle_stride,
                          const float *psi_in, int64_t in_stride, float *rho_out, int64_t out_stride,
                          double noise, int8_t *outcomes, double *probs, int64_t outcome_stride,
                          int32_t *status, uint32_t flags, uint64_t seed, mbqc_stream_t stream);

/*
 * mbqc_dm_forward with the measurement mode of NumpySimulatorDM.run:
 * flags MBQC_F_DM_EXPECTATION for mode="expectation" (0: "sample"), and the
 * seed of the counter-based draws (SplitMix64 of seed, run, step) of Z-basis
 * outcomes in sample mode.  For Z steps ``outcomes`` holds the drawn outcome,
 * or 2 in expectation mode with prob1/(prob0+prob1) in ``probs``.
 * mbqc_dm_forward is this call with flags 0 and seed 0.
 */
int mbqc_dm_forward_ex(const mbqc_plan *plan, int64_t batch, int32_t window,
                       const int32_t *run_circuit, const double *angles, int64_t angle_stride,
                       const float *psi_in, int64_t in_stride, float *rho_out, int64_t out_stride,
                       double noise, int8_t *outcomes, double *probs, int64_t outcome_stride,
                       int32_t *status, uint32_t flags, uint64_t seed, mbqc_stream_t stream);

/*
 * mbqc_dm_forward_ex for every window 1..11: windows 9..11 keep the factored
 * matrix (4^(w-1) complex64: 512 KB to 8 MB per run) in ``workspace``, one
 * 1024-thread block per resident run (mbqc_dm_forward_workspace gives the
 * bytes for ``batch`` runs; a smaller workspace runs fewer runs at a time,
 * the minimum is one run's matrix).  Windows <= 8 ignore the workspace.  The
 * reference runs these windows with dense 4^w x 4^w operators
 * (np_simulator_dm.py:33-346).
 */
int mbqc_dm_forward_workspace(const mbqc_plan *plan, int64_t batch, int32_t window, size_t *bytes);
int mbqc_dm_forward_ws(const mbqc_plan *plan, int64_t batch, int32_t window, const int32_t *run_circuit,
                       const double *angles, int64_t angle_stride, const float *psi_in, int64_t in_stride,
                       float *rho_out, int64_t out_stride, double noise, int8_t *outcomes, double *probs,
                       int64_t outcome_stride, int32_t *status, uint32_t flags, uint64_t seed, void *workspace,
                       size_t workspace_bytes, mbqc_stream_t stream);

/*
 * Reverse-mode gradient of the density-matrix sweep through the noisy channel
 * (windows <= 10: the matrix in shared memory to 7, in the workspace from 8);
 * no counterpart in the reference (whose gradients are finite
 * differences, gradients/_finite_difference.py:9-25).  Same run/row and noise
 * conventions as mbqc_dm_forward.  Given grad_out = dL/drho_out
 * ([row, gout_stride] complex64, dL = Re sum conj(grad_out) d rho_out,
 * outcomes held fixed), writes dL/dangles ([row, grad_stride] double) and,
 * when rho_out is not NULL, the forward output.  The workspace
 * (mbqc_dm_adjoint_workspace) holds the pre-step density matrices of the runs
 * in flight.
 */
int mbqc_dm_adjoint_workspace(const mbqc_plan *plan, int64_t batch, int32_t window,
                              const int32_t *run_circuit, size_t *bytes);
int mbqc_dm_adjoint(const mbqc_plan *plan, int64_t batch, int32_t window, const int32_t *run_circuit,
                    const double *angles, int64_t angle_stride, const float *psi_in, int64_t in_stride,
                    double noise, const float *grad_out, int64_t gout_stride, float *rho_out,
                    int64_t out_stride, double *grad_angles, int64_t grad_stride, int8_t *outcomes,
                    int64_t outcome_stride, int32_t *status, void *workspace, size_t workspace_bytes,
                    mbqc_stream_t stream);

/*
 * Reverse-mode gradient of the statevector sweep (windows <= 20: registers up
 * to 8, a block or a cluster of blocks per run above, and for plans with
 * XZ / YZ steps; the FP64 form to 8).  The reference has no autodiff; its
 * gradients are finite differences of whole simulations
 * (mentpy/gradients/_finite_difference.py:9-25, gradients/grad.py:13-33).
 * These entry points return the exact derivative of the sweep for the same
 * cost functions.
 *
 * Angle indices (all adjoint entry points, statevector and density matrix):
 * each angle is expected on at most one step, as in every plan built from an
 * MBQCircuit or a graph (one angle per measured node); the derivative of a
 * step is written to its angle's entry, not summed over steps sharing it.
 * An angle no step uses gets 0, except in mbqc_sv_adjoint at windows above
 * 8 or with XZ / YZ steps, which leaves its entry as the caller set it.
 *
 * mbqc_sv_adjoint_workspace: bytes of device workspace (period checkpoints of
 *   the runs in flight) the two calls below need for ``batch`` runs.
 * mbqc_sv_adjoint: given grad_out = dL/dz of the normalised outputs z of
 *   mbqc_sv_forward without MBQC_F_REF_PHASE ([batch, 2^n_out] complex64, the
 *   PyTorch convention dL = Re sum conj(grad_out) dz), writes dL/dangles
 *   ([batch, n_angles] double).  Recomputes the forward sweep itself.
 * mbqc_sv_fidelity_grad: for n_vectors angle vectors and n_inputs input
 *   states with targets t_j ([n_inputs, 2^n_out] complex64) computes
 *     loss[v] = 1 - (1/n_inputs) sum_j |<t_j | z(angles_v, psi_j)>|^2
 *   and grad[v, :] = dloss[v]/dangles_v (double, FP64 accumulation), all
 *   n_vectors * n_inputs runs in one launch: the cost function of
 *   docs/tutorials/intro-to-mbqml.rst:35-54 with its gradient.
 */
int mbqc_sv_adjoint_workspace(const mbqc_plan *plan, int64_t batch, int32_t f64, size_t *bytes);
int mbqc_sv_adjoint(const mbqc_plan *plan, int64_t batch, const double *angles,
                    int64_t angle_stride, const float *psi_in, int64_t in_stride,
                    const float *grad_out, double *grad_angles, int32_t *status,
                    void *workspace, size_t workspace_bytes, mbqc_stream_t stream);
int mbqc_sv_adjoint_f64(const mbqc_plan *plan, int64_t batch, const double *angles,
                        int64_t angle_stride, const double *psi_in, int64_t in_stride,
                        const double *grad_out, double *grad_angles, int32_t *status,
                        void *workspace, size_t workspace_bytes, mbqc_stream_t stream);
int mbqc_sv_fidelity_grad(const mbqc_plan *plan, int64_t n_vectors, const double *angles,
                          int64_t angle_stride, int64_t n_inputs, const float *psi_in,
                          const float *targets, double *loss, double *grad, int32_t *status,
                          void *workspace, size_t workspace_bytes, mbqc_stream_t stream);

/*
 * mbqc_sv_adjoint without a workspace argument, for callers that cannot
 * allocate device memory: plugins inside a host framework that owns the GPU
 * memory pool, fixed-footprint services that must not grow device memory
 * after start-up, and latency-bound loops that cannot afford the device-wide
 * synchronisation of cudaFree.  No counterpart in the reference.
 *
 * Same arguments and results as mbqc_sv_adjoint.  The period checkpoints live
 * in one fixed device array of MBQC_NOALLOC_SCRATCH_BYTES inside the library,
 * held on every GPU that loads the library until the process exits; the call
 * makes no allocation.  The first call on each device (and again after a
 * device reset re-creates its context) looks up that array's device address
 * (cudaGetSymbolAddress), so make the first call on a device before any
 * stream capture.  All calls share the array and it keeps the last call's
 * contents (nothing in it needs to start at zero: every checkpoint is written
 * before it is read); calls that overlap on the GPU, e.g. on two streams,
 * race on it and corrupt each other's results.  Windows above 8, and circuits
 * whose per-run step tables exceed shared memory, are rejected with
 * MBQC_E_UNSUPPORTED before anything is launched.  Shared memory is the
 * binding limit: any circuit that fits it needs at most ~2.9 MB of
 * checkpoints per warp of runs, so the array never rejects a circuit (a
 * defensive check remains); it only bounds the runs in flight, and large
 * batches run with fewer runs in flight.
 */
#define MBQC_NOALLOC_SCRATCH_BYTES (16u << 20)
int mbqc_sv_adjoint_noalloc(const mbqc_plan *plan, int64_t batch, const double *angles,
                            int64_t angle_stride, const float *psi_in, int64_t in_stride,
                            const float *grad_out, double *grad_angles, int32_t *status,
                            mbqc_stream_t stream);

/*
 * rho[b] = psi[b] psi[b]^dagger for ``batch`` complex64 vectors of
 * 2^n_qubits amplitudes: the default ``output_form="dm"`` of
 * NumpySimulatorSV.run (np_simulator_sv.py:292-293).
 */
int mbqc_outer(int64_t batch, int32_t n_qubits, const float *psi, float *rho,
               mbqc_stream_t stream);

/*
 * Measured FP32 FMA throughput of the current device (TFLOP/s, 2 flops per
 * FMA): the roofline denominator of the register-resident kernels, which run
 * on the FP32 pipe.  Synchronises ``stream``.  ``sink``: one device float.
 * No counterpart in the reference (measurement support).
 */
int mbqc_probe_fp32_fma(int64_t iters, float *sink, double *tflops, mbqc_stream_t stream);

/*
 * Measured shared-memory bandwidth of the current device (GB/s, loads plus
 * stores, 16-byte conflict-free accesses on every SM): the roofline
 * denominator of the density-matrix kernels, which stream their matrices
 * through shared memory.  Synchronises ``stream``.  No counterpart in the
 * reference (measurement support).
 */
int mbqc_probe_smem_bw(int64_t iters, float *sink, double *gbs, mbqc_stream_t stream);

/*
 * Adam step on n FP64 parameters, in place (x, m, v), from gradient g:
 * mentpy's AdamOptimizer.step (optimizers/adam.py:54-66).  The iteration
 * index and the bias corrections live in a device block state[3] =
 * {i, 1 - b1^(i+1), 1 - b2^(i+1)} that each step advances, so a captured CUDA
 * graph of (gradient, step) replays a whole training run.  Two launches on
 * ``stream``; state_init sets i = 0 (a host-to-device copy, outside capture).
 */
int mbqc_adam_state_init(double *state, double b1, double b2, mbqc_stream_t stream);
int mbqc_adam_step(int64_t n, double *x, const double *g, double *m, double *v, double *state,
                   double lr, double b1, double b2, double eps, mbqc_stream_t stream);

/* Device properties the host layer needs (SM count). */
int mbqc_device_sm_count(int32_t *sm_count);

/*
 * Device address of page-locked host memory (cudaHostAlloc / pinned
 * allocations, or cudaHostRegister'ed ranges) that the kernels may read and
 * write in place: on a Grace-Blackwell node the sweep then reads its angles
 * and inputs and writes its outputs over the coherent CPU-GPU link inside the
 * launch, with no staging copy.  Fails with MBQC_E_INVALID for pageable host
 * memory or device memory.  Every buffer argument of the sweep entry points
 * accepts such an address.  No counterpart in the reference (its buffers are
 * numpy arrays in host memory).
 */
int mbqc_mapped_pointer(const void *host, void **device_ptr);

#ifdef __cplusplus
}
#endif
#endif /* MBQC_GB300_H */
