/*
 * btgpu.h — C ABI of the GB300 engine for BlueTangle.jl's noisy-circuit hot path.
 *
 * The reference has no FFI: its boundary is Julia multiple dispatch on the
 * state argument of apply / measure / sample / expect / correlation /
 * born_measure_Z (BlueTangle.jl src/BlueTangle.jl:5-22).  Each entry point
 * below replaces the reference function cited beside it; a Julia package adds
 * methods of those generics for GPU-resident states and `ccall`s these symbols.
 *
 * Conventions
 *   qubits      1-based, exactly as in the reference; qubit q of an n-qubit
 *               register is bit (n - q) of the 0-based amplitude index, so
 *               qubit 1 is the most significant bit (src/bit.jl:9-14).
 *   complex     interleaved (re, im) float64 pairs on the host (Julia ComplexF64).
 *   matrices    column-major on the host (Julia layout): m[r + c*d] = M[r, c],
 *               d = 2^k; the first listed qubit is the most significant bit of
 *               the matrix index (the |b_q b_t> order of src/hilbert.jl:30).
 *   density     rho[i, j] at i + j*2^n (column-major), as a Julia Matrix.
 *   member      states hold `batch` independent members (trajectories,
 *               twirl/ZNE copies, serving slots); member = -1 means all.
 *   errors      every call returns a status (BT_OK or a negative BT_ERR_*);
 *               bt_last_error() gives the message.  Nothing aborts.
 *   threading   one ctx = one CUDA stream; calls on a ctx are serialised by the
 *               caller.  Separate ctxs may be used from separate threads.
 * Host pointers are borrowed for the duration of the call only.
 */
#ifndef BTGPU_H
#define BTGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BT_ABI_VERSION 1

#define BT_OK 0
#define BT_ERR_BAD_ARG (-1)
#define BT_ERR_NOT_CPTP (-2)
#define BT_ERR_OOM (-3)
#define BT_ERR_DEVICE (-4)
#define BT_ERR_TIMEOUT (-5)
#define BT_ERR_UNSUPPORTED (-6)
#define BT_ERR_NO_BRANCH (-7)

#define BT_REPR_SV 0 /* state vector, 2^n amplitudes per member */
#define BT_REPR_DM 1 /* density matrix, 4^n entries per member */

#define BT_PREC_C128 0 /* complex float64 (the drop-in precision) */
#define BT_PREC_C64 1  /* complex float32 bulk; norms, cdf and branch probabilities stay float64 */

/* bt_apply_kraus modes */
#define BT_KRAUS_TRAJ 0 /* Monte-Carlo branch per member (state vector) */
#define BT_KRAUS_SUM 1  /* rho <- sum_k K rho K^dagger (density matrix) */
/* flag: branch probabilities from the reduced state of the pair in ascending
 * qubit order while the branch operator acts in (q, t) order, which is what
 * __calc_prob does for a pair with q > t (src/struct.jl:17-29 with
 * src/linalg.jl:198-230 and src/hilbert.jl:30). */
#define BT_KRAUS_REF_ORDER 0x100
/* flag: every K_i is a multiple of a unitary (depolarizing, bit/phase flips,
 * rot_xyz): the branch probabilities |c_i|^2 do not depend on the normalised
 * state, so no reduction pass is made (the reference's probabilities differ only
 * by the state's norm, 1 to rounding).  Rejected when the Kraus set is not of
 * that form. */
#define BT_KRAUS_UNITARY_MIX 0x200

typedef struct bt_ctx bt_ctx;
typedef struct bt_state bt_state;
typedef struct bt_plan bt_plan;

/* ------------------------------------------------------------------ context */
int bt_abi_version(void);
const char* bt_status_string(int status);
/* Creates a context on CUDA device `device` with its own stream; `seed` keys the
 * on-device counter-based RNG (Philox4x32-10) used when no uniforms are given. */
int bt_ctx_create(int device, uint64_t seed, bt_ctx** out);
int bt_ctx_destroy(bt_ctx* ctx);
const char* bt_last_error(const bt_ctx* ctx); /* NULL ctx: last error of this thread */
int bt_ctx_synchronize(bt_ctx* ctx);
/* number of engine kernels this ctx has launched (instrumentation) */
int bt_ctx_launch_count(const bt_ctx* ctx, int64_t* out);
/* the ctx's cudaStream_t, for interop (events, CUDA.jl/torch stream sharing) */
int bt_ctx_stream(const bt_ctx* ctx, void** out);

/* -------------------------------------------------------------------- state */
/* zero_state / the 2^N vector and 4^N matrix the reference allocates
 * (src/hilbert.jl:866, src/ops.jl:806-810).  n <= 34 (SV) / 17 (DM). */
int bt_state_alloc(bt_ctx* ctx, int n, int repr, int prec, int batch, bt_state** out);
int bt_state_free(bt_state* s);
int bt_state_info(const bt_state* s, int* n, int* repr, int* prec, int* batch);
/* device address of member 0 (interop, e.g. DLPack); members are contiguous */
void* bt_state_device_ptr(bt_state* s);
/* |0...0> or |0..0><0..0| (zero_state, src/hilbert.jl:866) */
int bt_state_set_zero(bt_state* s, int64_t member);
/* computational basis state |index> (product_state of bits, src/hilbert.jl:835) */
int bt_state_set_basis(bt_state* s, int64_t member, uint64_t index);
/* every entry of the member (-1: all members) set to 0: the empty accumulator of
 * rho_construct (src/ops.jl:603) and the start of superpositions of basis states */
int bt_state_clear(bt_state* s, int64_t member);
/* random_state(N) (src/hilbert.jl:882): normalize(rand(ComplexF64, 2^N)), real
 * and imaginary parts uniform in [0, 1) from on-device Philox keyed by (ctx seed,
 * seed, member); member = -1 fills every member (each its own draws). */
int bt_state_random(bt_state* s, int64_t member, uint64_t seed);
/* copies member `src_member` of src into member `dst_member` of dst (same n/repr/prec);
 * dst_member = -1 broadcasts it to every member of dst */
int bt_state_copy(bt_state* dst, int64_t dst_member, const bt_state* src, int64_t src_member);
/* host complex128 <-> device, `len` complex entries starting at entry `offset`
 * of one member; converted to/from complex64 for BT_PREC_C64 states */
int bt_state_upload(bt_state* s, int64_t member, int64_t offset, int64_t len, const double* host);
int bt_state_download(const bt_state* s, int64_t member, int64_t offset, int64_t len, double* host);

/* ------------------------------------------------------------------- gates */
/* op.expand(N)*state for a k-qubit matrix with optional controls (all must read 1):
 * hilbert(N,U,q;control) (src/hilbert.jl:143-159), hilbert(N,U,q,t;control)
 * (src/hilbert.jl:18-70, including non-adjacent pairs and CCZX :73-103),
 * hilbert3 (src/hilbert.jl:106-128) and fused k <= 6 blocks.
 * On a density matrix it is e_op*rho*e_op' (src/hilbert.jl:655-656). */
int bt_apply_matrix(bt_state* s, int k, const int32_t* qubits, const double* mat, int nctrl,
                    const int32_t* ctrls, int64_t member);
/* the same gate position with a different matrix per member, in one pass over the
 * batch (state vectors): per-trajectory twirl frames, ZNE repetitions (identity
 * for members without them), per-client angles.  mats holds batch column-major
 * 2^k x 2^k matrices back to back. */
int bt_apply_matrix_members(bt_state* s, int k, const int32_t* qubits, const double* mats, int nctrl,
                            const int32_t* ctrls);

/* Kraus channel on qubits (1 <= k <= 3; qubits[0] = q, qubits[1] = t).
 *  BT_KRAUS_TRAJ (state vector): __QuantumChannel_new_apply (src/struct.jl:31-41,
 *    :51-55): p_i = Re tr(K_i rho_A K_i^dagger) from the reduced state
 *    (__calc_prob, src/struct.jl:9-29), branch = first i with u <= cumsum(p)[i]
 *    (_weighted_sample, src/hilbert.jl:810-819), psi <- normalize(K_branch psi).
 *    uniforms[m] is member m's draw (NULL: on-device Philox); forced[m] >= 0
 *    skips the draw (NULL: none).  branch_out[m] and probs_out[m*nk + i]
 *    (either may be NULL) receive the branch and the probabilities.
 *  BT_KRAUS_SUM (density matrix): rho <- sum_i K_i rho K_i^dagger
 *    (src/struct.jl:58-76) in one pass over rho.
 * `kraus` holds nk column-major 2^k x 2^k matrices back to back.
 * forced[m] = -2 makes member m skip the channel (no draw, state untouched):
 * members of one batch can follow different op sequences (ZNE repetitions). */
int bt_apply_kraus(bt_state* s, int k, const int32_t* qubits, int nk, const double* kraus, int mode,
                   const double* uniforms, const int32_t* forced, int32_t* branch_out,
                   double* probs_out);

/* -------------------------------------------------------------- measurement */
/* born_measure_Z(N, psi, q) (src/hilbert.jl:682-696) for every member:
 * p0 = rho_q[1,1]; outcome = u < p0 ? 0 : 1 (or forced); the other half is set
 * to exactly zero and the kept half renormalised.  outcome/p0 per member (may be NULL).
 * On a density matrix: born_measure_Z(N, rho, q) = sum_b P_b rho P_b
 * (src/hilbert.jl:784-796); uniforms/forced/outcome are ignored and p0 is
 * still reported.  forced[m] = -2: member m is not measured (outcome -1). */
int bt_measure_z(bt_state* s, int qubit, const double* uniforms, const int32_t* forced,
                 int32_t* outcome, double* p0);
/* born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721) for every member of a
 * state vector: weights p = |psi' P psi| for P = [P0 P0, P1 P0, P0 P1, P1 P1] on
 * (q1, q2) in that order, outcome = first k (1..4, the reference's 1-based index)
 * with u <= cumsum(p)[k] (not renormalised, as _weighted_sample), or forced[m]
 * (1..4; -2 skips member m, outcome -1); the state keeps the chosen projection,
 * renormalised, and every other amplitude is set to exactly zero.  probs: 4 per
 * member (may be NULL).  BT_ERR_NO_BRANCH when u exceeds the total weight. */
int bt_measure_z2(bt_state* s, int q1, int q2, const double* uniforms, const int32_t* forced, int32_t* outcome,
                  double* probs);
/* partial_trace(psi, keep) for k <= 3 kept qubits, in the listed order
 * (src/linalg.jl:83-230); out is a column-major 2^k x 2^k complex matrix */
int bt_reduced_dm(const bt_state* s, int k, const int32_t* qubits, int64_t member, double* out);

/* ------------------------------------------------------------------- plans */
/* A plan is a circuit of dense gates compiled once and run many times: the
 * gate-fusion pass of the circuit compiler (the role of compile/get_layers,
 * src/ops.jl:278-329, :421-445).  Each fused pass applies every gate acting
 * inside a 13-bit (complex64) / 12-bit (complex128) tile in one HBM round trip;
 * the result equals applying the gates one by one (bt_apply_matrix).
 * Specialised complex128 passes on states of 2^16 entries or more compute in
 * float-float arithmetic on the FP32 pipe (48-bit significands: relative error
 * ~2^-48 per operation, results within 1e-12 of FP64; environment BTGPU_JIT_FF=0
 * keeps FP64).
 * ctx may be NULL: planning and kernel specialisation need no GPU. */
int bt_plan_create(bt_ctx* ctx, int n, int repr, int prec, bt_plan** out);
int bt_plan_free(bt_plan* p);
/* appends op.expand(N) (state) or e_op*rho*e_op' (density), as bt_apply_matrix */
int bt_plan_add_matrix(bt_plan* p, int k, const int32_t* qubits, const double* mat, int nctrl,
                       const int32_t* ctrls);
/* appends rho <- sum_i K_i rho K_i^dagger (density plans, k <= 2; src/struct.jl:58-76) */
int bt_plan_add_kraus_sum(bt_plan* p, int k, const int32_t* qubits, int nk, const double* kraus);
/* mode 0: fused passes, kernels specialised before returning;
 * mode 1: one sweep per gate (the unfused reference form);
 * mode 2: fused passes that run on the generic kernel at once while their
 *         specialised kernels compile on a background thread (tiered);
 * mode 3: (complex64 state vectors) fused passes whose register phases each run
 *         as one dense 32 x 32 block on the tensor cores (tcgen05.mma kind::tf32,
 *         three TF32 products accumulated in FP32); passes of tiles smaller than
 *         2^13 amplitudes run as in mode 0.  The blocks are rebuilt at the next
 *         run after bt_plan_set_matrices. */
int bt_plan_compile(bt_plan* p, int mode);
/* new matrices for gates already in the plan (variational parameters: the
 * reference's type "f" ops evaluated at new pars, src/struct.jl:518-528):
 * add_index[i] counts bt_plan_add_* calls from 0, mats holds the matrices back to
 * back in the size each gate was added with.  The compiled passes are rewritten
 * in place; a gate whose structure changes (e.g. an angle making it diagonal)
 * makes the next run recompile.  Kraus sums cannot be updated. */
int bt_plan_set_matrices(bt_plan* p, int count, const int64_t* add_index, const double* mats);
/* marks the gates of these adds as variable (parameters updated in place): they
 * are compiled in forms whose structure does not depend on their entries, so
 * bt_plan_set_matrices never recompiles for them.  A gate becomes variable at its
 * first bt_plan_set_matrices anyway (one recompile); marking before
 * bt_plan_compile avoids that one too. */
int bt_plan_set_variable(bt_plan* p, int count, const int64_t* add_index);
/* njit: fused passes running as kernels specialised for the plan (NVRTC, compiled
 * by bt_plan_compile); the others run on the generic fused kernel */
/* algorithmic cost of one run per amplitude of a member: real flops of the
 * compiled passes' arithmetic (an FMA counts two) and HBM bytes moved (one read
 * and one write of the state per pass) */
int bt_plan_cost(const bt_plan* p, double* flops_per_amp, double* bytes_per_amp);
/* introspection of compiled pass `pass` (0 .. npasses-1), for checking plans on
 * the host.  kind 0 (fused): nops ops in application order, ops[6i..6i+5] =
 * {type, global bit of b0, global bit of b1, flags, unit, offset of its entries in
 * mats}, type and entries as the specialised code applies them (FOP_* in
 * csrc/bt_fused.cuh), mats = the pass's entries (cap_reals >= 4096).  kind 1
 * (sweep): one gate, ops[0..7] = {k, bits[0..4] (-1 past k), control mask low /
 * high 32 bits} (cap_ops >= 2), mats = its row-major interleaved 2^k x 2^k matrix. */
int bt_plan_pass_ops(const bt_plan* p, int64_t pass, int* kind, int* nops, int32_t* ops, double* mats, int cap_ops,
                     int cap_reals);
int bt_plan_stats(const bt_plan* p, int64_t* ngates, int64_t* npasses, int64_t* nfused, int64_t* nphases,
                  int64_t* njit);
/* tuning of the fused passes (applies at the next bt_plan_compile; 0 / -1 keep
 * the library default): gates per pass at most (1..192), register bits per
 * thread of complex64 passes specialised before the first run (4 or 5), and
 * two-lane FP32 arithmetic in specialised complex64 passes (0 or 1), and tile
 * bits per pass (10..13 complex64 / 9..12 complex128; a smaller tile spreads a
 * small state over more CTAs) */
int bt_plan_set_tuning(bt_plan* p, int max_ops, int tile_rb, int packed, int tile_bits);
/* Runs the plan on every member of s, member m with its own matrices for the
 * gates of these adds (mats: s's batch blocks, each the matrices of add_index
 * back to back as bt_plan_set_matrices reads them): one launch per pass for the
 * whole batch, the passes that hold those gates reading per-member entries from
 * a device table (parameter-shift evaluations, served requests of one circuit).
 * The gates become variable (one recompile if they were not); they must lie in
 * fused passes (one or two qubits, at most one folded control), and the
 * specialised kernels are needed (NVRTC).  The plan's own matrices stay as they
 * were. */
int bt_plan_run_members(bt_plan* p, bt_state* s, int count, const int64_t* add_index, const double* mats);
/* host-side parts of bt_plan_run_members, for inspection: building the per-member
 * kernels (written to BTGPU_JIT_DUMP when set), and the table of fused pass `pass`
 * (row m: member m's entries, *used reals per row; out, of cap reals, may be NULL) */
int bt_plan_prepare_members(bt_plan* p, int count, const int64_t* add_index);
int bt_plan_member_table(bt_plan* p, int64_t pass, int64_t members, int count, const int64_t* add_index,
                         const double* mats, double* out, int64_t cap, int* used);
/* runs the plan on member `member` (-1: every member) of a state of the same n/repr/prec */
int bt_plan_run(bt_plan* p, bt_state* s, int64_t member);

/* ---------------------------------------------------------------- programs */
/* A program is a noisy circuit run on every member of a batched state (state
 * vectors, 2 <= n <= 34): the per-shot loop of the noisy measure(circuit, shots)
 * (src/ops.jl:617-630) for a whole batch of shots at once.  Two executors:
 *   shared memory (members of n <= 14 qubits complex64 / 13 complex128): one CTA
 *     per member runs every op of the program in one launch;
 *   grouped (any n): consecutive ops inside at most two qubits form a group; per
 *     group one reduction of the members' reduced matrices on those qubits, one
 *     decision per member for every branch and outcome of the group (the reduced
 *     matrix transforms exactly under ops on its qubits), one pass applying the
 *     product of the chosen matrices; members with nothing to do in a group are
 *     not touched.
 * Both make the same decisions from the same draws (up to rounding at a branch
 * boundary).  Ops act on 1 or 2 qubits:
 *   gate     op.expand(N)*state; mats is one column-major matrix, or batch of them
 *            back to back when per_member (twirl frames, per-client angles);
 *   channel  apply_kraus (src/struct.jl:58-76, branch rule src/hilbert.jl:810-819)
 *            with flags BT_KRAUS_REF_ORDER / BT_KRAUS_UNITARY_MIX as in bt_apply_kraus;
 *   measure  _born_measure (src/hilbert.jl:682-703): outcome u < p0 ? 0 : 1, the
 *            other half set to zero, the kept half renormalised; the outcome goes to
 *            the next record slot.
 * skip (batch flags, or NULL) makes members pass over a channel or measurement
 * (their record slot reads -1).  Draw i of member m is uniforms[i*batch + m] when
 * uniforms is given to bt_program_run, else on-device Philox keyed by the ctx seed
 * and `seed` (the same pair gives the same draws).  A branch or outcome of zero
 * probability leaves that member as it
 * was at that op (record -1) and the run reports BT_ERR_NO_BRANCH / BT_ERR_BAD_ARG
 * after every member has finished. */
typedef struct bt_program bt_program;
int bt_program_create(bt_ctx* ctx, int n, int prec, int batch, bt_program** out);
int bt_program_free(bt_program* p);
int bt_program_add_gate(bt_program* p, int k, const int32_t* qubits, const double* mats, int per_member);
int bt_program_add_channel(bt_program* p, int k, const int32_t* qubits, int nk, const double* kraus, int flags,
                           const int32_t* skip);
int bt_program_add_measure(bt_program* p, int qubit, const int32_t* skip);
/* ops added after this call act on members [lo, hi) only (hi = -1: to the end of
 * the batch); the others pass over them (a gate leaves them as they are, a
 * measurement records -1), and a per_member gate takes hi - lo matrices.  Groups
 * of members running different circuits (trajectories beside twirled ZNE copies,
 * src/ops.jl:555-573) share one program this way; the grouped executor reads and
 * writes a member only in groups where it does something. */
int bt_program_set_range(bt_program* p, int64_t lo, int64_t hi);
int bt_program_info(const bt_program* p, int64_t* nops, int64_t* ndraws, int64_t* nrecords);
/* new matrices for gate op `op_index` (counting every bt_program_add_* call from
 * 0), in the count it was added with (variational angles between runs) */
int bt_program_set_gate(bt_program* p, int64_t op_index, const double* mats);
/* 0: shared memory when the member fits, else grouped (default); 1: shared
 * memory; 2: grouped */
int bt_program_set_executor(bt_program* p, int executor);
/* moves the program's tables to the device of ctx now (the first bt_program_run
 * otherwise does it): callers that compile programs ahead of a timed or
 * latency-critical loop prepare them there too */
int bt_program_prepare(bt_program* p, bt_ctx* ctx);
/* runs on every member of s (n, prec and batch as created); records: batch x
 * nrecords int32, member-major (may be NULL) */
int bt_program_run(bt_program* p, bt_state* s, const double* uniforms, uint64_t seed, int32_t* records);

/* ----------------------------------------------------------------- shadows */
/* rho = (1/nsnap) sum_m (x)_q T[codes[m*n + q]] into a density matrix of n <= 14
 * qubits (shadow, src/ops.jl:145-185): codes[m*n + q] = 2*basis + outcome of qubit
 * q+1 in snapshot m, tables holds the 6 single-qubit factors 3 U^dagger|b><b|U - I
 * as row-major interleaved complex 2x2 matrices (48 doubles) */
int bt_shadow_accumulate(bt_state* rho, int64_t nsnap, const uint8_t* codes, const double* tables);

/* ----------------------------------------------------------------- serving */
/* No counterpart in the reference: its VQE / Trotter loops (variational_apply +
 * expect(state, H), src/vqa.jl:420-456, src/func.jl:100) run one call at a time.
 * A server owns `lanes` contexts (CUDA streams) with one host thread each and
 * serves clients: a client is a compiled plan (state vector or density matrix)
 * or a program (a trajectory batch) plus a Pauli sum H; a request gives new
 * matrices for some of its gates and returns <H> (per member divided by the
 * member's norm, averaged over members).  Client states stay resident between
 * requests; clients are admitted by HBM footprint (state bytes) within
 * hbm_budget (0: 200 GiB), evicting idle residents least-recently-used first.
 * A client's requests run in submission order, one at a time; requests of
 * different clients run concurrently on free lanes.  Plans and programs are
 * borrowed: keep them alive until the server is destroyed and do not use them
 * elsewhere meanwhile. */
typedef struct bt_server bt_server;
int bt_serve_create(int device, int lanes, uint64_t seed, uint64_t hbm_budget, bt_server** out);
int bt_serve_destroy(bt_server* s);
int bt_serve_add_plan_client(bt_server* s, bt_plan* plan, int nterms, const uint64_t* xmask, const uint64_t* zmask,
                             const double* coef, int64_t* client);
int bt_serve_add_program_client(bt_server* s, bt_program* prog, int nterms, const uint64_t* xmask,
                                const uint64_t* zmask, const double* coef, int64_t* client);
/* index: plan add indices (as bt_plan_set_matrices) or program op indices (as
 * bt_program_set_gate); mats back to back, column-major, each in its gate's size;
 * seed keys the program's on-device draws */
/* a packed client: a program whose `batch` members are independent requests of
 * one circuit (its parameterised gates added with per-member matrices).  Up to
 * `batch` queued requests that name the same gates run as one launch, request m
 * in member m; each request's value is <H> / norm of its member.  Requests may
 * only name gates with per-member matrices. */
int bt_serve_add_packed_client(bt_server* s, bt_program* prog, int nterms, const uint64_t* xmask,
                               const uint64_t* zmask, const double* coef, int64_t* client);
int bt_serve_submit(bt_server* s, int64_t client, int count, const int64_t* index, const double* mats, uint64_t seed,
                    int64_t* ticket);
/* waits up to wait_ms (-1: until done, 0: no wait); BT_ERR_TIMEOUT while pending.
 * latency_s runs from submit to done, service_s from the lane's start to done
 * (either may be NULL).  A finished ticket is released by the call that reports it. */
int bt_serve_poll(bt_server* s, int64_t ticket, int64_t wait_ms, double* value, double* latency_s,
                  double* service_s);
/* completed requests, latency percentiles (over the most recent 65536 requests),
 * resident clients, HBM in use, and runs: launches of requests (a packed run
 * serves several requests) */
int bt_serve_stats(bt_server* s, int64_t* completed, double* p50_s, double* p99_s, int64_t* resident,
                   uint64_t* hbm_used, int64_t* runs);

/* dense TF32 throughput of the tensor cores (tcgen05.mma kind::tf32, M=128,
 * N=256, K=8, one CTA per SM issuing `iters` x 4 MMAs): a diagnostic for the
 * roofline of tensor-core plans (no counterpart in the reference) */
int bt_tc_tf32_peak(bt_ctx* ctx, int iters, double* tflops);

/* ---------------------------------------------------------------- sampling */
/* one shot from every member: out[m] drawn from member m's |psi|^2 (or diag rho)
 * as bt_sample draws, with uniforms[m] or on-device Philox keyed by (ctx seed,
 * seed).  The noisy branch of measure(circuit, shots) (src/ops.jl:617-630)
 * samples one shot from each re-simulated state: members are those states. */
int bt_sample_members(const bt_state* s, const double* uniforms, uint64_t seed, int64_t* out);
/* sample(psi, shots) (src/ops.jl:46-62): per shot t = u*sum|psi|^2, outcome =
 * first index with cumsum >= t.  uniforms (shots values) or NULL for on-device
 * Philox keyed by (ctx seed, seed).  On a density matrix samples diag(rho). */
int bt_sample(const bt_state* s, int64_t member, int64_t shots, const double* uniforms, uint64_t seed,
              int64_t* out);
/* abs2.(psi) or real(diag(rho)) (sample_exact, src/ops.jl:98-101, :129-132) */
int bt_probabilities(const bt_state* s, int64_t member, double* out);
/* No counterpart in the reference.  bt_sample for callers that must not allocate
 * device memory: callers whose device memory is owned by a host framework's pool
 * (CUDA.jl, PyTorch) that may hold nearly all of HBM, so a library cudaMalloc
 * could fail and a cudaFree would stall every stream, and callers recording
 * into CUDA graphs, where cudaMalloc/cudaFree are not captured.  It allocates
 * nothing: its only scratch (the chunk prefix) is a 512 KiB file-scope device
 * array, so it accepts state vectors of 1 <= n <= 28 qubits and rejects larger
 * ones.  Everything else is the caller's: d_state (2^n interleaved complex128 or
 * complex64 amplitudes in device memory), d_uniforms (shots draws in device
 * memory, or NULL for Philox keyed by `key` and `seed`; key = the ctx seed and
 * the same seed reproduce bt_sample's stream), d_out (shots int64 in device
 * memory) and the cudaStream_t `stream` (NULL = the legacy default stream).
 * The call only enqueues work and returns.  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept for the
 * life of the process: after cudaDeviceReset of a device (or anything else that
 * destroys its primary context) do not call this entry point on that device
 * again.  Each device holds its own copy of the array; calls on one device share
 * it, so calls that overlap on the same GPU race on it (calls on different
 * devices do not). */
int bt_sample_noalloc(const void* d_state, int n, int prec, int64_t shots, const double* d_uniforms, uint64_t key,
                      uint64_t seed, int64_t* d_out, void* stream);

/* ------------------------------------------------------------- observables */
/* Pauli strings as masks over the amplitude index (bit n-q for qubit q); Y sets
 * both masks.  out[t] = coef[t] * Re <P_t> (coef may be NULL = 1):
 *   state:   real(state'*expand_multi_op(...)*state) (src/func.jl:97, :139-142)
 *   density: real(tr(rho*M)) (src/func.jl:98, :144-147)
 * member = -1 writes batch*nterms values (member-major). */
int bt_expect_pauli(const bt_state* s, int nterms, const uint64_t* xmask, const uint64_t* zmask,
                    const double* coef, int64_t member, double* out);
/* <Z_q> for every qubit q = 1..n (expect(state, "Z"), src/func.jl:97-98) in one pass */
int bt_expect_z_all(const bt_state* s, int64_t member, double* out);
/* real(state' * op.expand(N) * state) for a k <= 2 qubit matrix (src/func.jl:91) */
int bt_expect_matrix(const bt_state* s, int k, const int32_t* qubits, const double* mat, int nctrl,
                     const int32_t* ctrls, int64_t member, double* out);
/* sum |psi|^2 (or tr rho) per member */
int bt_norm2(const bt_state* s, int64_t member, double* out);
/* fidelity(rho, sigma) = real(tr(sqrt(sqrt(rho) sigma sqrt(rho)))^2) for two
 * density matrices (src/tensor.jl:222-229), n <= 14: on the device from Hermitian
 * eigendecompositions (cuSOLVER zheevd and cuBLAS zgemm, loaded with dlopen on
 * first use): (sum_i sqrt(max(mu_i, 0)))^2 over the eigenvalues of
 * D V' sigma V D, rho = V diag(w) V', D = diag(sqrt(max(w, 0))). */
int bt_fidelity_dm(const bt_state* rho, int64_t rmember, const bt_state* sigma, int64_t smember, double* out);
/* rho[:, :] += weight * sum_m |psi_m><psi_m| over every member of the state vector
 * psi (same n; n <= 14): measure's density_matrix accumulation
 * (rho_construct += state*state'/shots, src/ops.jl:612, :626). */
int bt_rho_accumulate(bt_state* rho, int64_t rmember, const bt_state* psi, double weight);
/* fidelity(psi, phi) = |<psi|phi>|^2 (src/tensor.jl:219) */
int bt_fidelity(const bt_state* a, int64_t amember, const bt_state* b, int64_t bmember, double* out);

#ifdef __cplusplus
}
#endif
#endif
