/*
 * btoracle — CPU restatement of BlueTangle.jl's noisy-circuit semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA engine
 * (libbtgpu).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  The product path never calls it.
 *
 * Conventions (identical to the reference):
 *   - qubits are 1-based; qubit q is bit (n - q) of the 0-based amplitude index
 *     (src/bit.jl:9-14, src/hilbert.jl:154: foldl(kron, ...) puts qubit 1 first);
 *   - complex numbers are interleaved (re, im) doubles, as Julia's ComplexF64;
 *   - matrices are column-major (Julia layout): m[r + c*d] = M[r, c];
 *   - a density matrix rho[i, j] is stored column-major: rho[i + j*2^n];
 *   - control == -2 means "no control" (src/struct.jl:389).
 * Randomness is never drawn here: every random choice takes the caller's
 * uniform draw u in [0,1) or a forced outcome, so that results are reproducible.
 *
 * Return codes: 0 ok, -1 bad argument, -2 not supported by the reference
 * (the reference throws a String for the same input).
 */
#ifndef BTORACLE_H
#define BTORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* hilbert(N, U, q; control) * psi   (src/hilbert.jl:143-159) */
int bto_hilbert1(int n, double* psi, const double* m, int q, int control);
/* hilbert(N, U, q, t; control) * psi   (src/hilbert.jl:18-70, :73-103, :215-237) */
int bto_hilbert2(int n, double* psi, const double* m, int q, int t, int control);
/* hilbert3(N, U, first) * psi (src/hilbert.jl:106-128); acts on first, first+1, first+2 */
int bto_hilbert3(int n, double* psi, const double* m, int first);
/* generic dense k-qubit matrix; qubits[0] is the most significant bit of the
 * matrix index; all controls must read 1.  Used for fused blocks. */
int bto_apply_k(int n, double* psi, int k, const int* qubits, const double* m,
                int nctrl, const int* ctrls);

/* born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721): outcome 1..4 in the
 * order [P0 P0, P1 P0, P0 P1, P1 P1] on (q1, q2); probs[4] the weights */
int bto_born_measure_z2(int n, double* psi, int q1, int q2, double u, int forced, int* outcome, double* probs);
/* partial_trace(psi, q)      -> 2x2   (src/linalg.jl:167-192) */
int bto_partial_trace1(int n, const double* psi, int q, double* out);
/* partial_trace(psi, q, t)   -> 4x4 in (min, max) order (src/linalg.jl:198-230,
 * and :83-86 for the non-adjacent pair, which also orders kept qubits ascending) */
int bto_partial_trace2(int n, const double* psi, int q, int t, double* out);
/* partial_trace(psi, keep) for an ascending keep list (src/linalg.jl:83-140) */
int bto_partial_trace_k(int n, const double* psi, int k, const int* keep, double* out);

/* __calc_prob (src/struct.jl:9-29, :44-49): p_k = Re tr(K rho_A K^dagger);
 * k = 1, 2 or 3 qubits; for k = 2 the pair is (q, t); for k = 3 q is first. */
int bto_calc_prob(int n, const double* psi, int k, int q, int t, int nk,
                  const double* kraus, double* probs);
/* _weighted_sample (src/hilbert.jl:810-819): first i (0-based) with
 * u <= cumsum(p)[i]; -1 when none (the reference returns nothing). */
int bto_weighted_sample(int np, const double* p, double u);
/* __QuantumChannel_new_apply on a state (src/struct.jl:31-41, :51-55).
 * forced >= 0 skips the draw. */
int bto_channel_traj(int n, double* psi, int k, int q, int t, int nk, const double* kraus,
                     double u, int forced, int* branch, double* probs);
/* born_measure_Z(N, psi, q) (src/hilbert.jl:682-696); forced >= 0 skips the draw. */
int bto_born_measure_z(int n, double* psi, int q, double u, int forced, int* outcome, double* p0);

/* density matrix: rho <- E rho E^dagger with E = hilbert(...) (src/hilbert.jl:655-656) */
int bto_dm_gate(int n, double* rho, int k, const int* qubits, const double* m,
                int nctrl, const int* ctrls);
int bto_dm_hilbert1(int n, double* rho, const double* m, int q, int control);
int bto_dm_hilbert2(int n, double* rho, const double* m, int q, int t, int control);
/* rho <- sum_k E_k rho E_k^dagger (src/struct.jl:58-76) */
int bto_dm_channel(int n, double* rho, int k, int q, int t, int nk, const double* kraus);
/* born_measure_Z(N, rho, q) = sum_b P_b rho P_b (src/hilbert.jl:784-796) */
int bto_dm_dephase(int n, double* rho, int q);

/* observables (src/func.jl:91-147): Pauli string with bit masks over the amplitude
 * index (bit n-q for qubit q); Y sits in both masks. */
double bto_expect_pauli_sv(int n, const double* psi, uint64_t xmask, uint64_t zmask);
double bto_expect_pauli_dm(int n, const double* rho, uint64_t xmask, uint64_t zmask);
/* Re <psi| E |psi> for a k-qubit matrix (expect(state, op::QuantumOps)) */
double bto_expect_matrix_sv(int n, const double* psi, int k, const int* qubits,
                            const double* m, int nctrl, const int* ctrls);

/* sample (src/ops.jl:46-62): per shot t = u * sum(w), index = first i with
 * cumsum(w)[i] >= t (the direct search of StatsBase's weighted sample). */
int bto_sample(int n, const double* psi, int64_t shots, const double* u, int64_t* out);
/* |psi|^2 (sample_exact) */
void bto_probs(int n, const double* psi, double* out);

/* CPU baseline helper: applies a list of dense 1q/2q gates (generic form) with
 * OpenMP over the amplitude groups; returns the number of gates applied. */
int64_t bto_run_gates(int n, double* psi, int ngates, const int* ks, const int* qubits,
                      const double* mats, int nthreads);
int bto_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
