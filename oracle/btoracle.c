/*
 * btoracle.c — dense CPU restatement of BlueTangle.jl's noisy-circuit hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for libbtgpu; see btoracle.h).
 *
 * The reference builds every operator as a full 2^N x 2^N SparseMatrixCSC by
 * kron and multiplies (src/hilbert.jl:143-159, :18-70).  This file restates the
 * same linear maps by index arithmetic on dense arrays; each function cites the
 * reference lines whose result it reproduces.
 */
#include "btoracle.h"
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

static inline cplx C(const double* p, int64_t i) { return p[2 * i] + I * p[2 * i + 1]; }
static inline void S(double* p, int64_t i, cplx v) { p[2 * i] = creal(v); p[2 * i + 1] = cimag(v); }
/* column-major matrix element M[r, c] of a d x d complex matrix */
static inline cplx M(const double* m, int d, int r, int c) { return C(m, (int64_t)r + (int64_t)c * d); }

static inline int bitpos(int n, int q) { return n - q; } /* qubit q -> bit n-q (src/bit.jl:9-14) */

/* insert a zero bit at each sorted position in pos[0..k-1] (ascending) */
static inline uint64_t insert_zeros(uint64_t g, int k, const int* pos_sorted) {
    for (int i = 0; i < k; ++i) {
        int p = pos_sorted[i];
        uint64_t lo = g & ((1ULL << p) - 1);
        g = ((g >> p) << (p + 1)) | lo;
    }
    return g;
}

/* Core: psi[stride*idx] for a vector of 2^nb entries, apply k-qubit matrix m on
 * bit positions bits[0..k-1] (bits[0] = MSB of the matrix index), controls on
 * bit positions cbits (all must be 1).  conj_m applies conj(M). */
static int apply_bits(int nb, double* psi, int64_t stride, int k, const int* bits, const double* m,
                      int nc, const int* cbits, int conj_m, int par) {
    if (k < 1 || k > 10 || nb < k) return -1;
    int d = 1 << k;
    int sorted[16];
    for (int i = 0; i < k; ++i) sorted[i] = bits[i];
    for (int i = 0; i < k; ++i)
        for (int j = i + 1; j < k; ++j)
            if (sorted[j] < sorted[i]) { int t = sorted[i]; sorted[i] = sorted[j]; sorted[j] = t; }
    for (int i = 0; i + 1 < k; ++i) if (sorted[i] == sorted[i + 1]) return -1;
    uint64_t cmask = 0;
    for (int i = 0; i < nc; ++i) cmask |= 1ULL << cbits[i];
    int64_t offs[1024];
    for (int j = 0; j < d; ++j) {
        int64_t o = 0;
        for (int b = 0; b < k; ++b)
            if ((j >> (k - 1 - b)) & 1) o |= 1LL << bits[b];
        offs[j] = o;
    }
    cplx* mm = (cplx*)malloc(sizeof(cplx) * d * d);
    for (int r = 0; r < d; ++r)
        for (int c = 0; c < d; ++c) {
            cplx v = M(m, d, r, c);
            mm[r * d + c] = conj_m ? conj(v) : v;
        }
    int64_t ng = 1LL << (nb - k);
#pragma omp parallel for schedule(static) if (par && ng > 4096)
    for (int64_t g = 0; g < ng; ++g) {
        uint64_t base = insert_zeros((uint64_t)g, k, sorted);
        if ((base & cmask) != cmask) continue;
        cplx a[1024], o[1024];
        for (int j = 0; j < d; ++j) a[j] = C(psi, (int64_t)(base + offs[j]) * stride);
        for (int r = 0; r < d; ++r) {
            cplx s = 0;
            for (int c = 0; c < d; ++c) s += mm[r * d + c] * a[c];
            o[r] = s;
        }
        for (int j = 0; j < d; ++j) S(psi, (int64_t)(base + offs[j]) * stride, o[j]);
    }
    free(mm);
    return 0;
}

int bto_apply_k(int n, double* psi, int k, const int* qubits, const double* m, int nctrl,
                const int* ctrls) {
    int bits[16], cb[64];
    if (k > 10 || nctrl > 64) return -1;
    for (int i = 0; i < k; ++i) {
        if (qubits[i] < 1 || qubits[i] > n) return -1;
        bits[i] = bitpos(n, qubits[i]);
    }
    for (int i = 0; i < nctrl; ++i) {
        if (ctrls[i] < 1 || ctrls[i] > n) return -1;
        for (int j = 0; j < k; ++j) if (ctrls[i] == qubits[j]) return -1;
        cb[i] = bitpos(n, ctrls[i]);
    }
    return apply_bits(n, psi, 1, k, bits, m, nctrl, cb, 0, 1);
}

/* hilbert(N, U, q; control): foldl(kron) of I's with U at q, plus
 * P1(c) (x) U(q) + P0(c) (x) I when controlled (src/hilbert.jl:143-159). */
int bto_hilbert1(int n, double* psi, const double* m, int q, int control) {
    if (q > n || control > n) return -1; /* "N must be larger than qubit" */
    if (control == -2) return bto_apply_k(n, psi, 1, &q, m, 0, NULL);
    return bto_apply_k(n, psi, 1, &q, m, 1, &control);
}

/* _swap_control_target: M[p(i), p(j)] with p = [1,3,2,4] unless M commutes
 * with SWAP (src/hilbert.jl:191-237) */
static void swap_ct(const double* m, double* out) {
    static const int p[4] = {0, 2, 1, 3};
    /* invariance test: M*SWAP - SWAP*M == 0 exactly */
    int inv = 1;
    for (int r = 0; r < 4 && inv; ++r)
        for (int c = 0; c < 4; ++c) {
            cplx ms = M(m, 4, r, p[c]);      /* (M*SWAP)[r,c] = M[r, p(c)] */
            cplx sm = M(m, 4, p[r], c);      /* (SWAP*M)[r,c] = M[p(r), c] */
            if (ms - sm != 0) { inv = 0; break; }
        }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            cplx v = inv ? M(m, 4, r, c) : M(m, 4, p[r], p[c]);
            out[2 * (r + 4 * c)] = creal(v);
            out[2 * (r + 4 * c) + 1] = cimag(v);
        }
}

static int mat_equal_real(const double* m, const double* ref_real, int d) {
    for (int i = 0; i < d * d; ++i)
        if (m[2 * i] != ref_real[i] || m[2 * i + 1] != 0.0) return 0;
    return 1;
}

/* hilbert(N, U, q, t; control) (src/hilbert.jl:18-70): the matrix acts in the
 * basis |b_q b_t> with q as the most significant bit; when q > t it is first
 * permuted by _swap_control_target and then placed on (t, q) = (min, max).
 * Non-adjacent pairs go through a Pauli reconstruction that is the same linear
 * map; controlled non-adjacent pairs exist only for CX/CZ (CCZX, :73-103). */
int bto_hilbert2(int n, double* psi, const double* m, int q, int t, int control) {
    if (n < q || n < t || n < control) return -1;
    if (q == t) return -1;
    int dist = abs(q - t);
    if (control != -2 && dist != 1) {
        /* column-major real CX and CZ (src/gates.jl:42, :45) */
        static const double CX[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0};
        static const double CZ[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, -1};
        if (!mat_equal_real(m, CX, 4) && !mat_equal_real(m, CZ, 4)) return -2;
    }
    double fm[32];
    if (q > t) swap_ct(m, fm); else memcpy(fm, m, sizeof(fm));
    int lo = q < t ? q : t, hi = q < t ? t : q;
    int qs[2] = {lo, hi};
    if (control == -2) return bto_apply_k(n, psi, 2, qs, fm, 0, NULL);
    return bto_apply_k(n, psi, 2, qs, fm, 1, &control);
}

/* hilbert3: the 8x8 matrix on (first, first+1, first+2) (src/hilbert.jl:106-128) */
int bto_hilbert3(int n, double* psi, const double* m, int first) {
    if (n < first + 2) return -1;
    int qs[3] = {first, first + 1, first + 2};
    return bto_apply_k(n, psi, 3, qs, m, 0, NULL);
}

/* partial trace over all qubits except the ascending list keep[0..k-1];
 * the kept index is read MSB-first in keep order (src/linalg.jl:83-140). */
int bto_partial_trace_k(int n, const double* psi, int k, const int* keep, double* out) {
    if (k < 1 || k > 10) return -1;
    int d = 1 << k;
    int bits[16], sorted[16];
    for (int i = 0; i < k; ++i) {
        if (keep[i] < 1 || keep[i] > n) return -1;
        if (i && keep[i] <= keep[i - 1]) return -1;
        bits[i] = bitpos(n, keep[i]);
        sorted[k - 1 - i] = bits[i]; /* ascending bit positions */
    }
    int64_t offs[1024];
    for (int j = 0; j < d; ++j) {
        int64_t o = 0;
        for (int b = 0; b < k; ++b)
            if ((j >> (k - 1 - b)) & 1) o |= 1LL << bits[b];
        offs[j] = o;
    }
    cplx* acc = (cplx*)calloc((size_t)d * d, sizeof(cplx));
    int64_t ng = 1LL << (n - k);
    for (int64_t g = 0; g < ng; ++g) {
        uint64_t base = insert_zeros((uint64_t)g, k, sorted);
        for (int a = 0; a < d; ++a) {
            cplx va = C(psi, base + offs[a]);
            for (int b = 0; b < d; ++b) acc[a + b * d] += va * conj(C(psi, base + offs[b]));
        }
    }
    for (int i = 0; i < d * d; ++i) { out[2 * i] = creal(acc[i]); out[2 * i + 1] = cimag(acc[i]); }
    free(acc);
    return 0;
}

int bto_partial_trace1(int n, const double* psi, int q, double* out) {
    return bto_partial_trace_k(n, psi, 1, &q, out);
}

int bto_partial_trace2(int n, const double* psi, int q, int t, double* out) {
    if (q == t) return -1;
    int keep[2] = {q < t ? q : t, q < t ? t : q};
    return bto_partial_trace_k(n, psi, 2, keep, out);
}

/* p_k = Re tr(K rho K^dagger) for a d x d rho (column-major) */
static double tr_krk(int d, const double* K, const double* rho) {
    double s = 0;
    for (int i = 0; i < d; ++i)
        for (int a = 0; a < d; ++a)
            for (int b = 0; b < d; ++b)
                s += creal(M(K, d, i, a) * M(rho, d, a, b) * conj(M(K, d, i, b)));
    return s;
}

int bto_calc_prob(int n, const double* psi, int k, int q, int t, int nk, const double* kraus,
                  double* probs) {
    double rho[2 * 64];
    int d = 1 << k;
    int rc;
    if (k == 1) rc = bto_partial_trace1(n, psi, q, rho);
    else if (k == 2) rc = bto_partial_trace2(n, psi, q, t, rho);
    else if (k == 3) { int keep[3] = {q, q + 1, q + 2}; rc = bto_partial_trace_k(n, psi, 3, keep, rho); }
    else return -1;
    if (rc) return rc;
    for (int i = 0; i < nk; ++i) probs[i] = tr_krk(d, kraus + (size_t)i * 2 * d * d, rho);
    return 0;
}

int bto_weighted_sample(int np, const double* p, double u) {
    double cw = 0;
    for (int i = 0; i < np; ++i) {
        cw += p[i];
        if (u <= cw) return i;
    }
    return -1;
}

/* LinearAlgebra.normalize: x * inv(norm(x)) */
static void normalize(int64_t len, double* psi) {
    double s = 0;
    for (int64_t i = 0; i < 2 * len; ++i) s += psi[i] * psi[i];
    double inv = 1.0 / sqrt(s);
    for (int64_t i = 0; i < 2 * len; ++i) psi[i] *= inv;
}

int bto_channel_traj(int n, double* psi, int k, int q, int t, int nk, const double* kraus,
                     double u, int forced, int* branch, double* probs) {
    double pl[256];
    if (nk > 256) return -1;
    int rc = bto_calc_prob(n, psi, k, q, t, nk, kraus, pl);
    if (rc) return rc;
    if (probs) memcpy(probs, pl, sizeof(double) * nk);
    int ind = forced >= 0 ? forced : bto_weighted_sample(nk, pl, u);
    if (ind < 0 || ind >= nk) return -1;
    if (branch) *branch = ind;
    int d = 1 << k;
    const double* K = kraus + (size_t)ind * 2 * d * d;
    if (k == 1) rc = bto_hilbert1(n, psi, K, q, -2);
    else if (k == 2) rc = bto_hilbert2(n, psi, K, q, t, -2);
    else rc = bto_hilbert3(n, psi, K, q);
    if (rc) return rc;
    normalize(1LL << n, psi);
    return 0;
}

/* prob0 = real(partial_trace(psi, q))[1,1]; ind = rand() < prob0 ? 0 : 1;
 * psi = normalize(hilbert(N, P_ind, q) * psi) (src/hilbert.jl:682-696) */
int bto_born_measure_z(int n, double* psi, int q, double u, int forced, int* outcome, double* p0) {
    double rho[8];
    int rc = bto_partial_trace1(n, psi, q, rho);
    if (rc) return rc;
    double prob0 = rho[0];
    if (p0) *p0 = prob0;
    int ind = forced >= 0 ? forced : (u < prob0 ? 0 : 1);
    if (outcome) *outcome = ind;
    int b = bitpos(n, q);
    int64_t len = 1LL << n;
    for (int64_t i = 0; i < len; ++i)
        if ((int)((i >> b) & 1) != ind) { psi[2 * i] = 0.0; psi[2 * i + 1] = 0.0; }
    normalize(len, psi);
    return 0;
}

/* born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721): slist = the state
 * projected by P0 P0, P1 P0, P0 P1, P1 P1 on (q1, q2), weights |psi' slist[k]|,
 * k = _weighted_sample(weights) (src/hilbert.jl:810-819: first k with
 * u <= cumsum, not renormalised), result normalize(slist[k]).  outcome is the
 * reference's 1-based k; forced (1..4) replaces the draw; -1 and no change when
 * u exceeds the total weight (the reference has no index there). */
int bto_born_measure_z2(int n, double* psi, int q1, int q2, double u, int forced, int* outcome, double* probs) {
    if (q1 < 1 || q1 > n || q2 < 1 || q2 > n || q1 == q2) return -1;
    const int b1 = bitpos(n, q1), b2 = bitpos(n, q2);
    const int64_t len = 1LL << n;
    double p[4] = {0, 0, 0, 0};
    for (int64_t i = 0; i < len; ++i) {
        /* slot of [P0P0, P1P0, P0P1, P1P1]: q1's bit is the low digit */
        const int k = (int)((i >> b1) & 1) + 2 * (int)((i >> b2) & 1);
        p[k] += psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
    }
    if (probs)
        for (int k = 0; k < 4; ++k) probs[k] = p[k];
    int ind = -1;
    if (forced >= 1 && forced <= 4) ind = forced - 1;
    else {
        double cum = 0;
        for (int k = 0; k < 4 && ind < 0; ++k) {
            cum += p[k];
            if (u <= cum) ind = k;
        }
    }
    if (outcome) *outcome = ind < 0 ? -1 : ind + 1;
    if (ind < 0) return 0;
    for (int64_t i = 0; i < len; ++i) {
        const int k = (int)((i >> b1) & 1) + 2 * (int)((i >> b2) & 1);
        if (k != ind) { psi[2 * i] = 0.0; psi[2 * i + 1] = 0.0; }
    }
    normalize(len, psi);
    return 0;
}

/* e_op * rho * e_op': apply E to every column, then conj(E) to every row */
static int dm_apply_bits(int n, double* rho, int k, const int* bits, const double* m, int nc,
                         const int* cbits) {
    int64_t dim = 1LL << n;
    int rc = 0;
    for (int64_t j = 0; j < dim && !rc; ++j)   /* column j: contiguous */
        rc = apply_bits(n, rho + 2 * j * dim, 1, k, bits, m, nc, cbits, 0, 0);
    for (int64_t i = 0; i < dim && !rc; ++i)   /* row i: stride dim */
        rc = apply_bits(n, rho + 2 * i, dim, k, bits, m, nc, cbits, 1, 0);
    return rc;
}

int bto_dm_gate(int n, double* rho, int k, const int* qubits, const double* m, int nctrl,
                const int* ctrls) {
    int bits[16], cb[64];
    if (k > 10 || nctrl > 64) return -1;
    for (int i = 0; i < k; ++i) {
        if (qubits[i] < 1 || qubits[i] > n) return -1;
        bits[i] = bitpos(n, qubits[i]);
    }
    for (int i = 0; i < nctrl; ++i) {
        if (ctrls[i] < 1 || ctrls[i] > n) return -1;
        cb[i] = bitpos(n, ctrls[i]);
    }
    return dm_apply_bits(n, rho, k, bits, m, nctrl, cb);
}

int bto_dm_hilbert1(int n, double* rho, const double* m, int q, int control) {
    if (q > n || control > n) return -1;
    if (control == -2) return bto_dm_gate(n, rho, 1, &q, m, 0, NULL);
    return bto_dm_gate(n, rho, 1, &q, m, 1, &control);
}

int bto_dm_hilbert2(int n, double* rho, const double* m, int q, int t, int control) {
    if (n < q || n < t || n < control || q == t) return -1;
    if (control != -2 && abs(q - t) != 1) {
        static const double CX[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0};
        static const double CZ[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, -1};
        if (!mat_equal_real(m, CX, 4) && !mat_equal_real(m, CZ, 4)) return -2;
    }
    double fm[32];
    if (q > t) swap_ct(m, fm); else memcpy(fm, m, sizeof(fm));
    int qs[2] = {q < t ? q : t, q < t ? t : q};
    if (control == -2) return bto_dm_gate(n, rho, 2, qs, fm, 0, NULL);
    return bto_dm_gate(n, rho, 2, qs, fm, 1, &control);
}

int bto_dm_channel(int n, double* rho, int k, int q, int t, int nk, const double* kraus) {
    int64_t dim = 1LL << n;
    size_t bytes = sizeof(double) * 2 * (size_t)dim * dim;
    double* acc = (double*)calloc(1, bytes);
    double* tmp = (double*)malloc(bytes);
    int d = 1 << k, rc = 0;
    for (int i = 0; i < nk && !rc; ++i) {
        memcpy(tmp, rho, bytes);
        const double* K = kraus + (size_t)i * 2 * d * d;
        if (k == 1) rc = bto_dm_hilbert1(n, tmp, K, q, -2);
        else if (k == 2) rc = bto_dm_hilbert2(n, tmp, K, q, t, -2);
        else rc = -1;
        for (int64_t e = 0; e < 2 * dim * dim; ++e) acc[e] += tmp[e];
    }
    if (!rc) memcpy(rho, acc, bytes);
    free(acc);
    free(tmp);
    return rc;
}

int bto_dm_dephase(int n, double* rho, int q) {
    if (q < 1 || q > n) return -1;
    int b = bitpos(n, q);
    int64_t dim = 1LL << n;
    for (int64_t j = 0; j < dim; ++j)
        for (int64_t i = 0; i < dim; ++i)
            if (((i >> b) & 1) != ((j >> b) & 1)) { rho[2 * (i + j * dim)] = 0; rho[2 * (i + j * dim) + 1] = 0; }
    return 0;
}

/* P|i> = i^{popcount(x&z)} (-1)^{popcount(i&z)} |i^x> */
static inline cplx pauli_phase(uint64_t i, uint64_t x, uint64_t z) {
    int ny = __builtin_popcountll(x & z) & 3;
    int sg = __builtin_popcountll(i & z) & 1;
    static const cplx ip[4] = {1, I, -1, -I};
    cplx ph = ip[ny];
    return sg ? -ph : ph;
}

double bto_expect_pauli_sv(int n, const double* psi, uint64_t xmask, uint64_t zmask) {
    int64_t len = 1LL << n;
    double s = 0;
    for (int64_t i = 0; i < len; ++i)
        s += creal(conj(C(psi, (int64_t)((uint64_t)i ^ xmask))) * pauli_phase(i, xmask, zmask) * C(psi, i));
    return s;
}

/* tr(rho P) = sum_a rho[a, a^x] * phase(a) */
double bto_expect_pauli_dm(int n, const double* rho, uint64_t xmask, uint64_t zmask) {
    int64_t dim = 1LL << n;
    double s = 0;
    for (int64_t a = 0; a < dim; ++a) {
        int64_t b = (int64_t)((uint64_t)a ^ xmask);
        s += creal(C(rho, a + b * dim) * pauli_phase(a, xmask, zmask));
    }
    return s;
}

double bto_expect_matrix_sv(int n, const double* psi, int k, const int* qubits, const double* m,
                            int nctrl, const int* ctrls) {
    int64_t len = 1LL << n;
    double* tmp = (double*)malloc(sizeof(double) * 2 * len);
    memcpy(tmp, psi, sizeof(double) * 2 * len);
    double s = NAN;
    if (bto_apply_k(n, tmp, k, qubits, m, nctrl, ctrls) == 0) {
        s = 0;
        for (int64_t i = 0; i < len; ++i) s += creal(conj(C(psi, i)) * C(tmp, i));
    }
    free(tmp);
    return s;
}

int bto_sample(int n, const double* psi, int64_t shots, const double* u, int64_t* out) {
    int64_t len = 1LL << n;
    double* cdf = (double*)malloc(sizeof(double) * len);
    double cw = 0;
    for (int64_t i = 0; i < len; ++i) {
        cw += psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
        cdf[i] = cw;
    }
    for (int64_t s = 0; s < shots; ++s) {
        double t = u[s] * cw;
        int64_t lo = 0, hi = len - 1; /* first i with cdf[i] >= t */
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (cdf[mid] < t) lo = mid + 1; else hi = mid;
        }
        out[s] = lo;
    }
    free(cdf);
    return 0;
}

void bto_probs(int n, const double* psi, double* out) {
    int64_t len = 1LL << n;
    for (int64_t i = 0; i < len; ++i) out[i] = psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
}

int64_t bto_run_gates(int n, double* psi, int ngates, const int* ks, const int* qubits,
                      const double* mats, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    int64_t done = 0;
    size_t moff = 0;
    int qoff = 0;
    for (int g = 0; g < ngates; ++g) {
        int k = ks[g];
        if (bto_apply_k(n, psi, k, qubits + qoff, mats + moff, 0, NULL)) return -1;
        qoff += k;
        moff += (size_t)2 << (2 * k);
        ++done;
    }
    return done;
}

int bto_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
