/*
 * CPU oracle for the HiQ SimulatorMPI state-vector path.
 *
 * TEST INFRASTRUCTURE ONLY. This file restates, in plain C with OpenMP, the
 * arithmetic of the reference engine's hot path so that the CUDA product can
 * be checked against it. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm may load it; the product never links it.
 *
 * Pinning: every function here is checked in tests/test_oracle_pin.py against
 * golden vectors produced by the reference engine itself (the unmodified
 * _cppsim_mpi / _sched_cpp sources compiled by oracle/build_ref.sh), committed
 * under tests/golden/.
 *
 * Layout: a state of n qubits is 2^n complex128 values stored interleaved
 * (re, im) exactly like std::complex<double> (SimulatorMPI.hpp:47-51).
 * Matrices are dim x dim complex, row-major, interleaved.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) {
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cplx cadd(cplx a, cplx b) {
    cplx r = {a.re + b.re, a.im + b.im};
    return r;
}

/* Insert a zero bit at each of the sorted positions spos[0..nb) of index g. */
static inline uint64_t deposit_zeros(uint64_t g, const unsigned* spos, int nb) {
    for (int j = 0; j < nb; ++j) {
        uint64_t low = g & ((1ULL << spos[j]) - 1);
        g = ((g - low) << 1) | low;
    }
    return g;
}

/*
 * Apply a k-qubit matrix (k = 0..5) to the state in place.
 * Restates kernelK / kernel_core / kernel_core_diag
 * (src/simulator-mpi/kernels/nointrin/kernel1.hpp:18-78 ... kernel5.hpp:1134-1193,
 *  kernels_diag.hpp:9-81) and the dispatch in SimulatorMPI::Run
 * (src/simulator-mpi/SimulatorMPI.cpp:470-524): matrix row/column bit j
 * corresponds to state bit pos[j]; index groups whose bits at ctrlmask are not
 * all set are left unchanged. k == 0 multiplies every amplitude by m[0][0]
 * when it differs from 1 (kernelK_diag1).
 */
void orc_apply(double* psi_d, uint64_t n_amps, int k, const unsigned* pos,
               const double* m_d, uint64_t ctrlmask, int diag) {
    cplx* psi = (cplx*)psi_d;
    const cplx* m = (const cplx*)m_d;
    if (k == 0) {
        cplx d = m[0];
        if (d.re == 1.0 && d.im == 0.0) return;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n_amps; ++i) psi[i] = cmul(psi[i], d);
        return;
    }
    const int dim = 1 << k;
    unsigned spos[8];
    uint64_t off[32];
    for (int j = 0; j < k; ++j) spos[j] = pos[j];
    for (int a = 1; a < k; ++a)
        for (int b = a; b > 0 && spos[b - 1] > spos[b]; --b) {
            unsigned t = spos[b]; spos[b] = spos[b - 1]; spos[b - 1] = t;
        }
    for (int r = 0; r < dim; ++r) {
        uint64_t o = 0;
        for (int j = 0; j < k; ++j)
            if ((r >> j) & 1) o |= 1ULL << pos[j];
        off[r] = o;
    }
    const int64_t groups = (int64_t)(n_amps >> k);
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < groups; ++g) {
        uint64_t I = deposit_zeros((uint64_t)g, spos, k);
        if ((I & ctrlmask) != ctrlmask) continue;
        if (diag) {
            for (int r = 0; r < dim; ++r)
                psi[I + off[r]] = cmul(psi[I + off[r]], m[r * dim + r]);
        } else {
            cplx v[32];
            for (int c = 0; c < dim; ++c) v[c] = psi[I + off[c]];
            for (int r = 0; r < dim; ++r) {
                cplx acc = {0.0, 0.0};
                for (int c = 0; c < dim; ++c) acc = cadd(acc, cmul(m[r * dim + c], v[c]));
                psi[I + off[r]] = acc;
            }
        }
    }
}

/* Fill every amplitude with init (FillVector, SimulatorMPI.cpp:136-146,238-246). */
void orc_fill(double* psi_d, uint64_t n_amps, double re, double im) {
    cplx* psi = (cplx*)psi_d;
    cplx v = {re, im};
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n_amps; ++i) psi[i] = v;
}

/* Sum of |a_i|^2 over (i & msk) == val (getProbability_internal, SimulatorMPI.cpp:841-870). */
double orc_probability(const double* psi_d, uint64_t n_amps, uint64_t msk, uint64_t val) {
    const cplx* psi = (const cplx*)psi_d;
    double p = 0.0;
#pragma omp parallel for reduction(+ : p) schedule(static)
    for (int64_t i = 0; i < (int64_t)n_amps; ++i)
        if (((uint64_t)i & msk) == val) p += psi[i].re * psi[i].re + psi[i].im * psi[i].im;
    return p;
}

/* Zero amplitudes not matching (msk, val), scale the rest by 1/sqrt(norm)
 * (normalize, SimulatorMPI.cpp:872-895). */
void orc_normalize(double* psi_d, uint64_t n_amps, uint64_t msk, uint64_t val, double norm) {
    cplx* psi = (cplx*)psi_d;
    double s = 1.0 / sqrt(norm);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n_amps; ++i) {
        if (((uint64_t)i & msk) != val) {
            psi[i].re = 0.0; psi[i].im = 0.0;
        } else {
            psi[i].re *= s; psi[i].im *= s;
        }
    }
}

/* Block distribution used by measurement: nblocks sums of |a|^2, each summed
 * serially in index order, then an inclusive prefix sum
 * (calcLocalApproxDistribution, SimulatorMPI.cpp:817-839). */
void orc_block_cdf(const double* psi_d, uint64_t n_amps, uint64_t nblocks, double* out) {
    const cplx* psi = (const cplx*)psi_d;
    uint64_t K = n_amps / nblocks;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblocks; ++b) {
        double s = 0.0;
        for (uint64_t j = 0; j < K; ++j) {
            cplx a = psi[(uint64_t)b * K + j];
            s += a.re * a.re + a.im * a.im;
        }
        out[b] = s;
    }
    for (uint64_t b = 1; b < nblocks; ++b) out[b] += out[b - 1];
}

/* Sampled basis index for one uniform draw rnd given the block CDF cdf[nb]
 * (MeasureQubits, SimulatorMPI.cpp:897-964): first block whose CDF reaches
 * rnd, then a serial scan inside it until the running sum reaches rnd.
 * Returns -1 when rnd exceeds the total (the reference throws there).
 * margin_out receives the smallest distance between rnd and a CDF boundary
 * that decided the outcome. */
static int64_t sample_in_cdf(const cplx* psi, uint64_t n_amps, const double* cdf, uint64_t nb, double rnd,
                             double* margin_out) {
    uint64_t i = 0;
    for (; i < nb; ++i)
        if (rnd <= cdf[i]) break;
    if (i == nb) return -1;
    double margin = fabs(cdf[i] - rnd);
    if (i > 0 && fabs(rnd - cdf[i - 1]) < margin) margin = fabs(rnd - cdf[i - 1]);
    uint64_t K = n_amps / nb;
    double shift = i > 0 ? cdf[i - 1] : 0.0;
    uint64_t k = i * K;
    for (uint64_t j = 0; j < K; ++j, ++k) {
        double prev = shift;
        shift += psi[k].re * psi[k].re + psi[k].im * psi[k].im;
        if (shift >= rnd) {
            double m1 = fabs(shift - rnd), m0 = fabs(rnd - prev);
            double mm = m1 < m0 ? m1 : m0;
            if (mm < margin) margin = mm;
            break;
        }
    }
    /* the reference leaves k one past the block when the scan never reaches rnd */
    if (margin_out) *margin_out = margin;
    return (int64_t)k;
}

static uint64_t sample_blocks(uint64_t n_amps) { return n_amps < (1ULL << 15) ? n_amps : (1ULL << 15); }

int64_t orc_sample_index(const double* psi_d, uint64_t n_amps, double rnd, double* margin_out) {
    uint64_t nb = sample_blocks(n_amps);
    double* cdf = (double*)malloc(sizeof(double) * nb);
    orc_block_cdf(psi_d, n_amps, nb, cdf);
    int64_t k = sample_in_cdf((const cplx*)psi_d, n_amps, cdf, nb, rnd, margin_out);
    free(cdf);
    return k;
}

/* orc_sample_index for nrnd draws of one state: the block CDF once, then one
 * scan per draw (the state does not change between the draws). */
void orc_sample_many(const double* psi_d, uint64_t n_amps, int64_t nrnd, const double* rnd, int64_t* idx_out,
                     double* margin_out) {
    uint64_t nb = sample_blocks(n_amps);
    double* cdf = (double*)malloc(sizeof(double) * nb);
    orc_block_cdf(psi_d, n_amps, nb, cdf);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t r = 0; r < nrnd; ++r)
        idx_out[r] = sample_in_cdf((const cplx*)psi_d, n_amps, cdf, nb, rnd[r], &margin_out[r]);
    free(cdf);
}

/* P(bit pos = 0) and P(bit pos = 1) (DeallocateLocalQubit, SimulatorMPI.cpp:283-287). */
void orc_bit_probs(const double* psi_d, uint64_t n_amps, unsigned pos, double* p01) {
    const cplx* psi = (const cplx*)psi_d;
    double s0 = 0.0, s1 = 0.0;
    for (uint64_t i = 0; i < n_amps; ++i) {
        double v = psi[i].re * psi[i].re + psi[i].im * psi[i].im;
        if ((i >> pos) & 1) s1 += v; else s0 += v;
    }
    p01[0] = s0; p01[1] = s1;
}

/* Drop bit pos from the index, keeping the half where that bit equals keep
 * (the compaction loops of DeallocateLocalQubit, SimulatorMPI.cpp:303-318).
 * Writes n_amps/2 values into psi in place. */
void orc_drop_bit(double* psi_d, uint64_t n_amps, unsigned pos, int keep) {
    cplx* psi = (cplx*)psi_d;
    uint64_t half = n_amps / 2, lowm = (1ULL << pos) - 1;
    for (uint64_t i = 0; i < half; ++i) {
        uint64_t src = ((i & ~lowm) << 1) | (i & lowm) | ((uint64_t)keep << pos);
        psi[i] = psi[src];
    }
}

/* -sum p log2 p (Entropy, SimulatorMPI.cpp:681-694). */
double orc_entropy(const double* psi_d, uint64_t n_amps) {
    const cplx* psi = (const cplx*)psi_d;
    double e = 0.0;
#pragma omp parallel for reduction(+ : e) schedule(static)
    for (int64_t i = 0; i < (int64_t)n_amps; ++i) {
        double a = hypot(psi[i].re, psi[i].im);
        double pr = a * a;
        if (pr > 0) e += pr * log2(pr);
    }
    return -e;
}

/*
 * Pauli-string action. Term t is given by xmask (bits flipped by X or Y),
 * ymask (bits carrying Y) and zmask (bits carrying Z) in state-bit positions.
 * (P psi)_i = i^{|Y|} (-1)^{popcount(j & (Y|Z))} psi_j with j = i ^ xmask.
 * Restates the documented semantics of get_expectation_value /
 * apply_qubit_operator (hiq/projectq/backends/_sim/_simulator_mpi.py:148-223);
 * the reference engine has no C++ implementation of these (parity unpinned).
 */
static inline cplx pauli_phase(uint64_t j, uint64_t ymask, uint64_t zmask) {
    int ny = __builtin_popcountll(ymask) & 3;
    int sgn = __builtin_popcountll(j & (ymask | zmask)) & 1;
    static const cplx ipow[4] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};
    cplx r = ipow[ny];
    if (sgn) { r.re = -r.re; r.im = -r.im; }
    return r;
}

/* sum_t Re(c_t <psi|P_t|psi>) for nterms terms. coefs: interleaved complex. */
double orc_expectation(const double* psi_d, uint64_t n_amps, int nterms, const uint64_t* xm,
                       const uint64_t* ym, const uint64_t* zm, const double* coefs) {
    const cplx* psi = (const cplx*)psi_d;
    double total = 0.0;
    for (int t = 0; t < nterms; ++t) {
        double re = 0.0, im = 0.0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
        for (int64_t i = 0; i < (int64_t)n_amps; ++i) {
            uint64_t j = (uint64_t)i ^ xm[t];
            cplx v = cmul(pauli_phase(j, ym[t], zm[t]), psi[j]);
            cplx a = psi[i];
            re += a.re * v.re + a.im * v.im;
            im += a.re * v.im - a.im * v.re;
        }
        cplx c = {coefs[2 * t], coefs[2 * t + 1]};
        total += c.re * re - c.im * im;
    }
    return total;
}

/* psi <- sum_t c_t P_t psi (no renormalisation). */
void orc_apply_pauli_sum(double* psi_d, uint64_t n_amps, int nterms, const uint64_t* xm,
                         const uint64_t* ym, const uint64_t* zm, const double* coefs) {
    cplx* psi = (cplx*)psi_d;
    cplx* out = (cplx*)calloc(n_amps, sizeof(cplx));
    for (int t = 0; t < nterms; ++t) {
        cplx c = {coefs[2 * t], coefs[2 * t + 1]};
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n_amps; ++i) {
            uint64_t j = (uint64_t)i ^ xm[t];
            out[i] = cadd(out[i], cmul(c, cmul(pauli_phase(j, ym[t], zm[t]), psi[j])));
        }
    }
    memcpy(psi, out, n_amps * sizeof(cplx));
    free(out);
}

/*
 * MT19937 (Matsumoto & Nishimura 1998) and the libstdc++ mapping of
 * std::uniform_real_distribution<double>(0, 1) over it (generate_canonical
 * with two 32-bit draws). The reference draws one such number per
 * MeasureQubits call from std::mt19937(seed) (SimulatorMPI.cpp:88,100-101,920).
 */
typedef struct { uint32_t mt[624]; int idx; } orc_mt;

void orc_mt_seed(orc_mt* s, uint64_t seed) {
    s->mt[0] = (uint32_t)seed;
    for (int i = 1; i < 624; ++i)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->idx = 624;
}

uint32_t orc_mt_next(orc_mt* s) {
    if (s->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = s->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            s->mt[i] = v;
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double orc_mt_uniform(orc_mt* s) {
    double lo = (double)orc_mt_next(s);
    double hi = (double)orc_mt_next(s);
    double r = (lo + hi * 4294967296.0) / 18446744073709551616.0;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

size_t orc_mt_size(void) { return sizeof(orc_mt); }
