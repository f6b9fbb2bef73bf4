/*
 * CPU oracle for the statevector hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This file restates, in plain C with OpenMP, the scalar (non-SIMD) code paths
 * of pyquafu's qfvm complex128 statevector:
 *   src/qfvm/statevector.hpp  (gate kernels, expectation, sampling)
 *   src/qfvm/simulator.hpp    (named-gate dispatch, rzz = cx.rz.cx)
 * Every function names the reference lines it follows.  Only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load this library; the
 * GPU engine never calls it.
 *
 * Floating-point discipline: compiled with -ffp-contract=off so that every
 * product and sum is rounded separately, which fixes the probability and CDF
 * arithmetic used by measure_samples bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "qsv_oracle.h"

typedef struct {
    double re, im;
} cplx;

static inline cplx cmul(cplx a, cplx b) {
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cplx cadd(cplx a, cplx b) {
    cplx r = {a.re + b.re, a.im + b.im};
    return r;
}
static inline cplx rmul(double s, cplx a) {
    cplx r = {s * a.re, s * a.im};
    return r;
}

/* Insert a zero bit at position pos (statevector.hpp:460 getind_func). */
static inline uint64_t insert0(uint64_t j, unsigned pos) {
    return (j & ((1ULL << pos) - 1)) | ((j >> pos) << (pos + 1));
}

/* Index generator shared by the one-target kernels: statevector.hpp:454-500.
 * ctrl_num is 0, 1, or 2 (2 means "two or more controls"). */
typedef struct {
    int ctrl_num;
    unsigned targe, control, npos;
    unsigned posv[64], sorted[64];
    uint64_t offset, setbit, poffset, rsize;
} index_gen;

static int cmp_u(const void* a, const void* b) {
    unsigned x = *(const unsigned*)a, y = *(const unsigned*)b;
    return (x > y) - (x < y);
}

static void make_index_gen(index_gen* g, const int32_t* posv, int npos, int ctrl_num, uint64_t size) {
    memset(g, 0, sizeof(*g));
    g->ctrl_num = ctrl_num;
    g->npos = (unsigned)npos;
    for (int k = 0; k < npos; ++k) g->posv[k] = g->sorted[k] = (unsigned)posv[k];
    if (ctrl_num == 0) {
        g->targe = posv[0];
        g->offset = 1ULL << g->targe;
        g->rsize = size >> 1;
    } else if (ctrl_num == 1) {
        g->control = posv[0];
        g->targe = posv[1];
        g->offset = 1ULL << g->targe;
        g->setbit = 1ULL << g->control;
        if (g->control > g->targe) g->control--;
        g->poffset = 1ULL << g->control;
        g->rsize = size >> 2;
    } else {
        unsigned c = (unsigned)posv[0];
        for (int k = 0; k < npos - 1; ++k)
            if ((unsigned)posv[k] < c) c = (unsigned)posv[k];
        g->control = c;
        g->targe = posv[npos - 1];
        g->offset = 1ULL << g->targe;
        qsort(g->sorted, npos, sizeof(unsigned), cmp_u);
        g->rsize = size >> npos;
    }
}

/* getind_func of statevector.hpp:460 / :473-477 / :488-498. */
static inline uint64_t getind(const index_gen* g, uint64_t j) {
    if (g->ctrl_num == 0) return (j & (g->offset - 1)) | ((j >> g->targe) << (g->targe + 1));
    if (g->ctrl_num == 1) {
        uint64_t i = ((j >> g->control) << (g->control + 1)) | (j & (g->poffset - 1));
        i = ((i >> g->targe) << (g->targe + 1)) | (i & (g->offset - 1)) | g->setbit;
        return i;
    }
    uint64_t i = j;
    for (unsigned k = 0; k < g->npos; ++k) i = insert0(i, g->sorted[k]);
    for (unsigned k = 0; k + 1 < g->npos; ++k) i |= 1ULL << g->posv[k];
    return i;
}

/* getind_func_near: 2*j without controls, else getind (statevector.hpp:458, :479). */
static inline uint64_t getind_near(const index_gen* g, uint64_t j) {
    return g->ctrl_num == 0 ? 2 * j : getind(g, j);
}

static inline int has_control(const index_gen* g) { return g->ctrl_num != 0; }

/* apply_one_targe_gate_general<ctrl>: statevector.hpp:441-581 (scalar branch). */
void qor_one_targe_general(double* data_, uint64_t size, const int32_t* posv, int npos, int ctrl_num,
                           const double* mat /* 4 complex, row-major */) {
    cplx* data = (cplx*)data_;
    index_gen g;
    make_index_gen(&g, posv, npos, ctrl_num, size);
    const cplx m00 = {mat[0], mat[1]}, m01 = {mat[2], mat[3]}, m10 = {mat[4], mat[5]}, m11 = {mat[6], mat[7]};
    const int64_t rsize = (int64_t)g.rsize;
    if (g.targe == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind_near(&g, (uint64_t)j);
            cplx temp = data[i];
            data[i] = cadd(cmul(m00, data[i]), cmul(m01, data[i + 1]));
            data[i + 1] = cadd(cmul(m10, temp), cmul(m11, data[i + 1]));
        }
    } else if (has_control(&g) && g.control == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind(&g, (uint64_t)j);
            cplx temp = data[i];
            data[i] = cadd(cmul(m00, data[i]), cmul(m01, data[i + g.offset]));
            data[i + g.offset] = cadd(cmul(m10, temp), cmul(m11, data[i + g.offset]));
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j += 2) {
            uint64_t i = getind(&g, (uint64_t)j), i1 = i + 1, off = g.offset;
            cplx temp = data[i], temp1 = data[i1];
            data[i] = cadd(cmul(m00, data[i]), cmul(m01, data[i + off]));
            data[i + off] = cadd(cmul(m10, temp), cmul(m11, data[i + off]));
            data[i1] = cadd(cmul(m00, data[i1]), cmul(m01, data[i1 + off]));
            data[i1 + off] = cadd(cmul(m10, temp1), cmul(m11, data[i1 + off]));
        }
    }
}

/* apply_one_targe_gate_x<ctrl>: statevector.hpp:583-689 (scalar branch). */
void qor_one_targe_x(double* data_, uint64_t size, const int32_t* posv, int npos, int ctrl_num) {
    cplx* data = (cplx*)data_;
    index_gen g;
    make_index_gen(&g, posv, npos, ctrl_num, size);
    const int64_t rsize = (int64_t)g.rsize;
    if (g.targe == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind(&g, (uint64_t)j);
            cplx t = data[i];
            data[i] = data[i + 1];
            data[i + 1] = t;
        }
    } else if (has_control(&g) && g.control == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind(&g, (uint64_t)j);
            cplx t = data[i];
            data[i] = data[i + g.offset];
            data[i + g.offset] = t;
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j += 2) {
            uint64_t i = getind(&g, (uint64_t)j), i1 = i + 1, off = g.offset;
            cplx t = data[i];
            data[i] = data[i + off];
            data[i + off] = t;
            t = data[i1];
            data[i1] = data[i1 + off];
            data[i1 + off] = t;
        }
    }
}

/* apply_one_targe_gate_real<ctrl>: statevector.hpp:691-818 (scalar branch). */
void qor_one_targe_real(double* data_, uint64_t size, const int32_t* posv, int npos, int ctrl_num,
                        const double* mat /* 4 complex; real parts used */) {
    cplx* data = (cplx*)data_;
    index_gen g;
    make_index_gen(&g, posv, npos, ctrl_num, size);
    const double m00 = mat[0], m01 = mat[2], m10 = mat[4], m11 = mat[6];
    const int64_t rsize = (int64_t)g.rsize;
    if (g.targe == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind_near(&g, (uint64_t)j);
            cplx temp = data[i];
            data[i] = cadd(rmul(m00, data[i]), rmul(m01, data[i + 1]));
            data[i + 1] = cadd(rmul(m10, temp), rmul(m11, data[i + 1]));
        }
    } else if (has_control(&g) && g.control == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind(&g, (uint64_t)j);
            cplx temp = data[i];
            data[i] = cadd(rmul(m00, data[i]), rmul(m01, data[i + g.offset]));
            data[i + g.offset] = cadd(rmul(m10, temp), rmul(m11, data[i + g.offset]));
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j += 2) {
            uint64_t i = getind(&g, (uint64_t)j), i1 = i + 1, off = g.offset;
            cplx temp = data[i], temp1 = data[i1];
            data[i] = cadd(rmul(m00, data[i]), rmul(m01, data[i + off]));
            data[i + off] = cadd(rmul(m10, temp), rmul(m11, data[i + off]));
            data[i1] = cadd(rmul(m00, data[i1]), rmul(m01, data[i1 + off]));
            data[i1 + off] = cadd(rmul(m10, temp1), rmul(m11, data[i1 + off]));
        }
    }
}

/* apply_one_targe_gate_diag<ctrl>: statevector.hpp:820-943 (scalar branch). */
void qor_one_targe_diag(double* data_, uint64_t size, const int32_t* posv, int npos, int ctrl_num,
                        const double* mat /* 2 complex: diagonal */) {
    cplx* data = (cplx*)data_;
    index_gen g;
    make_index_gen(&g, posv, npos, ctrl_num, size);
    const cplx d0 = {mat[0], mat[1]}, d1 = {mat[2], mat[3]};
    const int64_t rsize = (int64_t)g.rsize;
    if (g.targe == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind_near(&g, (uint64_t)j);
            data[i] = cmul(data[i], d0);
            data[i + 1] = cmul(data[i + 1], d1);
        }
    } else if (has_control(&g) && g.control == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = getind(&g, (uint64_t)j);
            data[i] = cmul(data[i], d0);
            data[i + g.offset] = cmul(data[i + g.offset], d1);
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < rsize; j += 2) {
            uint64_t i = getind(&g, (uint64_t)j), i1 = i + 1, off = g.offset;
            data[i] = cmul(data[i], d0);
            data[i + off] = cmul(data[i + off], d1);
            data[i1] = cmul(data[i1], d0);
            data[i1 + off] = cmul(data[i1 + off], d1);
        }
    }
}

/* apply_x / apply_y / apply_z: statevector.hpp:206-338 (scalar branches). */
void qor_apply_x(double* data_, uint64_t size, int32_t pos) {
    cplx* data = (cplx*)data_;
    const uint64_t offset = 1ULL << pos, rsize = size >> 1;
    if (pos == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < (int64_t)size; j += 2) {
            cplx t = data[j];
            data[j] = data[j + 1];
            data[j + 1] = t;
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < (int64_t)rsize; j += 2) {
            uint64_t i = insert0((uint64_t)j, (unsigned)pos), i1 = i + 1;
            cplx t = data[i];
            data[i] = data[i + offset];
            data[i + offset] = t;
            t = data[i1];
            data[i1] = data[i1 + offset];
            data[i1 + offset] = t;
        }
    }
}

void qor_apply_y(double* data_, uint64_t size, int32_t pos) {
    cplx* data = (cplx*)data_;
    const uint64_t offset = 1ULL << pos, rsize = size >> 1;
    /* -i*(a+bi) = b - ai ; i*(a+bi) = -b + ai */
    if (pos == 0) {
#pragma omp parallel for
        for (int64_t j = 0; j < (int64_t)size; j += 2) {
            cplx temp = data[j], d1 = data[j + 1];
            data[j].re = d1.im;
            data[j].im = -d1.re;
            data[j + 1].re = -temp.im;
            data[j + 1].im = temp.re;
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < (int64_t)rsize; j += 2) {
            uint64_t i = insert0((uint64_t)j, (unsigned)pos);
            for (int u = 0; u < 2; ++u) {
                uint64_t a = i + u, b = i + u + offset;
                cplx temp = data[a], db = data[b];
                data[a].re = db.im;
                data[a].im = -db.re;
                data[b].re = -temp.im;
                data[b].im = temp.re;
            }
        }
    }
}

void qor_apply_z(double* data_, uint64_t size, int32_t pos) {
    cplx* data = (cplx*)data_;
    const uint64_t offset = 1ULL << pos, rsize = size >> 1;
    if (pos == 0) {
#pragma omp parallel for
        for (int64_t j = 1; j < (int64_t)size; j += 2) {
            data[j].re = -data[j].re;
            data[j].im = -data[j].im;
        }
    } else {
#pragma omp parallel for
        for (int64_t j = 0; j < (int64_t)rsize; j += 2) {
            uint64_t i = insert0((uint64_t)j, (unsigned)pos);
            data[i + offset].re = -data[i + offset].re;
            data[i + offset].im = -data[i + offset].im;
            data[i + offset + 1].re = -data[i + offset + 1].re;
            data[i + offset + 1].im = -data[i + offset + 1].im;
        }
    }
}

/* apply_multi_targe_gate_general: statevector.hpp:945-995.  Matrix row/column
 * bit j corresponds to targs[j] = posv[control_num + j]; controls forced to 1. */
void qor_multi_targe_general(double* data_, uint64_t size, const int32_t* posv, int npos, int control_num,
                             const double* mat /* (2^k)^2 complex, row-major */) {
    cplx* data = (cplx*)data_;
    const int targe_num = npos - control_num;
    const uint64_t matsize = 1ULL << targe_num;
    unsigned sorted[64];
    for (int k = 0; k < npos; ++k) sorted[k] = (unsigned)posv[k];
    qsort(sorted, npos, sizeof(unsigned), cmp_u);
    uint64_t* targ_mask = (uint64_t*)calloc(matsize, sizeof(uint64_t));
    for (uint64_t m = 0; m < matsize; m++)
        for (int j = 0; j < targe_num; j++)
            if ((m >> j) & 1) targ_mask[m] |= 1ULL << posv[control_num + j];
    const int64_t rsize = (int64_t)(size >> npos);
#pragma omp parallel
    {
        cplx* vin = (cplx*)malloc(matsize * sizeof(cplx));
        cplx* vout = (cplx*)malloc(matsize * sizeof(cplx));
#pragma omp for
        for (int64_t j = 0; j < rsize; j++) {
            uint64_t i = (uint64_t)j;
            for (int k = 0; k < npos; k++) i = insert0(i, sorted[k]);
            for (int k = 0; k < control_num; k++) i |= 1ULL << posv[k];
            for (uint64_t m = 0; m < matsize; m++) vin[m] = data[i | targ_mask[m]];
            /* plain row-wise sum of products (the Eigen product) */
            for (uint64_t r = 0; r < matsize; r++) {
                cplx acc = {0.0, 0.0};
                for (uint64_t c = 0; c < matsize; c++) {
                    cplx mv = {mat[2 * (r * matsize + c)], mat[2 * (r * matsize + c) + 1]};
                    acc = cadd(acc, cmul(mv, vin[c]));
                }
                vout[r] = acc;
            }
            for (uint64_t m = 0; m < matsize; m++) data[i | targ_mask[m]] = vout[m];
        }
        free(vin);
        free(vout);
    }
    free(targ_mask);
}

static inline unsigned popcount64(uint64_t x) { return (unsigned)__builtin_popcountll(x); }

/* expect_pauli: statevector.hpp:1250-1305.  x_mask = flip mask (X and Y),
 * z_mask = Z and Y positions, y_count = number of Y factors.  The 64-bit
 * popcount fixes the reference's 32-bit truncation (identical below 32 qubits). */
double qor_expect_pauli(const double* data_, uint64_t size, uint64_t x_mask, uint64_t z_mask, int y_count) {
    const cplx* data = (const cplx*)data_;
    double val = 0.0;
    if (!x_mask) {
#pragma omp parallel for reduction(+ : val)
        for (int64_t j = 0; j < (int64_t)size; ++j) {
            unsigned zp = popcount64((uint64_t)j & z_mask) % 2;
            int sign = 1 - 2 * (int)zp;
            val += (data[j].re * data[j].re + data[j].im * data[j].im) * sign;
        }
        return val;
    }
    unsigned flip_q = 63 - (unsigned)__builtin_clzll(x_mask);
    const int64_t rsize = (int64_t)(size >> 1);
    static const double PH[4][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}}; /* util.h:125 PHASE_YZ */
#pragma omp parallel for reduction(+ : val)
    for (int64_t j = 0; j < rsize; ++j) {
        uint64_t i0 = insert0((uint64_t)j, flip_q), i1 = i0 ^ x_mask;
        unsigned zp = popcount64(i0 & z_mask) % 2;
        unsigned tot = zp * 2 + (unsigned)y_count;
        cplx ph = {PH[tot % 4][0], PH[tot % 4][1]};
        cplx c1 = {data[i1].re, -data[i1].im};
        cplx t = cmul(cmul(data[i0], c1), ph);
        val += 2. * t.re;
    }
    return val;
}

/* measure_samples scan: statevector.hpp:1387-1401 with caller-supplied uniforms.
 * Writes the sampled basis index per shot; an index equal to size means the
 * uniform was not below the total probability (the reference's loop end). */
void qor_sample_indices(const double* data_, uint64_t size, const double* uniforms, int64_t shots, uint64_t* out) {
    const cplx* data = (const cplx*)data_;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t s = 0; s < shots; ++s) {
        double r = uniforms[s], p = 0.0;
        uint64_t sample;
        for (sample = 0; sample < size; ++sample) {
            double re = data[sample].re, im = data[sample].im;
            double pr = re * re;
            double pi = im * im;
            p += pr + pi;
            if (r < p) break;
        }
        out[s] = sample;
    }
}

/* The scan above for every shot in one walk of the running sum: `order`
 * lists the shots by ascending uniform, so each shot's first index whose
 * running sum exceeds its uniform is found in turn.  The sums and the
 * comparisons are those of the per-shot loop, so the indices are equal. */
void qor_sample_indices_sorted(const double* data_, uint64_t size, const double* uniforms, const int64_t* order,
                               int64_t shots, uint64_t* out) {
    const cplx* data = (const cplx*)data_;
    double p = 0.0;
    int64_t k = 0;
    for (uint64_t i = 0; i < size && k < shots; ++i) {
        double re = data[i].re, im = data[i].im;
        double pr = re * re;
        double pi = im * im;
        p += pr + pi;
        while (k < shots && uniforms[order[k]] < p) out[order[k++]] = i;
    }
    for (; k < shots; ++k) out[order[k]] = size;
}

/* Inclusive FP64 CDF in index order (the running sum of the scan above). */
void qor_sequential_cdf(const double* data_, uint64_t size, double* cdf) {
    const cplx* data = (const cplx*)data_;
    double p = 0.0;
    for (uint64_t i = 0; i < size; ++i) {
        double pr = data[i].re * data[i].re;
        double pi = data[i].im * data[i].im;
        p += pr + pi;
        cdf[i] = p;
    }
}

/* ---------------- named gates: statevector.hpp:340-437, simulator.hpp:30-113 ---------------- */

static void one_targe_named_general(double* d, uint64_t size, int32_t pos, const double* m) {
    int32_t p[1] = {pos};
    qor_one_targe_general(d, size, p, 1, 0, m);
}

int qor_apply_named(double* d, uint64_t size, int kind, const int32_t* q, const double* params) {
    const double PI_ = 3.14159265358979323846;
    switch (kind) {
        case QOR_X: qor_apply_x(d, size, q[0]); return 0;
        case QOR_Y: qor_apply_y(d, size, q[0]); return 0;
        case QOR_Z: qor_apply_z(d, size, q[0]); return 0;
        case QOR_H: {
            const double s = 1. / sqrt(2.);
            double m[8] = {s, 0, s, 0, s, 0, -s, 0};
            int32_t p[1] = {q[0]};
            qor_one_targe_real(d, size, p, 1, 0, m);
            return 0;
        }
        case QOR_S: case QOR_SDG: case QOR_T: case QOR_TDG: case QOR_P: case QOR_RZ: {
            double m[4];
            if (kind == QOR_S) { m[0] = 1; m[1] = 0; m[2] = 0; m[3] = 1; }
            else if (kind == QOR_SDG) { m[0] = 1; m[1] = 0; m[2] = 0; m[3] = -1; }
            else if (kind == QOR_T || kind == QOR_TDG) {
                /* std::exp(i*PI/4) = (cos(PI/4), sin(PI/4)) */
                double a = (kind == QOR_T ? 1.0 : -1.0) * PI_ / 4.;
                m[0] = 1; m[1] = 0; m[2] = cos(a); m[3] = sin(a);
            } else if (kind == QOR_P) {
                m[0] = 1; m[1] = 0; m[2] = cos(params[0]); m[3] = sin(params[0]);
            } else { /* rz: diag(exp(-i t/2), exp(i t/2)) */
                double h = params[0] / 2.;
                m[0] = cos(-h); m[1] = sin(-h); m[2] = cos(h); m[3] = sin(h);
            }
            int32_t p[1] = {q[0]};
            qor_one_targe_diag(d, size, p, 1, 0, m);
            return 0;
        }
        case QOR_RX: {
            double c = cos(params[0] / 2), s = sin(params[0] / 2);
            double m[8] = {c, 0, 0, -s, 0, -s, c, 0};
            one_targe_named_general(d, size, q[0], m);
            return 0;
        }
        case QOR_RY: {
            double c = cos(params[0] / 2), s = sin(params[0] / 2);
            double m[8] = {c, 0, -s, 0, s, 0, c, 0};
            int32_t p[1] = {q[0]};
            qor_one_targe_real(d, size, p, 1, 0, m);
            return 0;
        }
        case QOR_CX: { int32_t p[2] = {q[0], q[1]}; qor_one_targe_x(d, size, p, 2, 1); return 0; }
        case QOR_CZ: {
            double m[4] = {1, 0, -1, 0};
            int32_t p[2] = {q[0], q[1]};
            qor_one_targe_diag(d, size, p, 2, 1, m);
            return 0;
        }
        case QOR_CP: {
            double m[4] = {1, 0, cos(params[0]), sin(params[0])};
            int32_t p[2] = {q[0], q[1]};
            qor_one_targe_diag(d, size, p, 2, 1, m);
            return 0;
        }
        case QOR_CCX: { int32_t p[3] = {q[0], q[1], q[2]}; qor_one_targe_x(d, size, p, 3, 2); return 0; }
        case QOR_RZZ: {
            /* simulator.hpp:90-94: cx(q0,q1); rz(q1); cx(q0,q1) */
            int32_t p[2] = {q[0], q[1]};
            qor_one_targe_x(d, size, p, 2, 1);
            int32_t t[1] = {q[1]};
            double ang[1] = {params[0]};
            qor_apply_named(d, size, QOR_RZ, t, ang);
            qor_one_targe_x(d, size, p, 2, 1);
            return 0;
        }
        default: return -1;
    }
}

/* apply_op_general: simulator.hpp:12-28. */
int qor_apply_matrix(double* d, uint64_t size, const int32_t* posv, int npos, int control_num, const double* mat) {
    int targe_num = npos - control_num;
    if (targe_num == 1) {
        int c = control_num == 0 ? 0 : (control_num == 1 ? 1 : 2);
        qor_one_targe_general(d, size, posv, npos, c, mat);
        return 0;
    }
    if (targe_num > 1) {
        qor_multi_targe_general(d, size, posv, npos, control_num, mat);
        return 0;
    }
    return -1;
}
