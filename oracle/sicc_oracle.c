/*
 * sicc_oracle.c — CPU restatement of the SICC receive-path arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product; see sicc_oracle.h).
 * Reference citations: L = source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp,
 * MB = source/matlab/uhd_cpp/matlab/cpu_bp_osd_decode.m.
 */
#include "sicc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* code object                                                               */
/* ------------------------------------------------------------------------- */

struct or_code {
    int n, m, k, rank, words;
    int is_acc;
    int* row_ptr;   /* [m+1] */
    int* col_ind;   /* [E] edge e -> variable (row-major edge numbering, L:2817-2830) */
    int* col_ptr;   /* [n+1] */
    int* col_edge;  /* [E] edges of each column in increasing row order */
    int* info_cols; /* [k] */
    int* pivot_cols;/* [m] */
    uint64_t* rref; /* [m][words] reduced rows (L:2890-2932) */
};

static int get_bit(const uint64_t* row, int col) { return (int)((row[col >> 6] >> (col & 63)) & 1u); }
static void flip_bit(uint64_t* row, int col) { row[col >> 6] ^= (1ull << (col & 63)); }

static int popc64(uint64_t x)
{
    int c = 0;
    while (x) { x &= x - 1; ++c; }
    return c;
}

static int cmp_int(const void* a, const void* b)
{
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* Accumulator-parity detection: L:2838-2859. */
static int has_accumulator_parity(const or_code* c)
{
    if (c->n <= c->m) return 0;
    const int k = c->n - c->m;
    int* pc = (int*)malloc(sizeof(int) * (size_t)(c->n + 1));
    int ok = 1;
    for (int r = 0; r < c->m && ok; ++r) {
        int cnt = 0;
        for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; ++e)
            if (c->col_ind[e] >= k) pc[cnt++] = c->col_ind[e] - k;
        qsort(pc, (size_t)cnt, sizeof(int), cmp_int);
        if (r == 0) ok = (cnt == 1 && pc[0] == 0);
        else ok = (cnt == 2 && pc[0] == r - 1 && pc[1] == r);
    }
    free(pc);
    return ok;
}

or_code* or_code_create(int n, int m, const int* row_ptr, const int* col_ind, int systematic_front)
{
    if (n <= 0 || m <= 0) return NULL;
    or_code* c = (or_code*)calloc(1, sizeof(or_code));
    c->n = n;
    c->m = m;
    c->words = (n + 63) / 64;
    const int E = row_ptr[m];
    c->row_ptr = (int*)malloc(sizeof(int) * (size_t)(m + 1));
    c->col_ind = (int*)malloc(sizeof(int) * (size_t)(E > 0 ? E : 1));
    memcpy(c->row_ptr, row_ptr, sizeof(int) * (size_t)(m + 1));
    memcpy(c->col_ind, col_ind, sizeof(int) * (size_t)E);
    /* column edge lists in increasing edge (= row) order, L:2820-2830 */
    c->col_ptr = (int*)calloc((size_t)n + 1, sizeof(int));
    c->col_edge = (int*)malloc(sizeof(int) * (size_t)(E > 0 ? E : 1));
    for (int e = 0; e < E; ++e) c->col_ptr[col_ind[e] + 1]++;
    for (int v = 0; v < n; ++v) c->col_ptr[v + 1] += c->col_ptr[v];
    int* fill = (int*)malloc(sizeof(int) * (size_t)n);
    memcpy(fill, c->col_ptr, sizeof(int) * (size_t)n);
    for (int e = 0; e < E; ++e) c->col_edge[fill[col_ind[e]]++] = e;
    free(fill);

    c->info_cols = (int*)malloc(sizeof(int) * (size_t)n);
    c->pivot_cols = (int*)malloc(sizeof(int) * (size_t)m);

    if (systematic_front && has_accumulator_parity(c)) {
        c->is_acc = 1;
        c->rank = m;
        c->k = n - m;
        for (int i = 0; i < c->k; ++i) c->info_cols[i] = i;
        for (int i = 0; i < m; ++i) c->pivot_cols[i] = c->k + i;
        return c;
    }

    /* GF(2) reduced row echelon form over the column order of L:2868-2885 */
    uint64_t* rows = (uint64_t*)calloc((size_t)m * (size_t)c->words, sizeof(uint64_t));
    for (int r = 0; r < m; ++r)
        for (int e = row_ptr[r]; e < row_ptr[r + 1]; ++e) flip_bit(rows + (size_t)r * c->words, col_ind[e]);
    int* order = (int*)malloc(sizeof(int) * (size_t)n);
    int no = 0;
    if (systematic_front) {
        if (n <= m) { free(order); free(rows); or_code_destroy(c); return NULL; }
        for (int col = n - m; col < n; ++col) order[no++] = col;
        for (int col = 0; col < n - m; ++col) order[no++] = col;
    } else {
        for (int col = 0; col < n; ++col) order[no++] = col;
    }
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)c->words);
    int rank = 0;
    for (int oi = 0; oi < n; ++oi) {
        const int col = order[oi];
        if (rank >= m) break;
        int pivot = -1;
        for (int r = rank; r < m; ++r)
            if (get_bit(rows + (size_t)r * c->words, col)) { pivot = r; break; }
        if (pivot < 0) continue;
        if (pivot != rank) {
            memcpy(tmp, rows + (size_t)pivot * c->words, sizeof(uint64_t) * (size_t)c->words);
            memcpy(rows + (size_t)pivot * c->words, rows + (size_t)rank * c->words, sizeof(uint64_t) * (size_t)c->words);
            memcpy(rows + (size_t)rank * c->words, tmp, sizeof(uint64_t) * (size_t)c->words);
        }
        for (int r = 0; r < m; ++r) {
            if (r != rank && get_bit(rows + (size_t)r * c->words, col)) {
                for (int w = 0; w < c->words; ++w) rows[(size_t)r * c->words + w] ^= rows[(size_t)rank * c->words + w];
            }
        }
        c->pivot_cols[rank] = col;
        ++rank;
    }
    free(tmp);
    free(order);
    if (rank != m) { free(rows); or_code_destroy(c); return NULL; } /* rank deficient, L:2906-2908 */
    uint8_t* is_pivot = (uint8_t*)calloc((size_t)n, 1);
    for (int i = 0; i < m; ++i) is_pivot[c->pivot_cols[i]] = 1;
    int k = 0;
    for (int col = 0; col < n; ++col) if (!is_pivot[col]) c->info_cols[k++] = col;
    free(is_pivot);
    c->rank = rank;
    c->k = k;
    c->rref = rows;
    return c;
}

void or_code_destroy(or_code* c)
{
    if (!c) return;
    free(c->row_ptr); free(c->col_ind); free(c->col_ptr); free(c->col_edge);
    free(c->info_cols); free(c->pivot_cols); free(c->rref);
    free(c);
}

int or_code_n(const or_code* c) { return c->n; }
int or_code_m(const or_code* c) { return c->m; }
int or_code_k(const or_code* c) { return c->k; }
int or_code_is_accumulator(const or_code* c) { return c->is_acc; }

void or_code_info_cols(const or_code* c, int* out_info, int* out_pivot)
{
    if (out_info) memcpy(out_info, c->info_cols, sizeof(int) * (size_t)c->k);
    if (out_pivot) memcpy(out_pivot, c->pivot_cols, sizeof(int) * (size_t)c->m);
}

/* L:2947-2997 */
void or_encode(const or_code* c, const uint8_t* info, uint8_t* cw)
{
    memset(cw, 0, (size_t)c->n);
    if (c->is_acc) {
        for (int i = 0; i < c->k; ++i) cw[i] = (uint8_t)(info[i] & 1u);
        uint8_t prev = 0;
        for (int r = 0; r < c->m; ++r) {
            uint8_t s = 0;
            for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; ++e)
                if (c->col_ind[e] < c->k) s ^= cw[c->col_ind[e]];
            const uint8_t p = (uint8_t)(s ^ (r == 0 ? 0u : prev));
            cw[c->k + r] = p;
            prev = p;
        }
        return;
    }
    uint64_t* w = (uint64_t*)calloc((size_t)c->words, sizeof(uint64_t));
    for (int i = 0; i < c->k; ++i) {
        if (info[i] & 1u) { cw[c->info_cols[i]] = 1; flip_bit(w, c->info_cols[i]); }
    }
    for (int r = 0; r < c->rank; ++r) {
        int par = 0;
        for (int x = 0; x < c->words; ++x) par ^= popc64(c->rref[(size_t)r * c->words + x] & w[x]) & 1;
        if (par) { cw[c->pivot_cols[r]] = 1; flip_bit(w, c->pivot_cols[r]); }
    }
    free(w);
}

/* number of unsatisfied checks; L:2999-3011 tests it against zero */
int or_syndrome_weight(const or_code* c, const uint8_t* bits)
{
    int wgt = 0;
    for (int r = 0; r < c->m; ++r) {
        int s = 0;
        for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; ++e) s ^= (bits[c->col_ind[e]] & 1);
        wgt += s;
    }
    return wgt;
}

/* L:3096-3118 (front-systematic test) and L:3133-3160 (table) */
int or_systematic_parity(const or_code* c, uint64_t* out_table, int* out_words)
{
    const int k = c->k, n = c->n, m = c->m;
    if (k <= 0 || m <= 0 || k + m != n) return 1;
    for (int i = 0; i < k; ++i) if (c->info_cols[i] != i) return 1;
    for (int i = 0; i < m; ++i) if (c->pivot_cols[i] < k) return 1;
    const int words = (n - k + 63) / 64;
    *out_words = words;
    if (!out_table) return 0;
    memset(out_table, 0, sizeof(uint64_t) * (size_t)k * (size_t)words);
    uint8_t* unit = (uint8_t*)calloc((size_t)k, 1);
    uint8_t* cw = (uint8_t*)malloc((size_t)n);
    for (int row = 0; row < k; ++row) {
        memset(unit, 0, (size_t)k);
        unit[row] = 1;
        or_encode(c, unit, cw);
        for (int p = 0; p < n - k; ++p)
            if (cw[k + p]) out_table[(size_t)row * words + (size_t)(p / 64)] |= (1ull << (p % 64));
    }
    free(unit);
    free(cw);
    return 0;
}

int or_greedy_color_order(const or_code* c, int* out_order, int* out_color_of_row)
{
    const int m = c->m, n = c->n;
    int* color = (int*)malloc(sizeof(int) * (size_t)m);
    /* used[color][var] as a growing byte table */
    int cap = 8, ncol = 0;
    uint8_t* used = (uint8_t*)calloc((size_t)cap * (size_t)n, 1);
    for (int r = 0; r < m; ++r) {
        int chosen = -1;
        for (int col = 0; col < ncol && chosen < 0; ++col) {
            int clash = 0;
            for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1] && !clash; ++e)
                clash = used[(size_t)col * n + c->col_ind[e]];
            if (!clash) chosen = col;
        }
        if (chosen < 0) {
            if (ncol == cap) {
                used = (uint8_t*)realloc(used, (size_t)cap * 2 * (size_t)n);
                memset(used + (size_t)cap * n, 0, (size_t)cap * (size_t)n);
                cap *= 2;
            }
            chosen = ncol++;
        }
        color[r] = chosen;
        for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; ++e) used[(size_t)chosen * n + c->col_ind[e]] = 1;
    }
    int o = 0;
    for (int col = 0; col < ncol; ++col)
        for (int r = 0; r < m; ++r)
            if (color[r] == col) out_order[o++] = r;
    if (out_color_of_row) memcpy(out_color_of_row, color, sizeof(int) * (size_t)m);
    free(used);
    free(color);
    return ncol;
}

/* ------------------------------------------------------------------------- */
/* belief propagation                                                        */
/* ------------------------------------------------------------------------- */

static int hard_and_weight_f(const or_code* c, const float* app, uint8_t* hard)
{
    for (int v = 0; v < c->n; ++v) hard[v] = (app[v] < 0.0f) ? 1 : 0;
    return or_syndrome_weight(c, hard);
}

/* L:3013-3094, restated operation for operation. */
int or_nms_flooding_ref(const or_code* c, const float* llr, int max_iter, double normalization,
                        uint8_t* out_bits, float* out_app, int* out_iter)
{
    const int E = c->row_ptr[c->m];
    float* q = (float*)malloc(sizeof(float) * (size_t)(E > 0 ? E : 1));
    float* rmsg = (float*)calloc((size_t)(E > 0 ? E : 1), sizeof(float));
    float* app = (float*)calloc((size_t)c->n, sizeof(float));
    uint8_t* hard = (uint8_t*)calloc((size_t)c->n, 1);
    for (int e = 0; e < E; ++e) q[e] = llr[c->col_ind[e]];
    int used = 0, ok = 0;
    for (int it = 0; it < max_iter; ++it) {
        used = it + 1;
        for (int row = 0; row < c->m; ++row) {
            float min1 = FLT_MAX, min2 = FLT_MAX;
            int min1_edge = -1, sign_prod = 1;
            for (int e = c->row_ptr[row]; e < c->row_ptr[row + 1]; ++e) {
                const float v = q[e];
                if (v < 0.0f) sign_prod = -sign_prod;
                const float av = fabsf(v);
                if (av < min1) { min2 = min1; min1 = av; min1_edge = e; }
                else if (av < min2) { min2 = av; }
            }
            for (int e = c->row_ptr[row]; e < c->row_ptr[row + 1]; ++e) {
                const int sw = (q[e] < 0.0f) ? -sign_prod : sign_prod;
                const float mag = (e == min1_edge) ? min2 : min1;
                rmsg[e] = (float)normalization * (float)sw * mag;
            }
        }
        for (int col = 0; col < c->n; ++col) {
            float v = llr[col];
            for (int j = c->col_ptr[col]; j < c->col_ptr[col + 1]; ++j) v += rmsg[c->col_edge[j]];
            app[col] = v;
            hard[col] = (v < 0.0f) ? 1 : 0;
        }
        ok = (or_syndrome_weight(c, hard) == 0);
        if (ok) break;
        for (int col = 0; col < c->n; ++col)
            for (int j = c->col_ptr[col]; j < c->col_ptr[col + 1]; ++j) {
                const int e = c->col_edge[j];
                q[e] = app[col] - rmsg[e];
            }
    }
    if (out_bits) memcpy(out_bits, hard, (size_t)c->n);
    if (out_app) memcpy(out_app, app, sizeof(float) * (size_t)c->n);
    if (out_iter) *out_iter = used;
    free(q); free(rmsg); free(app); free(hard);
    return ok;
}

/* check-node magnitude: alpha*min (beta == 0) or max(alpha*min - beta, 0) */
static float nms_mag_f(float alpha, float beta, float mn)
{
    const float a = alpha * mn;
    if (beta == 0.0f) return a;
    const float d = a - beta;
    return d > 0.0f ? d : 0.0f;
}

int or_nms_flooding_f32(const or_code* c, const float* llr, int max_iter, float alpha, float beta,
                        float damping, uint8_t* out_bits, float* out_app, float* out_best_app,
                        int* out_iter, int* out_best_w)
{
    const int E = c->row_ptr[c->m];
    float* q = (float*)malloc(sizeof(float) * (size_t)(E > 0 ? E : 1));
    float* rmsg = (float*)calloc((size_t)(E > 0 ? E : 1), sizeof(float));
    float* app = (float*)malloc(sizeof(float) * (size_t)c->n);
    float* best = (float*)malloc(sizeof(float) * (size_t)c->n);
    uint8_t* hard = (uint8_t*)calloc((size_t)c->n, 1);
    for (int e = 0; e < E; ++e) q[e] = llr[c->col_ind[e]];
    memcpy(app, llr, sizeof(float) * (size_t)c->n);
    memcpy(best, llr, sizeof(float) * (size_t)c->n);
    int best_w = hard_and_weight_f(c, llr, hard); /* MB:121-126 */
    const float keep = 1.0f - damping;
    int used = 0, ok = 0;
    for (int it = 0; it < max_iter; ++it) {
        used = it + 1;
        for (int row = 0; row < c->m; ++row) {
            float min1 = FLT_MAX, min2 = FLT_MAX;
            int min1_edge = -1;
            unsigned neg = 0;
            for (int e = c->row_ptr[row]; e < c->row_ptr[row + 1]; ++e) {
                const float v = q[e];
                if (v < 0.0f) neg ^= 1u;
                const float av = fabsf(v);
                if (av < min1) { min2 = min1; min1 = av; min1_edge = e; }
                else if (av < min2) { min2 = av; }
            }
            const float m1 = nms_mag_f(alpha, beta, min1), m2 = nms_mag_f(alpha, beta, min2);
            for (int e = c->row_ptr[row]; e < c->row_ptr[row + 1]; ++e) {
                const unsigned s = neg ^ (q[e] < 0.0f ? 1u : 0u);
                const float mag = (e == min1_edge) ? m2 : m1;
                rmsg[e] = s ? -mag : mag;
            }
        }
        for (int col = 0; col < c->n; ++col) {
            float v = llr[col];
            for (int j = c->col_ptr[col]; j < c->col_ptr[col + 1]; ++j) v += rmsg[c->col_edge[j]];
            app[col] = v;
        }
        const int w = hard_and_weight_f(c, app, hard);
        if (w < best_w) { best_w = w; memcpy(best, app, sizeof(float) * (size_t)c->n); }
        if (w == 0) { ok = 1; break; }
        for (int col = 0; col < c->n; ++col)
            for (int j = c->col_ptr[col]; j < c->col_ptr[col + 1]; ++j) {
                const int e = c->col_edge[j];
                const float fresh = app[col] - rmsg[e];
                if (damping == 0.0f) {
                    q[e] = fresh;
                } else {
                    const float a = keep * fresh;
                    const float b = damping * q[e];
                    q[e] = a + b;
                }
            }
    }
    if (out_bits) memcpy(out_bits, hard, (size_t)c->n);
    if (out_app) memcpy(out_app, app, sizeof(float) * (size_t)c->n);
    if (out_best_app) memcpy(out_best_app, best, sizeof(float) * (size_t)c->n);
    if (out_iter) *out_iter = used;
    if (out_best_w) *out_best_w = best_w;
    free(q); free(rmsg); free(app); free(best); free(hard);
    return ok;
}

int or_nms_layered_f32(const or_code* c, const int* row_order, const float* llr, int max_iter,
                       float alpha, float beta, uint8_t* out_bits, float* out_app, float* out_best_app,
                       int* out_iter, int* out_best_w)
{
    const int E = c->row_ptr[c->m];
    float* R = (float*)calloc((size_t)(E > 0 ? E : 1), sizeof(float));
    float* q = (float*)malloc(sizeof(float) * (size_t)(E > 0 ? E : 1));
    float* app = (float*)malloc(sizeof(float) * (size_t)c->n);
    float* best = (float*)malloc(sizeof(float) * (size_t)c->n);
    uint8_t* hard = (uint8_t*)calloc((size_t)c->n, 1);
    memcpy(app, llr, sizeof(float) * (size_t)c->n);
    memcpy(best, llr, sizeof(float) * (size_t)c->n);
    int best_w = hard_and_weight_f(c, llr, hard);
    int used = 0, ok = 0;
    for (int it = 0; it < max_iter; ++it) {
        used = it + 1;
        for (int ri = 0; ri < c->m; ++ri) {
            const int row = row_order ? row_order[ri] : ri;
            const int b = c->row_ptr[row], eend = c->row_ptr[row + 1];
            float min1 = FLT_MAX, min2 = FLT_MAX;
            int arg = -1;
            unsigned neg = 0;
            for (int e = b; e < eend; ++e) {
                const float qe = app[c->col_ind[e]] - R[e];
                q[e] = qe;
                if (qe < 0.0f) neg ^= 1u;
                const float a = fabsf(qe);
                if (a < min1) { min2 = min1; min1 = a; arg = e; }
                else if (a < min2) { min2 = a; }
            }
            const float m1 = nms_mag_f(alpha, beta, min1), m2 = nms_mag_f(alpha, beta, min2);
            for (int e = b; e < eend; ++e) {
                const unsigned s = neg ^ (q[e] < 0.0f ? 1u : 0u);
                const float mag = (e == arg) ? m2 : m1;
                const float r = s ? -mag : mag;
                R[e] = r;
                app[c->col_ind[e]] = q[e] + r;
            }
        }
        const int w = hard_and_weight_f(c, app, hard);
        if (w < best_w) { best_w = w; memcpy(best, app, sizeof(float) * (size_t)c->n); }
        if (w == 0) { ok = 1; break; }
    }
    if (out_bits) memcpy(out_bits, hard, (size_t)c->n);
    if (out_app) memcpy(out_app, app, sizeof(float) * (size_t)c->n);
    if (out_best_app) memcpy(out_best_app, best, sizeof(float) * (size_t)c->n);
    if (out_iter) *out_iter = used;
    if (out_best_w) *out_best_w = best_w;
    free(R); free(q); free(app); free(best); free(hard);
    return ok;
}

int or_nms_layered_f64(const or_code* c, const int* row_order, const float* llr, int max_iter,
                       double alpha, double beta, uint8_t* out_bits, double* out_app, int* out_iter)
{
    const int E = c->row_ptr[c->m];
    double* R = (double*)calloc((size_t)(E > 0 ? E : 1), sizeof(double));
    double* q = (double*)malloc(sizeof(double) * (size_t)(E > 0 ? E : 1));
    double* app = (double*)malloc(sizeof(double) * (size_t)c->n);
    uint8_t* hard = (uint8_t*)calloc((size_t)c->n, 1);
    for (int v = 0; v < c->n; ++v) app[v] = (double)llr[v];
    int used = 0, ok = 0;
    for (int it = 0; it < max_iter; ++it) {
        used = it + 1;
        for (int ri = 0; ri < c->m; ++ri) {
            const int row = row_order ? row_order[ri] : ri;
            const int b = c->row_ptr[row], eend = c->row_ptr[row + 1];
            double min1 = DBL_MAX, min2 = DBL_MAX;
            int arg = -1;
            unsigned neg = 0;
            for (int e = b; e < eend; ++e) {
                const double qe = app[c->col_ind[e]] - R[e];
                q[e] = qe;
                if (qe < 0.0) neg ^= 1u;
                const double a = fabs(qe);
                if (a < min1) { min2 = min1; min1 = a; arg = e; }
                else if (a < min2) { min2 = a; }
            }
            double m1 = alpha * min1, m2 = alpha * min2;
            if (beta != 0.0) { m1 = fmax(m1 - beta, 0.0); m2 = fmax(m2 - beta, 0.0); }
            for (int e = b; e < eend; ++e) {
                const unsigned s = neg ^ (q[e] < 0.0 ? 1u : 0u);
                const double mag = (e == arg) ? m2 : m1;
                const double r = s ? -mag : mag;
                R[e] = r;
                app[c->col_ind[e]] = q[e] + r;
            }
        }
        for (int v = 0; v < c->n; ++v) hard[v] = app[v] < 0.0 ? 1 : 0;
        if (or_syndrome_weight(c, hard) == 0) { ok = 1; break; }
    }
    if (out_bits) memcpy(out_bits, hard, (size_t)c->n);
    if (out_app) memcpy(out_app, app, sizeof(double) * (size_t)c->n);
    if (out_iter) *out_iter = used;
    free(R); free(q); free(app); free(hard);
    return ok;
}

/* ------------------------------------------------------------------------- */
/* OSD (MB:187-305)                                                          */
/* ------------------------------------------------------------------------- */

/* stable sort helpers: reliability descending (MB:194, MATLAB sort is stable) */
typedef struct { float key; int idx; } or_kv;

static int cmp_desc_stable(const void* a, const void* b)
{
    const or_kv* x = (const or_kv*)a; const or_kv* y = (const or_kv*)b;
    if (x->key > y->key) return -1;
    if (x->key < y->key) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

static int cmp_asc_stable(const void* a, const void* b)
{
    const or_kv* x = (const or_kv*)a; const or_kv* y = (const or_kv*)b;
    if (x->key < y->key) return -1;
    if (x->key > y->key) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

/* The candidate metric is the single-precision sum of |llr| over the positions
 * where the candidate differs from the hard decision, accumulated in decreasing
 * reliability order (the order of the sorted positions).  MB sums the same set
 * in double; the summation order is this restatement's definition. */
static float osd_metric(int n, const uint8_t* cand_rel, const uint8_t* hard_rel, const float* rel_sorted)
{
    float acc = 0.0f;
    for (int j = 0; j < n; ++j)
        if (cand_rel[j] != hard_rel[j]) acc = acc + rel_sorted[j];
    return acc;
}

int or_osd(int n, int k, const uint64_t* parity_table, int parity_words, const float* llr, int order,
           int max_flip_positions, int max_tests, uint8_t* out_code, float* out_metric, int* out_best_test)
{
    const int words = (n + 63) / 64;
    or_kv* kv = (or_kv*)malloc(sizeof(or_kv) * (size_t)n);
    int* relperm = (int*)malloc(sizeof(int) * (size_t)n);   /* reliabilityPerm */
    float* rel_sorted = (float*)malloc(sizeof(float) * (size_t)n);
    uint8_t* hard_rel = (uint8_t*)malloc((size_t)n);
    for (int i = 0; i < n; ++i) { kv[i].key = fabsf(llr[i]); kv[i].idx = i; }
    qsort(kv, (size_t)n, sizeof(or_kv), cmp_desc_stable);
    for (int j = 0; j < n; ++j) {
        relperm[j] = kv[j].idx;
        rel_sorted[j] = kv[j].key;
        hard_rel[j] = (llr[kv[j].idx] < 0.0f) ? 1 : 0;
    }
    /* Grel = G(:, reliabilityPerm), G = [I_k | P] */
    uint64_t* g = (uint64_t*)calloc((size_t)k * (size_t)words, sizeof(uint64_t));
    for (int r = 0; r < k; ++r) {
        uint64_t* row = g + (size_t)r * words;
        for (int j = 0; j < n; ++j) {
            const int col = relperm[j];
            int bit;
            if (col < k) bit = (col == r);
            else bit = (int)((parity_table[(size_t)r * parity_words + (size_t)((col - k) >> 6)] >> ((col - k) & 63)) & 1u);
            if (bit) flip_bit(row, j);
        }
    }
    /* generator_to_systematic, MB:270-305: column-pivoted elimination with
     * explicit row and column swaps; perm tracks the column order. */
    int* perm = (int*)malloc(sizeof(int) * (size_t)n);
    for (int j = 0; j < n; ++j) perm[j] = j;
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)words);
    for (int t = 0; t < k; ++t) {
        int prow = -1, pcol = -1;
        for (int col = t; col < n && prow < 0; ++col)
            for (int r = t; r < k; ++r)
                if (get_bit(g + (size_t)r * words, col)) { prow = r; pcol = col; break; }
        if (prow < 0) { /* rank deficient generator */
            free(kv); free(relperm); free(rel_sorted); free(hard_rel); free(g); free(perm); free(tmp);
            return -1;
        }
        if (prow != t) {
            memcpy(tmp, g + (size_t)t * words, sizeof(uint64_t) * (size_t)words);
            memcpy(g + (size_t)t * words, g + (size_t)prow * words, sizeof(uint64_t) * (size_t)words);
            memcpy(g + (size_t)prow * words, tmp, sizeof(uint64_t) * (size_t)words);
        }
        if (pcol != t) {
            for (int r = 0; r < k; ++r) {
                uint64_t* row = g + (size_t)r * words;
                const int a = get_bit(row, t), b = get_bit(row, pcol);
                if (a != b) { flip_bit(row, t); flip_bit(row, pcol); }
            }
            const int x = perm[t]; perm[t] = perm[pcol]; perm[pcol] = x;
        }
        for (int r = 0; r < k; ++r) {
            if (r != t && get_bit(g + (size_t)r * words, t))
                for (int w = 0; w < words; ++w) g[(size_t)r * words + w] ^= g[(size_t)t * words + w];
        }
    }
    free(tmp);
    /* hardSys / relSys in systematic order; MB:200-203 */
    uint8_t* base_msg = (uint8_t*)malloc((size_t)k);
    for (int i = 0; i < k; ++i) base_msg[i] = hard_rel[perm[i]];
    /* weakest-first flip pool, MB:208-209 (stable ascending sort of relSys(1:k)) */
    for (int i = 0; i < k; ++i) { kv[i].key = rel_sorted[perm[i]]; kv[i].idx = i; }
    qsort(kv, (size_t)k, sizeof(or_kv), cmp_asc_stable);
    const int pool = (k < max_flip_positions) ? k : max_flip_positions;
    int* flip = (int*)malloc(sizeof(int) * (size_t)(pool > 0 ? pool : 1));
    for (int i = 0; i < pool; ++i) flip[i] = kv[i].idx;

    uint8_t* cand_rel = (uint8_t*)malloc((size_t)n);
    uint8_t* best_rel = (uint8_t*)malloc((size_t)n);
    uint64_t* acc = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)words);
    uint8_t* msg = (uint8_t*)malloc((size_t)k);

    /* encode msg with Gsys into reliability-order positions (codeRel(sysPerm) = codeSys) */
#define OSD_EVAL(MSG, OUTM)                                                           \
    do {                                                                              \
        memset(acc, 0, sizeof(uint64_t) * (size_t)words);                             \
        for (int r_ = 0; r_ < k; ++r_)                                                \
            if ((MSG)[r_])                                                            \
                for (int w_ = 0; w_ < words; ++w_) acc[w_] ^= g[(size_t)r_ * words + w_]; \
        for (int j_ = 0; j_ < n; ++j_) cand_rel[perm[j_]] = (uint8_t)get_bit(acc, j_); \
        (OUTM) = osd_metric(n, cand_rel, hard_rel, rel_sorted);                        \
    } while (0)

    float best_metric;
    OSD_EVAL(base_msg, best_metric);
    memcpy(best_rel, cand_rel, (size_t)n);
    int best_test = 0;
    int tests = 1;
    int* comb = (int*)malloc(sizeof(int) * (size_t)(order > 0 ? order : 1));
    for (int o = 1; o <= order; ++o) {
        if (pool < o || tests >= max_tests) break;
        for (int i = 0; i < o; ++i) comb[i] = i; /* lexicographic nchoosek over the pool */
        int done = 0;
        while (!done) {
            memcpy(msg, base_msg, (size_t)k);
            for (int i = 0; i < o; ++i) msg[flip[comb[i]]] ^= 1u;
            float metric;
            OSD_EVAL(msg, metric);
            ++tests;
            if (metric < best_metric) {
                best_metric = metric;
                memcpy(best_rel, cand_rel, (size_t)n);
                best_test = tests - 1;
            }
            if (tests >= max_tests) break;
            int i = o - 1;
            while (i >= 0 && comb[i] == pool - o + i) --i;
            if (i < 0) { done = 1; break; }
            ++comb[i];
            for (int j = i + 1; j < o; ++j) comb[j] = comb[j - 1] + 1;
        }
    }
#undef OSD_EVAL
    /* codeBits(reliabilityPerm) = codeRel, MB:231-235 */
    for (int j = 0; j < n; ++j) out_code[relperm[j]] = best_rel[j];
    if (out_metric) *out_metric = best_metric;
    if (out_best_test) *out_best_test = best_test;
    free(kv); free(relperm); free(rel_sorted); free(hard_rel); free(g); free(perm);
    free(base_msg); free(flip); free(cand_rel); free(best_rel); free(acc); free(msg); free(comb);
    return tests;
}

int or_bp_osd_batch(const or_code* c, const uint64_t* parity_table, int parity_words, const float* llrs, int count,
                    int schedule, int max_iter, float alpha, int osd_order, int osd_max_flip, int osd_max_tests,
                    uint8_t* out_info, uint8_t* out_used_osd)
{
    const int n = c->n, k = c->k;
    uint8_t* bits = (uint8_t*)malloc((size_t)n);
    float* app = (float*)malloc(sizeof(float) * (size_t)n);
    float* best = (float*)malloc(sizeof(float) * (size_t)n);
    int osd = 0;
    for (int b = 0; b < count; ++b) {
        const float* x = llrs + (size_t)b * n;
        int it = 0, bw = 0, ok;
        const float* post = app;
        if (schedule == 0) {
            /* cpu_bp_osd_decode.m as the reference runs it (MB:55-62): flooding min-sum
             * (with no damping and no offset the same operations as L:3013-3094), and on
             * a failed syndrome OSD on bestAppLlr, the posterior of the lowest syndrome
             * weight seen (MB:116-119, 160-171). */
            ok = or_nms_flooding_f32(c, x, max_iter, alpha, 0.0f, 0.0f, bits, app, best, &it, &bw);
            post = best;
        } else {
            ok = or_nms_layered_f32(c, NULL, x, max_iter, alpha, 0.0f, bits, app, best, &it, &bw);
            post = best;
        }
        const int use = (!ok && osd_order >= 0);
        if (use) {
            float metric;
            int bt;
            or_osd(n, k, parity_table, parity_words, post, osd_order, osd_max_flip, osd_max_tests, bits, &metric, &bt);
            ++osd;
        }
        memcpy(out_info + (size_t)b * k, bits, (size_t)k);
        if (out_used_osd) out_used_osd[b] = (uint8_t)use;
    }
    free(bits); free(app); free(best);
    return osd;
}

/* ------------------------------------------------------------------------- */
/* OFDM receive                                                              */
/* ------------------------------------------------------------------------- */

static const double kPi = 3.141592653589793238462643383279502884;

typedef struct { double re, im; } cd;

static cd cd_mul(cd a, cd b)
{
    cd r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}

/* iterative radix-2 DIT FFT in double, L:3788-3827 (forward, unnormalised) */
static void fft_forward(cd* a, int n)
{
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { cd t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int len = 2; len <= n; len <<= 1) {
        const double ang = 2.0 * kPi / (double)len * -1.0;
        cd wlen; wlen.re = cos(ang); wlen.im = sin(ang);
        for (int i = 0; i < n; i += len) {
            cd w; w.re = 1.0; w.im = 0.0;
            for (int j = 0; j < len / 2; ++j) {
                const cd u = a[i + j];
                const cd v = cd_mul(a[i + j + len / 2], w);
                a[i + j].re = u.re + v.re; a[i + j].im = u.im + v.im;
                a[i + j + len / 2].re = u.re - v.re; a[i + j + len / 2].im = u.im - v.im;
                w = cd_mul(w, wlen);
            }
        }
    }
}

/* L:3845-3859 */
void or_fft_shifted(const float* time_iq, int nfft, float* out)
{
    cd* a = (cd*)malloc(sizeof(cd) * (size_t)nfft);
    for (int i = 0; i < nfft; ++i) { a[i].re = time_iq[2 * i]; a[i].im = time_iq[2 * i + 1]; }
    fft_forward(a, nfft);
    for (int i = 0; i < nfft; ++i) {
        const int nat = (i + nfft / 2) % nfft;
        out[2 * i] = (float)a[nat].re;
        out[2 * i + 1] = (float)a[nat].im;
    }
    free(a);
}

/* std::norm of a single-precision complex: x*x + y*y evaluated in float */
static float fnorm(float re, float im) { return re * re + im * im; }

/* L:5214-5274 */
static int sync_refine(const or_phy* p, const float* buf, long long coarse_start, double coarse_metric,
                       long long available, long long* out_start, double* out_fine, double* out_cfo,
                       int* incomplete)
{
    const long long L = p->pre_half_len, pre_len = 2 * L;
    const long long frame_len = pre_len + (long long)p->num_symbols * (p->nfft + p->cp);
    const long long radius = p->cp < 16 ? p->cp : 16;
    const long long search_limit = available - pre_len + 1;
    const long long lo = coarse_start > radius ? coarse_start - radius : 0;
    const long long hi = (search_limit - 1 < coarse_start + radius) ? search_limit - 1 : coarse_start + radius;
    double pre_energy = 0.0;
    for (long long i = 0; i < pre_len; ++i) pre_energy += fnorm(p->preamble[2 * i], p->preamble[2 * i + 1]);
    double best_m = 0.0;
    long long best = coarse_start;
    for (long long d = lo; d <= hi; ++d) {
        double cr = 0.0, ci = 0.0, eng = 0.0;
        for (long long i = 0; i < pre_len; ++i) {
            const double yr = buf[2 * (d + i)], yi = buf[2 * (d + i) + 1];
            const double pr = p->preamble[2 * i], pi = -(double)p->preamble[2 * i + 1];
            cr += yr * pr - yi * pi;
            ci += yr * pi + yi * pr;
            eng += fnorm(buf[2 * (d + i)], buf[2 * (d + i) + 1]);
        }
        const double den = eng * pre_energy > 1e-18 ? eng * pre_energy : 1e-18;
        const double m = (cr * cr + ci * ci) / den;
        if (m > best_m) { best_m = m; best = d; }
    }
    (void)coarse_metric;
    if (best_m < p->sync_threshold) return 0;
    if (best + frame_len > available) { *incomplete = 1; *out_start = best; *out_fine = best_m; return 0; }
    double ar = 0.0, ai = 0.0;
    for (long long i = 0; i < L; ++i) {
        const double x0r = buf[2 * (best + i)], x0i = -(double)buf[2 * (best + i) + 1];
        const double x1r = buf[2 * (best + i + L)], x1i = buf[2 * (best + i + L) + 1];
        ar += x0r * x1r - x0i * x1i;
        ai += x0r * x1i + x0i * x1r;
    }
    *out_start = best;
    *out_fine = best_m;
    *out_cfo = atan2(ai, ar) * p->rate / (2.0 * kPi * (double)L);
    return 1;
}

/* L:5276-5329 with base = 0 */
int or_sync_earliest(const or_phy* p, const float* buf, long long count, long long max_search,
                     long long* out_start, double* out_coarse, double* out_fine, double* out_cfo_hz)
{
    const long long L = p->pre_half_len, pre_len = 2 * L;
    *out_start = 0; *out_coarse = 0.0; *out_fine = 0.0; *out_cfo_hz = 0.0;
    if (count < pre_len) return 0;
    const long long available = count;
    long long search_limit = available - pre_len + 1;
    if (max_search > 0 && max_search + 1 < search_limit) search_limit = max_search + 1;
    double pr = 0.0, pi = 0.0, e1 = 0.0, e2 = 0.0;
    for (long long i = 0; i < L; ++i) {
        const double ar = buf[2 * i], ai = -(double)buf[2 * i + 1];
        const double br = buf[2 * (i + L)], bi = buf[2 * (i + L) + 1];
        pr += ar * br - ai * bi;
        pi += ar * bi + ai * br;
        e1 += fnorm(buf[2 * i], buf[2 * i + 1]);
        e2 += fnorm(buf[2 * (i + L)], buf[2 * (i + L) + 1]);
    }
    for (long long d = 0; d < search_limit; ++d) {
        const double den = e1 * e2 > 1e-18 ? e1 * e2 : 1e-18;
        const double metric = (pr * pr + pi * pi) / den;
        if (metric >= p->sync_threshold) {
            int incomplete = 0;
            if (sync_refine(p, buf, d, metric, available, out_start, out_fine, out_cfo_hz, &incomplete)) {
                *out_coarse = metric;
                return 1;
            }
            if (incomplete) { *out_coarse = metric; return 2; }
        }
        if (d + pre_len >= available) break;
        const double x0r = buf[2 * d], x0i = buf[2 * d + 1];
        const double x1r = buf[2 * (d + L)], x1i = buf[2 * (d + L) + 1];
        const double x2r = buf[2 * (d + pre_len)], x2i = buf[2 * (d + pre_len) + 1];
        /* p += conj(x1)*x2 - conj(x0)*x1 */
        const double ar = x1r * x2r + x1i * x2i, ai = x1r * x2i - x1i * x2r;
        const double br = x0r * x1r + x0i * x1i, bi = x0r * x1i - x0i * x1r;
        pr += ar - br;
        pi += ai - bi;
        e1 += fnorm((float)x1r, (float)x1i) - fnorm((float)x0r, (float)x0i);
        e2 += fnorm((float)x2r, (float)x2i) - fnorm((float)x1r, (float)x1i);
    }
    return 0;
}

/* L:2552-2568 */
static void llr_maxlog_one(const or_phy* p, float xr, float xi, double sigma2, float* out)
{
    if (sigma2 < 1e-8) sigma2 = 1e-8;
    const int m = 1 << p->bits_per_symbol;
    for (int bit = 0; bit < p->bits_per_symbol; ++bit) {
        float d0 = INFINITY, d1 = INFINITY;
        for (int s = 0; s < m; ++s) {
            const float dr = xr - p->constellation[2 * s], di = xi - p->constellation[2 * s + 1];
            const float d2 = fnorm(dr, di);
            const int b = (s >> (p->bits_per_symbol - 1 - bit)) & 1;
            if (b == 0) { if (d2 < d0) d0 = d2; }
            else { if (d2 < d1) d1 = d2; }
        }
        out[bit] = (float)((double)(d1 - d0) / sigma2);
    }
}

void or_llr_maxlog(const or_phy* p, const float* x_iq, int count, const double* sigma2, float* out)
{
    for (int i = 0; i < count; ++i)
        llr_maxlog_one(p, x_iq[2 * i], x_iq[2 * i + 1], sigma2[i], out + (size_t)i * p->bits_per_symbol);
}

/* single-precision complex helpers (std::complex<float> arithmetic) */
static void cf_mul(float ar, float ai, float br, float bi, float* rr, float* ri)
{
    *rr = ar * br - ai * bi;
    *ri = ar * bi + ai * br;
}

/* L:5331-5521 with a known noise variance (the demod half of decode_frame) */
void or_demod_frame(const or_phy* p, const float* frame_iq, double cfo_hz, double noise_var, float* out_llr)
{
    const int nfft = p->nfft, sc_n = p->active_sc;
    const long long pre_len = 2LL * p->pre_half_len;
    const long long frame_len = pre_len + (long long)p->num_symbols * (nfft + p->cp);
    float* fr = (float*)malloc(sizeof(float) * 2 * (size_t)frame_len);
    for (long long n = 0; n < frame_len; ++n) {
        const double a = -2.0 * kPi * cfo_hz * (double)n / p->rate;
        const float cr = (float)cos(a), ci = (float)sin(a);
        cf_mul(frame_iq[2 * n], frame_iq[2 * n + 1], cr, ci, &fr[2 * n], &fr[2 * n + 1]);
    }
    float* y = (float*)malloc(sizeof(float) * 2 * (size_t)p->num_symbols * (size_t)sc_n);
    float* shifted = (float*)malloc(sizeof(float) * 2 * (size_t)nfft);
    long long off = pre_len;
    for (int sym = 0; sym < p->num_symbols; ++sym) {
        or_fft_shifted(fr + 2 * (off + p->cp), nfft, shifted);
        for (int sc = 0; sc < sc_n; ++sc) {
            y[2 * ((size_t)sym * sc_n + sc)] = shifted[2 * p->used_indices[sc]];
            y[2 * ((size_t)sym * sc_n + sc) + 1] = shifted[2 * p->used_indices[sc] + 1];
        }
        off += nfft + p->cp;
    }
    /* LS pilot estimates, L:5389-5399 */
    float* hp = (float*)malloc(sizeof(float) * 2 * (size_t)(p->num_pilots > 0 ? p->num_pilots : 1) * (size_t)sc_n);
    for (int q = 0; q < p->num_pilots; ++q) {
        const int sym = p->pilot_symbols[q];
        for (int sc = 0; sc < sc_n; ++sc) {
            const float pr = p->pilot_grid[2 * ((size_t)q * sc_n + sc)], pi = p->pilot_grid[2 * ((size_t)q * sc_n + sc) + 1];
            float den = fnorm(pr, pi);
            if (den < 1e-9f) den = 1e-9f;
            float tr, ti;
            cf_mul(y[2 * ((size_t)sym * sc_n + sc)], y[2 * ((size_t)sym * sc_n + sc) + 1], pr, -pi, &tr, &ti);
            hp[2 * ((size_t)q * sc_n + sc)] = tr / den;
            hp[2 * ((size_t)q * sc_n + sc) + 1] = ti / den;
        }
    }
    /* interpolation (L:5401-5427), MMSE (L:5508-5521) */
    const int bps = p->bits_per_symbol;
    size_t i = 0;
    for (int di = 0; di < p->num_data; ++di) {
        const int sym = p->data_symbols[di];
        int hi = 0;
        while (hi + 1 < p->num_pilots && sym > p->pilot_symbols[hi + 1]) ++hi;
        int p0 = hi, p1 = (hi + 1 < p->num_pilots - 1) ? hi + 1 : p->num_pilots - 1;
        if (sym <= p->pilot_symbols[0]) { p0 = p1 = 0; }
        else if (sym >= p->pilot_symbols[p->num_pilots - 1]) { p0 = p1 = p->num_pilots - 1; }
        double alpha = 0.0;
        if (p0 != p1) alpha = (double)(sym - p->pilot_symbols[p0]) / (double)(p->pilot_symbols[p1] - p->pilot_symbols[p0]);
        const float w0 = (float)(1.0 - alpha), w1 = (float)alpha;
        for (int sc = 0; sc < sc_n; ++sc, ++i) {
            const float h0r = hp[2 * ((size_t)p0 * sc_n + sc)], h0i = hp[2 * ((size_t)p0 * sc_n + sc) + 1];
            const float h1r = hp[2 * ((size_t)p1 * sc_n + sc)], h1i = hp[2 * ((size_t)p1 * sc_n + sc) + 1];
            const float hr = h0r * w0 + h1r * w1, hi_ = h0i * w0 + h1i * w1;
            const float yr = y[2 * ((size_t)sym * sc_n + sc)], yi = y[2 * ((size_t)sym * sc_n + sc) + 1];
            float h2 = fnorm(hr, hi_);
            if (h2 < 1e-9f) h2 = 1e-9f;
            float tr, ti;
            cf_mul(yr, yi, hr, -hi_, &tr, &ti);
            const float den = h2 + (float)noise_var;
            const float er = tr / den, ei = ti / den;
            const double sigma2 = noise_var / (double)h2;
            llr_maxlog_one(p, er, ei, sigma2, out_llr + i * (size_t)bps);
        }
    }
    free(fr); free(y); free(shifted); free(hp);
}
