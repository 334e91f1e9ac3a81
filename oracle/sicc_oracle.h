/*
 * sicc_oracle.h — CPU restatement of the SICC receive-path arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA product
 * path: tests, the smoke check and the bench's CPU-baseline leg call it; the
 * product library never links it and has no CPU fallback.
 *
 * Every function cites the reference file:line it restates.  Citations are by
 * path inside the reference project:
 *   L   = source/cpp_cuda/uhd_cpp/src/uhd_ldpc_ofdm_link.cpp
 *   MB  = source/matlab/uhd_cpp/matlab/cpu_bp_osd_decode.m
 *
 * Parity pins (see tests/test_oracle_pins.py):
 *   - code construction, encoder, syndrome, flooding min-sum, FFT, max-log LLR,
 *     Schmidl-Cox sync and the full demod are checked against the reference's
 *     own CPU code compiled from its sources (oracle/_ref) and against the
 *     committed fixtures under tests/golden/ that it generated;
 *   - OSD restates MB, which has no runnable form here (no MATLAB): it is pinned
 *     by known-answer properties (maximum-likelihood equality at full order on
 *     small codes, noiseless recovery, codeword validity);
 *   - the layered schedule has no reference source anywhere; this file is its
 *     specification (row-sequential normalized min-sum, below).
 *
 * Floating-point rules: compiled with -ffp-contract=off; single-precision
 * routines perform exactly one IEEE operation per source operator, in the
 * stated order, so a device kernel that issues the same operations in the same
 * order reproduces them bit for bit.
 */
#ifndef SICC_ORACLE_H
#define SICC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_code or_code;

/* ---- code construction (L:2811-2945, L:2947-2997, L:2999-3011, L:3133-3160) ---- */
or_code* or_code_create(int n, int m, const int* row_ptr, const int* col_ind, int systematic_front);
void or_code_destroy(or_code* c);
int or_code_n(const or_code* c);
int or_code_m(const or_code* c);
int or_code_k(const or_code* c);
int or_code_is_accumulator(const or_code* c);
void or_code_info_cols(const or_code* c, int* out_info, int* out_pivot);
void or_encode(const or_code* c, const uint8_t* info, uint8_t* out_cw);
int or_syndrome_weight(const or_code* c, const uint8_t* bits);
/* systematic parity table [k][words], bit p of row i = parity bit p of encode(e_i).
 * Returns 0 on success, 1 when the code is not systematic-front. */
int or_systematic_parity(const or_code* c, uint64_t* out_table, int* out_words);
/* greedy row colouring: rows in ascending order take the smallest colour with no
 * shared variable; out_order = rows sorted by (colour, row); returns #colours. */
int or_greedy_color_order(const or_code* c, int* out_order, int* out_color_of_row);

/* ---- belief propagation ---- */
/* Flooding normalized min-sum exactly as L:3013-3094 (single precision). */
int or_nms_flooding_ref(const or_code* c, const float* llr, int max_iter, double normalization,
                        uint8_t* out_bits, float* out_app, int* out_iter);

/* Generalised single-precision flooding: offset beta, MB-style variable-message
 * damping (MB:180-183), best-syndrome tracking (MB:160-171).  With beta = 0 and
 * damping = 0 it performs the same operations as L:3013-3094. */
int or_nms_flooding_f32(const or_code* c, const float* llr, int max_iter, float alpha, float beta,
                        float damping, uint8_t* out_bits, float* out_app, float* out_best_app,
                        int* out_iter, int* out_best_w);

/* Row-sequential layered normalized min-sum (single precision).  row_order may be
 * NULL (natural order).  Per row, in the row's CSR edge order:
 *   q_e   = app[v_e] - R_e
 *   min1/min2/first-argmin of |q_e| (strict <), sign bits (q_e < 0)
 *   mag_j = alpha*min_j            (beta == 0)
 *   mag_j = max(alpha*min_j - beta, 0)   (beta > 0)
 *   R_e   = sign(prod other q) * (e == argmin ? mag2 : mag1)
 *   app[v_e] = q_e + R_e
 * After each full pass: hard = app < 0, syndrome weight w; if w < best then the
 * best posterior is this app; stop when w == 0.  At least one pass always runs.
 * Returns 1 when the final syndrome is zero. */
int or_nms_layered_f32(const or_code* c, const int* row_order, const float* llr, int max_iter,
                       float alpha, float beta, uint8_t* out_bits, float* out_app, float* out_best_app,
                       int* out_iter, int* out_best_w);
/* The same schedule in double precision (the FP64 reference for posterior LLRs). */
int or_nms_layered_f64(const or_code* c, const int* row_order, const float* llr, int max_iter,
                       double alpha, double beta, uint8_t* out_bits, double* out_app, int* out_iter);

/* ---- ordered-statistics decoding (MB:187-305) ---- */
/* G = [I_k | P] from the systematic parity table.  Returns the number of tests
 * run; writes the decoded codeword (original positions), the winning metric and
 * the index of the winning test (0 = hard decision of the most reliable basis). */
int or_osd(int n, int k, const uint64_t* parity_table, int parity_words, const float* llr, int order,
           int max_flip_positions, int max_tests, uint8_t* out_code, float* out_metric,
           int* out_best_test);

/* Batch BP -> OSD decode: `schedule` 0 = the reference's BP + OSD decoder
 * (cpu_bp_osd_decode.m, MB:55-62: flooding min-sum, which without damping or
 * offset performs the operations of L:3013-3094), 3 = row-sequential layered.
 * Frames whose syndrome is not zero go to OSD when osd_order >= 0, on the
 * posterior of the lowest syndrome weight seen (MB's bestAppLlr, MB:160-171;
 * the channel LLRs when no iteration improved on them) for both schedules.
 * Writes the first k decoded bits of each codeword and whether OSD ran.
 * Returns the number of OSD frames. */
int or_bp_osd_batch(const or_code* c, const uint64_t* parity_table, int parity_words, const float* llrs, int count,
                    int schedule, int max_iter, float alpha, int osd_order, int osd_max_flip, int osd_max_tests,
                    uint8_t* out_info, uint8_t* out_used_osd);

/* ---- OFDM receive (L:3788-3859, L:5214-5329, L:5331-5521, L:2552-2568) ---- */
typedef struct or_phy {
    int nfft, cp, num_symbols, active_sc, pre_half_len, bits_per_symbol;
    int num_pilots, num_data;
    double rate, sync_threshold;
    const int* used_indices;   /* [active_sc], shifted-grid bins */
    const int* pilot_symbols;  /* [num_pilots] */
    const int* data_symbols;   /* [num_data] */
    const float* preamble;     /* [2*pre_half_len] interleaved re,im */
    const float* pilot_grid;   /* [num_pilots][active_sc] interleaved */
    const float* constellation;/* [2^bps] interleaved, index bits MSB-first */
} or_phy;

void or_fft_shifted(const float* time_iq, int nfft, float* out_shifted_iq);
/* 1 found, 2 incomplete frame, 0 not found */
int or_sync_earliest(const or_phy* p, const float* buf_iq, long long count, long long max_search,
                     long long* out_start, double* out_coarse, double* out_fine, double* out_cfo_hz);
/* Demodulates one frame starting at sample 0 with known noise variance:
 * CFO derotation, per-symbol FFT, LS pilot estimate + linear interpolation,
 * MMSE equalisation, exhaustive max-log LLRs.  out_llr: [num_data*active_sc*bps]. */
void or_demod_frame(const or_phy* p, const float* frame_iq, double cfo_hz, double noise_var, float* out_llr);
void or_llr_maxlog(const or_phy* p, const float* x_iq, int count, const double* sigma2, float* out);

#ifdef __cplusplus
}
#endif
#endif
