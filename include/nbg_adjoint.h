/*
 * nbg_adjoint.h -- fused elementwise kernels of a differentiable recurrent
 * voltage-jump LIF network, forward step and hand-written adjoint step.
 * Pointers are device pointers; `stream` is a cudaStream_t (NULL = default).
 *
 * There is no counterpart in the reference: it has no gradient path.  The
 * neuron is the reference's voltage-jump LIF (TimeDrivenLIF_Voltage_jump.cpp
 * :49-113) written as a differentiable recurrence, one step of dt:
 *
 *   m_t = (ref_{t-1} == 0)                                  integrating
 *   u_t = m_t ? v_{t-1} + alpha (V_rest - v_{t-1}) + I_t : V_reset
 *   s_t = H(u_t - theta)        spiking mode   (surrogate 1/(1+k|u-theta|)^2)
 *       = sigmoid(k (u_t - theta))  smoothed mode (exact derivative)
 *   v_t = u_t - s_t (u_t - V_reset)
 *   ref_t = s_t ? t_ref : max(ref_{t-1} - 1, 0)             (spiking mode)
 *   z    += c_t s_t                                         readout weight
 *
 * with I_t = x_t W_in + s_{t-1} W_rec computed by the caller, alpha = dt/tau
 * and theta per neuron.  The adjoint step receives g_ext = dL/ds_t from the
 * recurrent path (dI_{t+1} W_rec^T), adds c_t * g_read (the readout term),
 * and returns dI_t = dL/dI_t, the running lambda_v = dL/dv_{t-1}, and
 * accumulates dL/dtheta and dL/dalpha per (instance, neuron).
 */
#ifndef NBG_ADJOINT_H
#define NBG_ADJOINT_H

#include "nbg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float v_rest, v_reset, slope;
    int t_ref;  /* refractory steps (spiking mode) */
    int smooth; /* 0: Heaviside spikes + fast-sigmoid surrogate; 1: sigmoid spikes */
} nbg_lif_grad_params;

/* One forward step over B x N neurons.  u_rec, m_rec, vprev_rec (optional,
 * NULL to skip) record u_t, m_t and v_{t-1} for the adjoint; s_out receives
 * s_t; z += c_t * s_t. */
nbg_status nbg_lif_forward_step(const float *I, float *v, int32_t *ref, float *s_out, float *u_rec, uint8_t *m_rec,
                                float *vprev_rec, float *z, float c_t, const float *alpha, const float *theta,
                                const nbg_lif_grad_params *p, int B, int N, void *stream);

/* Spike-driven forward step (spiking mode only): I_t = xi_t + the sum, in
 * ascending neuron order, of the rows of w_rec (N x N, row = pre) listed in
 * spk_in/cnt_in (row b's spikes of step t-1: spk_in[b*N .. b*N + cnt_in[b]]),
 * then the step of nbg_lif_forward_step; writes row b's ascending spike list
 * of step t to spk_out/cnt_out.  N <= 2048.  Same equations as the dense form
 * with s_{t-1} W_rec as a gather-sum over the spikes. */
nbg_status nbg_lif_forward_step_sparse(const float *xi, const float *w_rec, const int32_t *spk_in,
                                       const int32_t *cnt_in, int32_t *spk_out, int32_t *cnt_out, float *v,
                                       int32_t *ref, float *s_out, float *u_rec, uint8_t *m_rec, float *vprev_rec,
                                       float *z, float c_t, const float *alpha, const float *theta,
                                       const nbg_lif_grad_params *p, int B, int N, void *stream);

/* Ascending spike list of every row of the 0/1 matrix s (B x N). */
/* L steps of nbg_lif_forward_step_sparse in one launch (rows are
 * independent: each CTA runs its row through the L steps).  xi: L x B x N
 * (x_t W_in of the L steps); spk/cnt: in, row b's ascending spike list of the
 * step before the first, out, of the last step.  Optional outputs (NULL to
 * skip), each L x B x N: s_out (s_t), u_rec, m_rec, vprev_rec; s_last (B x N,
 * the last step's s); z += c[l] * s_t with c the L readout coefficients.
 * Results are identical to L calls of nbg_lif_forward_step_sparse. */
nbg_status nbg_lif_forward_segment_sparse(const float *xi, const float *w_rec, int32_t *spk, int32_t *cnt, float *v,
                                          int32_t *ref, float *s_out, float *s_last, float *u_rec, uint8_t *m_rec,
                                          float *vprev_rec, float *z, const float *c, const float *alpha,
                                          const float *theta, const nbg_lif_grad_params *p, int L, int B, int N,
                                          void *stream);
/* nbg_lif_forward_segment_sparse with the input term as a gather too: x is
 * L x B x C (the segment's inputs), w_in C x N; at each step row b's input
 * current starts from the sum, in ascending channel order, of x_t[b][c] *
 * w_in[c] over its nonzero inputs, then adds the recurrent rows.  With spike
 * inputs (x in {0, 1}) this is a gather-sum like the recurrent one, and no
 * L x B x N product of the inputs is formed.  The lists live in shared
 * memory, (2N + 2C) * 4 bytes; larger sizes than 200 KiB are rejected. */
nbg_status nbg_lif_forward_segment_gather(const float *x, const float *w_in, int C, const float *w_rec, int32_t *spk,
                                          int32_t *cnt, float *v, int32_t *ref, float *s_out, float *s_last,
                                          float *u_rec, uint8_t *m_rec, float *vprev_rec, float *z, const float *c,
                                          const float *alpha, const float *theta, const nbg_lif_grad_params *p,
                                          int L, int B, int N, void *stream);
nbg_status nbg_spike_lists(const float *s, int32_t *spk, int32_t *cnt, int B, int N, void *stream);

/* One adjoint step (reverse time).  g_ext may be NULL (last step). */
nbg_status nbg_lif_adjoint_step(const float *g_ext, const float *g_read, float c_t, const float *u, const float *s,
                                const uint8_t *m, const float *vprev, float *lam_v, float *dI, float *g_theta,
                                float *g_alpha, const float *alpha, const float *theta, const nbg_lif_grad_params *p,
                                int B, int N, void *stream);

/* The recurrent product of the adjoint, g_ext = dI_{t+1} W_rec^T, on the
 * tensor cores in split BF16 (x = x_hi + x_lo, three BF16 products
 * accumulated in FP32, about 16 mantissa bits of each operand), for
 * B = 128 rows and N a multiple of 128:
 *   nbg_adjoint_rec_prepare   W_rec (N x N FP32) -> w_hi, w_lo (N x N BF16
 *                             each, blocked; once per backward)
 *   nbg_lif_adjoint_step_split  nbg_lif_adjoint_step with g_ext the sum, in
 *                             order, of n_parts consecutive B x N partials
 *                             (NULL: none), also writing dI as dI_hi, dI_lo
 *                             (B x N BF16 each, blocked)
 *   nbg_adjoint_rec_grad      g_parts[split][B][N] = the split-K partials of
 *                             dI W_rec^T from those operands; *err gets 4 if
 *                             a bounded wait of the kernel gave up
 * There is no counterpart in the reference (it has no gradient path). */
nbg_status nbg_adjoint_rec_prepare(const float *w_rec, void *w_hi, void *w_lo, int N, void *stream);
nbg_status nbg_lif_adjoint_step_split(const float *g_parts, int n_parts, const float *g_read, float c_t,
                                      const float *u, const float *s, const uint8_t *m, const float *vprev,
                                      float *lam_v, float *dI, void *dI_hi, void *dI_lo, float *g_theta,
                                      float *g_alpha, const float *alpha, const float *theta,
                                      const nbg_lif_grad_params *p, int B, int N, void *stream);
nbg_status nbg_adjoint_rec_grad(const void *w_hi, const void *w_lo, const void *dI_hi, const void *dI_lo,
                                float *g_parts, int split, int B, int N, int *err, void *stream);

/* One adjoint step t in one launch, N >= 512 (a multiple of 128), B = 128:
 * the recurrent term dI_{t+1} W_rec^T on the tensor cores (as
 * nbg_adjoint_rec_grad, from dI_hi_in / dI_lo_in) and the step of
 * nbg_lif_adjoint_step_split on it, which writes dI_t: the split BF16
 * operand of the next step's product into dI_hi_out / dI_lo_out (the in and
 * out operand buffers must differ), FP32 into dI unless dI is NULL, and,
 * unless dT_hi is NULL, dI_t^T split into dT_hi / dT_lo as columns
 * k_off .. k_off + 127 of the N x k_cols blocked matrix that
 * nbg_adjoint_blocked_t would make of it (k_off a multiple of 128, k_cols
 * of 64): the weight gradients' operand without a transpose.  With dI_hi_in
 * / dI_lo_in all zeros (the last step of the run) the results equal
 * nbg_lif_adjoint_step_split's without a recurrent term (a zero may differ
 * in sign).  The split-K partials never leave the chip: the 8
 * CTAs of a cluster that share a 128-row tile reduce them through
 * distributed shared memory, in the same order as the two-launch form, so
 * the results are identical to it.  A bounded wait that gives up sets
 * kUmmaTimeout (4) in *err and the step's results are invalid.  No
 * counterpart in the reference (the reference has no adjoint). */
nbg_status nbg_lif_adjoint_step_fused(const void *w_hi, const void *w_lo, const void *dI_hi_in, const void *dI_lo_in,
                                      void *dI_hi_out, void *dI_lo_out, const float *g_read, float c_t,
                                      const float *u, const float *s, const uint8_t *m, const float *vprev,
                                      float *lam_v, float *dI, float *g_theta, float *g_alpha, const float *alpha,
                                      const float *theta, const nbg_lif_grad_params *p, int B, int N, void *dT_hi,
                                      void *dT_lo, int64_t k_off, int64_t k_cols, int *err, void *stream);

/* The recurrent weight gradient of a checkpoint segment on the tensor cores,
 * dW_rec += sum over its L steps of S_{t-1}^T dI_t, in three calls:
 *   nbg_adjoint_blocked_t   src [L][B][R] FP32 -> the R_pad x (L*B) matrix,
 *                           row r, column l*B + b, blocked BF16, rows R ..
 *                           R_pad - 1 zero; split into hi and lo when lo is
 *                           not NULL (else the values must be exact in BF16,
 *                           as spikes are).  R_pad >= R a multiple of 128,
 *                           L*B a multiple of 64.
 *   nbg_adjoint_wgrad       part[split][Nc][M] = split-K partials of
 *                           (a_hi + a_lo)(b + b_lo)^T without the lo x lo
 *                           term (b_lo NULL: b exact), a: M x K, b: Nc x K (from
 *                           nbg_adjoint_blocked_t), M a multiple of 128, Nc
 *                           of 256, K of 64; *err gets 4 if a bounded wait
 *                           gave up
 *   nbg_adjoint_reduce_add  g[e] += sum over q, in order, of part[q * stride
 *                           + e], e < count (stride >= count: the partials of
 *                           a padded Nc keep their padding rows after the
 *                           gradient's)
 * With a = dI^T (split) and b = S^T (or X^T, split) part[q] is laid out as
 * dW_rec (or dW_in): row = presynaptic neuron (or input channel).  A row
 * count that is not a multiple of the tile (Nc of 256) is padded with zero
 * rows by nbg_adjoint_blocked_t; the padding rows of part are not added. */
nbg_status nbg_adjoint_blocked_t(const float *src, int L, int B, int R, int R_pad, void *hi, void *lo,
                                 void *stream);
nbg_status nbg_adjoint_wgrad(const void *a_hi, const void *a_lo, const void *b, const void *b_lo, int M, int Nc,
                             int K, float *part, int split, int *err, void *stream);
nbg_status nbg_adjoint_reduce_add(float *g, const float *part, int split, int64_t count, int64_t stride,
                                  void *stream);

/* C = A B for the readout's small products (B x N by N x O, its transposes):
 * element (r, c) of A at A[r * a_rs + c * a_cs], likewise B; C is M x N row
 * major, FP32 sums.  K < 64: one thread per output, k ascending; K >= 64: one
 * warp per output, lane l adding k = l, l + 32, ... in order and the 32 lane
 * sums added in a fixed tree.  The order depends only on K, so results do
 * not depend on the launch.  No counterpart in the reference. */
nbg_status nbg_small_gemm(const float *A, int a_rs, int a_cs, const float *B, int b_rs, int b_cs, float *C, int M,
                          int N, int K, void *stream);

/* Poisson input spikes x[t][b][c] in {0, 1}: channel c fires with
 * probability min(1, rate_c * dt * 1e-3) from the PoissonRate hash of
 * (seed-offset index b*C + c + seed, step t). */
nbg_status nbg_poisson_inputs(float *x, const float *rates_hz, int T, int B, int C, float dt_ms, int seed,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NBG_ADJOINT_H */
