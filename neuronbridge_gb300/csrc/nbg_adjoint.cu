// nbg_adjoint.cu -- forward and adjoint step kernels of the differentiable
// recurrent LIF (C ABI and equations in include/nbg_adjoint.h).  The dense
// products (x W_in, s W_rec, dI W_rec^T and the weight gradients) are plain
// library GEMMs issued by the caller; everything elementwise of a step --
// leak, jump, threshold, surrogate, reset, refractory, readout weighting and
// the parameter gradients -- is one fused kernel each way.

#include <cuda_runtime.h>

#include "nbg_adjoint.h"
#include "nbg_common.cuh"

namespace {

__device__ __forceinline__ float surrogate(float x, float k) {
    const float d = 1.0f + k * fabsf(x);
    return 1.0f / (d * d);
}

__global__ void __launch_bounds__(256) k_lif_fwd(const float *__restrict__ I, float *__restrict__ v,
                                                 int *__restrict__ ref, float *__restrict__ s_out,
                                                 float *__restrict__ u_rec, unsigned char *__restrict__ m_rec,
                                                 float *__restrict__ vprev_rec, float *__restrict__ z, float c_t,
                                                 const float *__restrict__ alpha, const float *__restrict__ theta,
                                                 nbg_lif_grad_params p, int N, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int j = idx % N;
    const float vp = v[idx];
    const int rf = p.smooth ? 0 : ref[idx];
    const bool m = rf == 0;
    const float a = alpha[j], th = theta[j];
    const float u = m ? vp + a * (p.v_rest - vp) + I[idx] : p.v_reset;
    float s;
    if (p.smooth) s = 1.0f / (1.0f + expf(-p.slope * (u - th)));
    else s = u > th ? 1.0f : 0.0f;
    v[idx] = u - s * (u - p.v_reset);
    if (!p.smooth) ref[idx] = s > 0.0f ? p.t_ref : (rf > 0 ? rf - 1 : 0);
    s_out[idx] = s;
    if (u_rec) u_rec[idx] = u;
    if (m_rec) m_rec[idx] = m ? 1 : 0;
    if (vprev_rec) vprev_rec[idx] = vp;
    if (z) z[idx] = z[idx] + c_t * s;
}

__global__ void __launch_bounds__(256) k_lif_adj(const float *__restrict__ g_ext, const float *__restrict__ g_read,
                                                 float c_t, const float *__restrict__ u, const float *__restrict__ s,
                                                 const unsigned char *__restrict__ m, const float *__restrict__ vprev,
                                                 float *__restrict__ lam_v, float *__restrict__ dI,
                                                 float *__restrict__ g_theta, float *__restrict__ g_alpha,
                                                 const float *__restrict__ alpha, const float *__restrict__ theta,
                                                 nbg_lif_grad_params p, int N, int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int j = idx % N;
    const float uu = u[idx], ss = s[idx], lv = lam_v[idx];
    const float th = theta[j];
    const float dsdu = p.smooth ? p.slope * ss * (1.0f - ss) : surrogate(uu - th, p.slope);
    // dL/ds_t: recurrent path + readout + the reset's dependence on s
    float gs = c_t * g_read[idx] - lv * (uu - p.v_reset);
    if (g_ext) gs = gs + g_ext[idx];
    // dL/du_t through the spike and through v_t = u - s (u - V_reset)
    const float gu = gs * dsdu + lv * (1.0f - ss);
    const float gm = m[idx] ? gu : 0.0f;
    dI[idx] = gm;
    lam_v[idx] = gm * (1.0f - alpha[j]);
    g_theta[idx] = g_theta[idx] - gs * dsdu;
    g_alpha[idx] = g_alpha[idx] + gm * (p.v_rest - vprev[idx]);
}

__global__ void k_poisson(float *__restrict__ x, const float *__restrict__ rates, int T, int B, int C, float dt,
                          int seed, long long total) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int c = (int)(idx % C);
    const int bc = (int)(idx % ((long long)B * C));
    const int t = (int)(idx / ((long long)B * C));
    float r = rates[c];
    r = r > 0.0f ? r : 0.0f;
    float prob = r * dt * 0.001f;
    prob = prob < 1.0f ? prob : 1.0f;
    x[idx] = nbg_hash_uniform01(bc + seed, t) < prob ? 1.0f : 0.0f;
}

} // namespace

extern "C" {

nbg_status nbg_lif_forward_step(const float *I, float *v, int32_t *ref, float *s_out, float *u_rec, uint8_t *m_rec,
                                float *vprev_rec, float *z, float c_t, const float *alpha, const float *theta,
                                const nbg_lif_grad_params *p, int B, int N, void *stream) {
    if (!I || !v || !ref || !s_out || !alpha || !theta || !p || B <= 0 || N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_forward_step: bad arguments");
    const int total = B * N;
    k_lif_fwd<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(I, v, ref, s_out, u_rec, m_rec, vprev_rec, z,
                                                                      c_t, alpha, theta, *p, N, total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_lif_adjoint_step(const float *g_ext, const float *g_read, float c_t, const float *u, const float *s,
                                const uint8_t *m, const float *vprev, float *lam_v, float *dI, float *g_theta,
                                float *g_alpha, const float *alpha, const float *theta, const nbg_lif_grad_params *p,
                                int B, int N, void *stream) {
    if (!g_read || !u || !s || !m || !vprev || !lam_v || !dI || !g_theta || !g_alpha || !alpha || !theta || !p ||
        B <= 0 || N <= 0)
        return nbg_fail(NBG_ERR_INVALID, "nbg_lif_adjoint_step: bad arguments");
    const int total = B * N;
    k_lif_adj<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(g_ext, g_read, c_t, u, s, m, vprev, lam_v, dI,
                                                                      g_theta, g_alpha, alpha, theta, *p, N, total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

nbg_status nbg_poisson_inputs(float *x, const float *rates_hz, int T, int B, int C, float dt_ms, int seed,
                              void *stream) {
    if (!x || !rates_hz || T <= 0 || B <= 0 || C <= 0) return nbg_fail(NBG_ERR_INVALID, "nbg_poisson_inputs: bad arguments");
    const long long total = (long long)T * B * C;
    k_poisson<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, rates_hz, T, B, C, dt_ms, seed,
                                                                                  total);
    NBG_CUDA(cudaGetLastError());
    return NBG_OK;
}

} // extern "C"
