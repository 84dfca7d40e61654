// tsph_gnn.cu -- the learned surrogate's graph network on the device:
// forward, backward, Adam (no counterpart in the reference, which has no
// learned part).
//
// Network (hidden width H = 64, two message-passing layers, SiLU):
//   node input  x_i = (u_i / U, v_i / U, (rho_i - rho0) / S, wall_i)
//   edge input  e_ij = (dx / h, dy / h, |r| / h, (u_i - u_j) / U, (v_i - v_j) / U)
//   encoder     h = SiLU(A0 x + a0)
//   layer       P = h Wp^T, Q = h Wq^T;  S_i = sum_j SiLU(P_i + Q_j + We e_ij + be)
//               m_i = W2 S_i + deg_i b2;  h <- h + Wn2 SiLU(Wn1 [h, m] + bn1) + bn2
//   decoder     y = Wd h + bd
// The edge MLP's first layer is split into the two per-node products P, Q
// (64 x 64 per node instead of 133 x 64 per edge) and its second layer
// commutes with the neighbour sum, so the per-edge work is one 64-wide
// activation.  The graph is the SPH pair set (tsph_export_graph), symmetric,
// so the backward pass gathers too (atomic-free): node n collects
// dz_nj = dS_n SiLU'(z_nj) for dP_n and dz_jn = dS_j SiLU'(z_jn) for dQ_n.
// Weight gradients are reduced per block into partial sums and then summed
// in a fixed order (deterministic).
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tsph.h"
#include "tsph_engine.h"

namespace tsph {
namespace {

constexpr int H = 64, NL = 2, NIN = 4, EIN = 5, NOUT = 3;
constexpr int kGB = 256;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// flat parameter layout (the order of oracle/gnn_oracle.py param_shapes)
struct Layout {
    int A0, a0, Wp[NL], Wq[NL], We[NL], be[NL], W2[NL], b2[NL], Wn1[NL], bn1[NL], Wn2[NL],
        bn2[NL], Wd, bd, total;
    Layout() {
        int o = 0;
        auto take = [&](int n) {
            const int r = o;
            o += n;
            return r;
        };
        A0 = take(H * NIN);
        a0 = take(H);
        for (int l = 0; l < NL; l++) {
            Wp[l] = take(H * H);
            Wq[l] = take(H * H);
            We[l] = take(H * EIN);
            be[l] = take(H);
            W2[l] = take(H * H);
            b2[l] = take(H);
            Wn1[l] = take(H * 2 * H);
            bn1[l] = take(H);
            Wn2[l] = take(H * H);
            bn2[l] = take(H);
        }
        Wd = take(NOUT * H);
        bd = take(NOUT);
        total = o;
    }
};

struct GraphDev {
    const double2 *pos;
    const float2 *vel;
    const float *srho, *wall;
    const int32_t *deg, *nbr;
    int n, K;
    float inv_h, inv_U, inv_S;
};

// the edge input of (i, j): the position difference in FP64, then FP32
__device__ __forceinline__ void edge_in(const GraphDev &G, double2 pi, float2 vi, int j,
                                        float e[EIN]) {
    const double2 pj = G.pos[j];
    const float2 vj = G.vel[j];
    const float dx = (float)(pi.x - pj.x), dy = (float)(pi.y - pj.y);
    e[0] = dx * G.inv_h;
    e[1] = dy * G.inv_h;
    e[2] = sqrtf(fmaf(dx, dx, dy * dy)) * G.inv_h;
    e[3] = (vi.x - vj.x) * G.inv_U;
    e[4] = (vi.y - vj.y) * G.inv_U;
}

// a warp's edges are computed one per lane (slots k0 + lane), then broadcast
struct EdgeLane {
    int j;
    float e[EIN];
};
__device__ __forceinline__ EdgeLane edge_lane(const GraphDev &G, int i, double2 pi, float2 vi,
                                              int k) {
    EdgeLane r;
    r.j = 0;
#pragma unroll
    for (int q = 0; q < EIN; q++) r.e[q] = 0.f;
    if (k < G.deg[i]) {
        r.j = G.nbr[(size_t)i * G.K + k];
        edge_in(G, pi, vi, r.j, r.e);
    }
    return r;
}

// encoder: thread per (node, channel); z0 kept for the backward pass
__global__ void k_encode(GraphDev G, const float *__restrict__ A0, const float *__restrict__ a0,
                         float *__restrict__ z0, float *__restrict__ h) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G.n * H) return;
    const int i = t / H, c = t - i * H;
    const float2 v = G.vel[i];
    const float x[NIN] = {v.x * G.inv_U, v.y * G.inv_U, G.srho[i] * G.inv_S, G.wall[i]};
    float z = a0[c];
#pragma unroll
    for (int k = 0; k < NIN; k++) z = fmaf(A0[c * NIN + k], x[k], z);
    z0[t] = z;
    h[t] = silu(z);
}

// Y[n][m] = epi( sum_k X[n][k] W(m, k) + b[m] + deg[n] b2[m] ), X = [X1 | X2]
// (K1 + K2 <= 128 columns), W(m, k) = W[m * wm + k * wk] (W or its
// transpose), M = 64 or 128 outputs.  Epilogue, in order: keep the
// pre-activation in `pre`, SiLU (act), times SiLU'(aux[n][m]) (for the
// backward pass), + res[n][m], and = or += into Y.  A block takes 16 nodes;
// W is staged transposed in shared memory.
struct LinArgs {
    const float *X1, *X2;
    int K1, K2;
    int ld1, ld2;  // row strides of X1, X2
    const float *W;
    int wm, wk;
    const float *b, *b2;
    const int32_t *deg;
    float *pre;
    int act;
    const float *aux;
    const float *res;
    float *Y;
    int accumulate;
    int n;
};

constexpr int kLinTN = 16;
constexpr int kLinBlocks = 152 * 4;  // persistent: W is staged once per block

template <int M>
__global__ void __launch_bounds__(kGB) k_linear(LinArgs a) {
    __shared__ float Ws[128 * 64];
    __shared__ float Xs[kLinTN * 128];
    const int K = a.K1 + a.K2;
    const int tid = threadIdx.x;
    // stage W transposed (Ws[k][m]), reading it in its own order (coalesced)
    if (a.wk == 1) {
        for (int e = tid; e < K * M; e += kGB) {
            const int m = e / K, k = e - m * K;
            Ws[k * M + m] = a.W[m * a.wm + k];
        }
    } else {
        for (int e = tid; e < K * M; e += kGB) {
            const int k = e / M, m = e - k * M;
            Ws[k * M + m] = a.W[m * a.wm + k * a.wk];
        }
    }
    constexpr int G = kGB / M;          // node groups
    constexpr int PER = kLinTN / G;     // nodes per thread
    const int m = tid % M, grp = tid / M;
    for (int n0 = blockIdx.x * kLinTN; n0 < a.n; n0 += gridDim.x * kLinTN) {
        __syncthreads();
        for (int e = tid; e < kLinTN * K; e += kGB) {
            const int r = e / K, k = e - r * K;
            const int n = n0 + r;
            float v = 0.f;
            if (n < a.n) v = k < a.K1 ? a.X1[(size_t)n * a.ld1 + k] : a.X2[(size_t)n * a.ld2 + (k - a.K1)];
            Xs[e] = v;
        }
        __syncthreads();
        float acc[PER];
#pragma unroll
        for (int q = 0; q < PER; q++) acc[q] = 0.f;
        for (int k = 0; k < K; k++) {
            const float w = Ws[k * M + m];
#pragma unroll
            for (int q = 0; q < PER; q++) acc[q] = fmaf(Xs[(grp + q * G) * K + k], w, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int n = n0 + grp + q * G;
            if (n >= a.n) continue;
            float y = acc[q];
            if (a.b) y += a.b[m];
            if (a.b2) y = fmaf((float)a.deg[n], a.b2[m], y);
            const size_t o = (size_t)n * M + m;
            if (a.pre) a.pre[o] = y;
            if (a.act) y = silu(y);
            if (a.aux) y *= dsilu(a.aux[o]);
            if (a.res) y += a.res[o];
            if (a.accumulate) y += a.Y[o];
            a.Y[o] = y;
        }
    }
}

// decoder y = Wd h + bd (3 outputs): thread per (node, output)
__global__ void k_decode(const float *__restrict__ h, int n, const float *__restrict__ Wd,
                         const float *__restrict__ bd, float *__restrict__ y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * NOUT) return;
    const int i = t / NOUT, o = t - i * NOUT;
    float s = bd[o];
    const float *hi = h + (size_t)i * H;
#pragma unroll 8
    for (int k = 0; k < H; k++) s = fmaf(Wd[o * H + k], hi[k], s);
    y[t] = s;
}

// edge aggregation, warp per node, lane c holds channels c and c + 32:
// S_i = sum_j SiLU(P_i + Q_j + We e_ij + be)
__global__ void __launch_bounds__(kGB) k_edge_forward(GraphDev G, const float *__restrict__ P,
                                                      const float *__restrict__ Q,
                                                      const float *__restrict__ We,
                                                      const float *__restrict__ be,
                                                      float *__restrict__ S) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= G.n) return;
    float w0[EIN], w1[EIN];
#pragma unroll
    for (int k = 0; k < EIN; k++) {
        w0[k] = We[lane * EIN + k];
        w1[k] = We[(lane + 32) * EIN + k];
    }
    const float p0 = P[(size_t)i * H + lane] + be[lane];
    const float p1 = P[(size_t)i * H + lane + 32] + be[lane + 32];
    float s0 = 0.f, s1 = 0.f;
    const int d = G.deg[i];
    const double2 pi = G.pos[i];
    const float2 vi = G.vel[i];
    for (int k0 = 0; k0 < d; k0 += 32) {
        const EdgeLane mine = edge_lane(G, i, pi, vi, k0 + lane);
        const int cnt = min(32, d - k0);
        for (int t = 0; t < cnt; t++) {
            const int j = __shfl_sync(0xffffffffu, mine.j, t);
            float z0 = p0 + Q[(size_t)j * H + lane], z1 = p1 + Q[(size_t)j * H + lane + 32];
#pragma unroll
            for (int q = 0; q < EIN; q++) {
                const float eq = __shfl_sync(0xffffffffu, mine.e[q], t);
                z0 = fmaf(w0[q], eq, z0);
                z1 = fmaf(w1[q], eq, z1);
            }
            s0 += silu(z0);
            s1 += silu(z1);
        }
    }
    S[(size_t)i * H + lane] = s0;
    S[(size_t)i * H + lane + 32] = s1;
}

// edge backward, warp per node n (symmetric graph):
//   dP_n = sum_{j in N(n)} dS_n SiLU'(z_nj),  dQ_n = sum_{j in N(n)} dS_j SiLU'(z_jn)
// and this warp's share of dWe = sum dz_nj e_nj^T, dbe = sum dz_nj, written
// to part[warp][H][EIN + 1] for the ordered reduction
__global__ void __launch_bounds__(kGB) k_edge_backward(GraphDev G, const float *__restrict__ P,
                                                       const float *__restrict__ Q,
                                                       const float *__restrict__ We,
                                                       const float *__restrict__ be,
                                                       const float *__restrict__ dS,
                                                       float *__restrict__ dP,
                                                       float *__restrict__ dQ,
                                                       float *__restrict__ part) {
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int n = wid;
    float gw0[EIN + 1], gw1[EIN + 1];
#pragma unroll
    for (int q = 0; q <= EIN; q++) gw0[q] = gw1[q] = 0.f;
    if (n < G.n) {
        float w0[EIN], w1[EIN];
#pragma unroll
        for (int k = 0; k < EIN; k++) {
            w0[k] = We[lane * EIN + k];
            w1[k] = We[(lane + 32) * EIN + k];
        }
        const float b0 = be[lane], b1 = be[lane + 32];
        const float pn0 = P[(size_t)n * H + lane], pn1 = P[(size_t)n * H + lane + 32];
        const float qn0 = Q[(size_t)n * H + lane], qn1 = Q[(size_t)n * H + lane + 32];
        const float ds0 = dS[(size_t)n * H + lane], ds1 = dS[(size_t)n * H + lane + 32];
        float dp0 = 0.f, dp1 = 0.f, dq0 = 0.f, dq1 = 0.f;
        const int d = G.deg[n];
        const double2 pn = G.pos[n];
        const float2 vn = G.vel[n];
        for (int k0 = 0; k0 < d; k0 += 32) {
            const EdgeLane mine = edge_lane(G, n, pn, vn, k0 + lane);
            const int cnt = min(32, d - k0);
            for (int tt = 0; tt < cnt; tt++) {
                const int j = __shfl_sync(0xffffffffu, mine.j, tt);
                float e[EIN];  // e_nj; e_jn = (-e0, -e1, e2, -e3, -e4)
#pragma unroll
                for (int q = 0; q < EIN; q++) e[q] = __shfl_sync(0xffffffffu, mine.e[q], tt);
                float a0 = pn0 + Q[(size_t)j * H + lane] + b0, a1 = pn1 + Q[(size_t)j * H + lane + 32] + b1;
                float c0 = P[(size_t)j * H + lane] + qn0 + b0, c1 = P[(size_t)j * H + lane + 32] + qn1 + b1;
#pragma unroll
                for (int q = 0; q < EIN; q++) {
                    const float sgn = (q == 2) ? 1.f : -1.f;
                    a0 = fmaf(w0[q], e[q], a0);
                    a1 = fmaf(w1[q], e[q], a1);
                    c0 = fmaf(w0[q], sgn * e[q], c0);
                    c1 = fmaf(w1[q], sgn * e[q], c1);
                }
                const float dz0 = ds0 * dsilu(a0), dz1 = ds1 * dsilu(a1);
                dp0 += dz0;
                dp1 += dz1;
#pragma unroll
                for (int q = 0; q < EIN; q++) {
                    gw0[q] = fmaf(dz0, e[q], gw0[q]);
                    gw1[q] = fmaf(dz1, e[q], gw1[q]);
                }
                gw0[EIN] += dz0;
                gw1[EIN] += dz1;
                dq0 = fmaf(dS[(size_t)j * H + lane], dsilu(c0), dq0);
                dq1 = fmaf(dS[(size_t)j * H + lane + 32], dsilu(c1), dq1);
            }
        }
        dP[(size_t)n * H + lane] = dp0;
        dP[(size_t)n * H + lane + 32] = dp1;
        dQ[(size_t)n * H + lane] = dq0;
        dQ[(size_t)n * H + lane + 32] = dq1;
    }
    // block-level sum of the warps' weight-gradient shares, one partial per block
    __shared__ float red[kGB / 32][H * (EIN + 1)];
    const int w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q <= EIN; q++) {
        red[w][lane * (EIN + 1) + q] = gw0[q];
        red[w][(lane + 32) * (EIN + 1) + q] = gw1[q];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < H * (EIN + 1); e += blockDim.x) {
        float s = 0.f;
        for (int ww = 0; ww < kGB / 32; ww++) s += red[ww][e];
        part[(size_t)blockIdx.x * H * (EIN + 1) + e] = s;
    }
}

// weight gradients dW[m][k] = sum_n dY[n][m] X[n][k] (X = [X1 | X2]), with
// optional extra columns X = 1 (bias gradient) and X = deg[n] (degree-bias
// gradient): each block sums a contiguous range of nodes into its partial
// part[block][M][Kt], the reduction adds the partials in block order
struct WgArgs {
    const float *dY;
    int ldy, M;
    const float *X1, *X2;
    int K1, K2, ld1, ld2;
    int bias_col;
    const int32_t *deg;
    int n;
    float *part;
};

constexpr int kWgBlocks = 304;  // 2 per SM
constexpr int kWgTN = 16;
constexpr int kWgMaxOut = 64 * 130;

__global__ void __launch_bounds__(kGB) k_wgrad(WgArgs a) {
    __shared__ float dYs[kWgTN * 64];
    __shared__ float Xs[kWgTN * 130];
    const int K = a.K1 + a.K2;
    const int Kt = K + (a.bias_col ? 1 : 0) + (a.deg ? 1 : 0);
    const int nout = a.M * Kt;
    constexpr int PER = (kWgMaxOut + kGB - 1) / kGB;
    float acc[PER];
#pragma unroll
    for (int q = 0; q < PER; q++) acc[q] = 0.f;
    const int chunk = (a.n + gridDim.x - 1) / gridDim.x;
    const int nb = blockIdx.x * chunk, ne = min(a.n, nb + chunk);
    for (int t0 = nb; t0 < ne; t0 += kWgTN) {
        __syncthreads();
        for (int e = threadIdx.x; e < kWgTN * a.M; e += kGB) {
            const int r = e / a.M, m = e - r * a.M;
            const int n = t0 + r;
            dYs[e] = n < ne ? a.dY[(size_t)n * a.ldy + m] : 0.f;
        }
        for (int e = threadIdx.x; e < kWgTN * Kt; e += kGB) {
            const int r = e / Kt, k = e - r * Kt;
            const int n = t0 + r;
            float v = 0.f;
            if (n < ne) {
                if (k < a.K1) v = a.X1[(size_t)n * a.ld1 + k];
                else if (k < K) v = a.X2[(size_t)n * a.ld2 + (k - a.K1)];
                else if (a.bias_col && k == K) v = 1.f;
                else v = (float)a.deg[n];
            }
            Xs[e] = v;
        }
        __syncthreads();
        const int rows = min(kWgTN, ne - t0);
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int o = threadIdx.x + q * kGB;
            if (o >= nout) break;
            const int m = o / Kt, k = o - m * Kt;
            float s = acc[q];
            for (int r = 0; r < rows; r++) s = fmaf(dYs[r * a.M + m], Xs[r * Kt + k], s);
            acc[q] = s;
        }
    }
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int o = threadIdx.x + q * kGB;
        if (o < nout) a.part[(size_t)blockIdx.x * nout + o] = acc[q];
    }
}

// ordered sum of the partials into the gradient vector: column k < K of row
// m -> g[w_off + m * K + k], the bias column -> g[b_off + m], the degree
// column -> g[d_off + m]; `accumulate` adds to what is there
__global__ void k_wgrad_reduce(const float *__restrict__ part, int nparts, int M, int K,
                               int bias_col, int deg_col, float *__restrict__ g, int w_off,
                               int b_off, int d_off, int accumulate) {
    const int Kt = K + bias_col + deg_col;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= M * Kt) return;
    float s = 0.f;
    for (int b = 0; b < nparts; b++) s += part[(size_t)b * M * Kt + o];
    const int m = o / Kt, k = o - m * Kt;
    int dst;
    if (k < K) dst = w_off + m * K + k;
    else if (bias_col && k == K) dst = b_off + m;
    else dst = d_off + m;
    g[dst] = accumulate ? g[dst] + s : s;
}

// dWe (H x EIN) and dbe (H) from the edge-backward partials [blocks][H][EIN+1]
__global__ void k_edge_wgrad_reduce(const float *__restrict__ part, int nparts,
                                    float *__restrict__ g, int we_off, int be_off) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= H * (EIN + 1)) return;
    float s = 0.f;
    for (int b = 0; b < nparts; b++) s += part[(size_t)b * H * (EIN + 1) + o];
    const int m = o / (EIN + 1), q = o - m * (EIN + 1);
    if (q < EIN) g[we_off + m * EIN + q] = s;
    else g[be_off + m] = s;
}

// x (node inputs, kept for the encoder's weight gradient)
__global__ void k_node_inputs(GraphDev G, float *__restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G.n) return;
    const float2 v = G.vel[i];
    x[4 * i] = v.x * G.inv_U;
    x[4 * i + 1] = v.y * G.inv_U;
    x[4 * i + 2] = G.srho[i] * G.inv_S;
    x[4 * i + 3] = G.wall[i];
}

// y - target on the fluid nodes: dy = 2 (y - t) / nfluid, per-block loss sums
__global__ void k_loss(const float *__restrict__ y, const float *__restrict__ t,
                       const float *__restrict__ wall, int n, float inv_nf,
                       float *__restrict__ dy, float *__restrict__ lpart) {
    __shared__ float red[kGB / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const bool fl = wall[i] == 0.f;
#pragma unroll
        for (int o = 0; o < NOUT; o++) {
            const float r = fl ? y[NOUT * i + o] - t[NOUT * i + o] : 0.f;
            l = fmaf(r, r, l);
            dy[NOUT * i + o] = 2.f * r * inv_nf;
        }
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < kGB / 32; w++) s += red[w];
        lpart[blockIdx.x] = s;
    }
}

// elementwise helpers of the backward pass
__global__ void k_add_strided(const float *__restrict__ a, const float *__restrict__ b, int ldb,
                              int n, float *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * H) return;
    const int i = t / H, c = t - i * H;
    out[t] = a[t] + b[(size_t)i * ldb + c];
}
__global__ void k_mul_dsilu(const float *__restrict__ a, const float *__restrict__ z, int n,
                            float *__restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = a[t] * dsilu(z[t]);
}

// Adam (bias-corrected), one thread per parameter
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = fmaf(b1, m[i], (1.f - b1) * gi);
    const float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// ------------------------------------------------------------------ inference
// The rollout's forward pass: the same network with BF16 weights and
// activations on the tensor cores (mma.sync m16n8k16, FP32 accumulation),
// fused per layer, and the edge sums in FP32 with SiLU(z) = (z/2)(1 +
// tanh(z/2)) on the hardware tanh.  Five launches:
//   node<0>  h0 = SiLU(A0 x + a0), P0 = h0 Wp0^T + be0, Q0 = h0 Wq0^T
//   edge     S0 = sum_j SiLU(P0_i + Q0_j + We0 e_ij)
//   node<1>  m = W2 S + deg b2, h1 = h0 + Wn2 SiLU(Wn1 [h0, m] + bn1) + bn2,
//            P1 = h1 Wp1^T + be1, Q1 = h1 Wq1^T
//   edge     S1
//   node<2>  h2 from h1, S1 as in node<1>; y = Wd h2 + bd
// A warp owns 16 nodes (one m16 tile); the weights are staged per block in
// shared memory as BF16 [out][in] rows padded to in + 8 (conflict-free B
// fragment loads); a GEMM's FP32 accumulators are repacked in registers as
// the next GEMM's A fragments.
typedef __nv_bfloat16 bf16;
constexpr int kInfWarps = 4;
constexpr int kInfBlocks = 152 * 4;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
    __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162 *>(&u);
    return __bfloat1622float2(v);
}
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float silu_hw(float z) {
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_hw(hz), hz);
}
// D = A B + D, A 16 x 16 (row), B 16 x 8 (col), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc[j] (n-blocks j0 .. j0 + NB - 1) += A (KB k-blocks) W^T, W in shared
// memory as [out][ld] BF16, input columns k0 + 16 kb
template <int NB, int KB>
__device__ __forceinline__ void warp_gemm(float (&acc)[NB][4], const uint32_t (&A)[KB][4],
                                          const bf16 *W, int ld, int j0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < NB; j++) {
#pragma unroll
        for (int kb = 0; kb < KB; kb++) {
            const bf16 *w = W + (size_t)(8 * (j0 + j) + g) * ld + k0 + 16 * kb + 2 * t;
            const uint32_t b0 = *reinterpret_cast<const uint32_t *>(w);
            const uint32_t b1 = *reinterpret_cast<const uint32_t *>(w + 8);
            mma_bf16(acc[j], A[kb], b0, b1);
        }
    }
}

// 64 accumulator columns (8 n-blocks) -> A fragments of a K = 64 input
__device__ __forceinline__ void acc_to_a(const float (&acc)[8][4], uint32_t (&A)[4][4]) {
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
        A[kb][0] = pack_bf16(acc[2 * kb][0], acc[2 * kb][1]);
        A[kb][1] = pack_bf16(acc[2 * kb][2], acc[2 * kb][3]);
        A[kb][2] = pack_bf16(acc[2 * kb + 1][0], acc[2 * kb + 1][1]);
        A[kb][3] = pack_bf16(acc[2 * kb + 1][2], acc[2 * kb + 1][3]);
    }
}

// A fragments of rows r0 .. r0 + 15 of a BF16 [n][64] array (0 past n)
__device__ __forceinline__ void load_a(const bf16 *X, int r0, int n, int lane, uint32_t (&A)[4][4]) {
    const int g = lane >> 2, t = lane & 3;
    const int ra = r0 + g, rb = r0 + g + 8;
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
        const int c = 16 * kb + 2 * t;
        A[kb][0] = ra < n ? *reinterpret_cast<const uint32_t *>(X + (size_t)ra * H + c) : 0u;
        A[kb][1] = rb < n ? *reinterpret_cast<const uint32_t *>(X + (size_t)rb * H + c) : 0u;
        A[kb][2] = ra < n ? *reinterpret_cast<const uint32_t *>(X + (size_t)ra * H + c + 8) : 0u;
        A[kb][3] = rb < n ? *reinterpret_cast<const uint32_t *>(X + (size_t)rb * H + c + 8) : 0u;
    }
}

// accumulator columns of n-blocks 0..7 -> BF16 [n][64] rows r0 .. r0 + 15
__device__ __forceinline__ void store_acc(const float (&acc)[8][4], bf16 *Y, int r0, int n,
                                          int lane) {
    const int g = lane >> 2, t = lane & 3;
    const int ra = r0 + g, rb = r0 + g + 8;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int c = 8 * j + 2 * t;
        if (ra < n) *reinterpret_cast<uint32_t *>(Y + (size_t)ra * H + c) = pack_bf16(acc[j][0], acc[j][1]);
        if (rb < n) *reinterpret_cast<uint32_t *>(Y + (size_t)rb * H + c) = pack_bf16(acc[j][2], acc[j][3]);
    }
}

struct InfArgs {
    GraphDev G;
    const float *p;  // FP32 parameters (Layout order)
    int A0, a0;                              // encoder (MODE 0)
    int W2, b2, Wn1, bn1, Wn2, bn2;          // the layer finished here (MODE 1, 2)
    int Wpq, be;                             // the next layer's [Wp; Wq] and be (MODE 0, 1)
    int Wd, bd;                              // decoder (MODE 2)
    bf16 *h, *P, *Q;
    const bf16 *S;
    float *y;
};

// shared memory of node<MODE>: BF16 weights, then FP32 vectors
constexpr int kLd64 = H + 8, kLd128 = 2 * H + 8;
template <int MODE> struct InfSmem {
    static constexpr int w2 = 0;
    static constexpr int wn1 = w2 + (MODE ? H * kLd64 : 0);
    static constexpr int wn2 = wn1 + (MODE ? H * kLd128 : 0);
    static constexpr int wpq = wn2 + (MODE ? H * kLd64 : 0);
    static constexpr int wd = wpq + (MODE < 2 ? 2 * H * kLd64 : 0);
    static constexpr int bf16_end = wd + (MODE == 2 ? 8 * kLd64 : 0);
    static constexpr int bytes_bf16 = ((bf16_end * 2 + 15) / 16) * 16;
    // FP32: A0 (H*NIN), a0, b2, bn1, bn2, be, bd (8)
    static constexpr int f_A0 = 0, f_a0 = f_A0 + H * NIN, f_b2 = f_a0 + H, f_bn1 = f_b2 + H,
                         f_bn2 = f_bn1 + H, f_be = f_bn2 + H, f_bd = f_be + H, f_end = f_bd + 8;
    static constexpr int bytes = bytes_bf16 + 4 * f_end;
};

__device__ __forceinline__ void stage_w(bf16 *dst, int ld, const float *src, int rows, int cols,
                                        int rows_pad) {
    for (int e = threadIdx.x; e < rows_pad * ld; e += blockDim.x) {
        const int r = e / ld, c = e - r * ld;
        dst[e] = __float2bfloat16_rn(r < rows && c < cols ? src[r * cols + c] : 0.f);
    }
}

template <int MODE>
__global__ void __launch_bounds__(32 * kInfWarps) k_inf_node(InfArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typedef InfSmem<MODE> SM;
    bf16 *sb = reinterpret_cast<bf16 *>(smem_raw);
    float *sf = reinterpret_cast<float *>(smem_raw + SM::bytes_bf16);
    const float *p = a.p;
    if (MODE) {
        stage_w(sb + SM::w2, kLd64, p + a.W2, H, H, H);
        stage_w(sb + SM::wn1, kLd128, p + a.Wn1, H, 2 * H, H);
        stage_w(sb + SM::wn2, kLd64, p + a.Wn2, H, H, H);
    }
    if (MODE < 2) stage_w(sb + SM::wpq, kLd64, p + a.Wpq, 2 * H, H, 2 * H);
    if (MODE == 2) stage_w(sb + SM::wd, kLd64, p + a.Wd, NOUT, H, 8);
    for (int e = threadIdx.x; e < H; e += blockDim.x) {
        if (MODE == 0) {
            sf[SM::f_a0 + e] = p[a.a0 + e];
            for (int k = 0; k < NIN; k++) sf[SM::f_A0 + e * NIN + k] = p[a.A0 + e * NIN + k];
        } else {
            sf[SM::f_b2 + e] = p[a.b2 + e];
            sf[SM::f_bn1 + e] = p[a.bn1 + e];
            sf[SM::f_bn2 + e] = p[a.bn2 + e];
        }
        if (MODE < 2) sf[SM::f_be + e] = p[a.be + e];
        if (MODE == 2 && e < 8) sf[SM::f_bd + e] = e < NOUT ? p[a.bd + e] : 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int n = a.G.n;
    for (int tile = blockIdx.x * kInfWarps + warp; tile * 16 < n; tile += gridDim.x * kInfWarps) {
        const int r0 = tile * 16, ra = r0 + g, rb = r0 + g + 8;
        float hc[8][4];  // h of this layer's output, FP32, accumulator layout
        if (MODE == 0) {
            float xa[NIN] = {0.f, 0.f, 0.f, 0.f}, xb[NIN] = {0.f, 0.f, 0.f, 0.f};
            if (ra < n) {
                const float2 v = a.G.vel[ra];
                xa[0] = v.x * a.G.inv_U; xa[1] = v.y * a.G.inv_U;
                xa[2] = a.G.srho[ra] * a.G.inv_S; xa[3] = a.G.wall[ra];
            }
            if (rb < n) {
                const float2 v = a.G.vel[rb];
                xb[0] = v.x * a.G.inv_U; xb[1] = v.y * a.G.inv_U;
                xb[2] = a.G.srho[rb] * a.G.inv_S; xb[3] = a.G.wall[rb];
            }
#pragma unroll
            for (int j = 0; j < 8; j++) {
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const int c = 8 * j + 2 * t + q;
                    float za = sf[SM::f_a0 + c], zb = za;
#pragma unroll
                    for (int k = 0; k < NIN; k++) {
                        const float w = sf[SM::f_A0 + c * NIN + k];
                        za = fmaf(w, xa[k], za);
                        zb = fmaf(w, xb[k], zb);
                    }
                    hc[j][q] = silu(za);
                    hc[j][2 + q] = silu(zb);
                }
            }
        } else {
            uint32_t AS[4][4], Ah[4][4], Am[4][4], At[4][4];
            load_a(a.S, r0, n, lane, AS);
            float m[8][4];
            const float da = ra < n ? (float)a.G.deg[ra] : 0.f, db = rb < n ? (float)a.G.deg[rb] : 0.f;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int c = 8 * j + 2 * t;
                m[j][0] = da * sf[SM::f_b2 + c];
                m[j][1] = da * sf[SM::f_b2 + c + 1];
                m[j][2] = db * sf[SM::f_b2 + c];
                m[j][3] = db * sf[SM::f_b2 + c + 1];
            }
            warp_gemm<8, 4>(m, AS, sb + SM::w2, kLd64, 0, 0, lane);
            acc_to_a(m, Am);
            load_a(a.h, r0, n, lane, Ah);
            float u[8][4];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int c = 8 * j + 2 * t;
                u[j][0] = u[j][2] = sf[SM::f_bn1 + c];
                u[j][1] = u[j][3] = sf[SM::f_bn1 + c + 1];
            }
            warp_gemm<8, 4>(u, Ah, sb + SM::wn1, kLd128, 0, 0, lane);
            warp_gemm<8, 4>(u, Am, sb + SM::wn1, kLd128, 0, H, lane);
#pragma unroll
            for (int j = 0; j < 8; j++)
#pragma unroll
                for (int q = 0; q < 4; q++) u[j][q] = silu(u[j][q]);
            acc_to_a(u, At);
            // h + bn2 in the accumulator layout (h from its A fragments)
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    const int j = 2 * kb + half, c = 8 * j + 2 * t;
                    const float2 lo = unpack_bf16(Ah[kb][2 * half]), hi = unpack_bf16(Ah[kb][2 * half + 1]);
                    hc[j][0] = lo.x + sf[SM::f_bn2 + c];
                    hc[j][1] = lo.y + sf[SM::f_bn2 + c + 1];
                    hc[j][2] = hi.x + sf[SM::f_bn2 + c];
                    hc[j][3] = hi.y + sf[SM::f_bn2 + c + 1];
                }
            }
            warp_gemm<8, 4>(hc, At, sb + SM::wn2, kLd64, 0, 0, lane);
        }
        uint32_t Ahn[4][4];
        acc_to_a(hc, Ahn);
        if (MODE < 2) {
            store_acc(hc, a.h, r0, n, lane);
            float pq[8][4];
#pragma unroll
            for (int half = 0; half < 2; half++) {  // P (+ be), then Q
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int c = 8 * j + 2 * t;
                    const float b0 = half ? 0.f : sf[SM::f_be + c], b1 = half ? 0.f : sf[SM::f_be + c + 1];
                    pq[j][0] = pq[j][2] = b0;
                    pq[j][1] = pq[j][3] = b1;
                }
                warp_gemm<8, 4>(pq, Ahn, sb + SM::wpq, kLd64, 8 * half, 0, lane);
                store_acc(pq, half ? a.Q : a.P, r0, n, lane);
            }
        } else {
            float yd[1][4];
            yd[0][0] = yd[0][2] = sf[SM::f_bd + 2 * t];
            yd[0][1] = yd[0][3] = sf[SM::f_bd + 2 * t + 1];
            warp_gemm<1, 4>(yd, Ahn, sb + SM::wd, kLd64, 0, 0, lane);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int c = 2 * t + q;
                if (c < NOUT) {
                    if (ra < n) a.y[(size_t)ra * NOUT + c] = yd[0][q];
                    if (rb < n) a.y[(size_t)rb * NOUT + c] = yd[0][2 + q];
                }
            }
        }
    }
}

// S_i = sum_j SiLU(P_i + Q_j + We e_ij) (P holds be), warp per node, lane
// c holds channels 2c and 2c + 1
__global__ void __launch_bounds__(kGB) k_inf_edge(GraphDev G, const bf16 *__restrict__ P,
                                                  const bf16 *__restrict__ Q,
                                                  const float *__restrict__ We,
                                                  bf16 *__restrict__ S) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= G.n) return;
    const int c0 = 2 * lane;
    float w0[EIN], w1[EIN];
#pragma unroll
    for (int k = 0; k < EIN; k++) {
        w0[k] = We[c0 * EIN + k];
        w1[k] = We[(c0 + 1) * EIN + k];
    }
    const float2 pi = unpack_bf16(*reinterpret_cast<const uint32_t *>(P + (size_t)i * H + c0));
    float s0 = 0.f, s1 = 0.f;
    const int d = G.deg[i];
    const double2 ri = G.pos[i];
    const float2 vi = G.vel[i];
    // kEdgeU neighbours' Q rows are gathered before any is used, so a warp
    // keeps that many L2 round trips in flight; the sums still run in
    // neighbour order
    constexpr int kEdgeU = 4;
    for (int k0 = 0; k0 < d; k0 += 32) {
        const EdgeLane mine = edge_lane(G, i, ri, vi, k0 + lane);
        const int cnt = min(32, d - k0);
        for (int tt = 0; tt < cnt; tt += kEdgeU) {
            uint32_t qv[kEdgeU];
#pragma unroll
            for (int u = 0; u < kEdgeU; u++) {
                const int j = __shfl_sync(0xffffffffu, mine.j, (tt + u) & 31);
                qv[u] = tt + u < cnt ? *reinterpret_cast<const uint32_t *>(Q + (size_t)j * H + c0)
                                     : 0u;
            }
#pragma unroll
            for (int u = 0; u < kEdgeU; u++) {
                if (tt + u >= cnt) break;  // (warp-uniform)
                const float2 qj = unpack_bf16(qv[u]);
                float z0 = pi.x + qj.x, z1 = pi.y + qj.y;
#pragma unroll
                for (int q = 0; q < EIN; q++) {
                    const float eq = __shfl_sync(0xffffffffu, mine.e[q], tt + u);
                    z0 = fmaf(w0[q], eq, z0);
                    z1 = fmaf(w1[q], eq, z1);
                }
                s0 += silu_hw(z0);
                s1 += silu_hw(z1);
            }
        }
    }
    *reinterpret_cast<uint32_t *>(S + (size_t)i * H + c0) = pack_bf16(s0, s1);
}

#define GCK(call)                                                                 \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));   \
            return TSPH_ERR_CUDA;                                                 \
        }                                                                         \
    } while (0)

inline int gblocks(long long n, int b = kGB) { return (int)((n + b - 1) / b > 0 ? (n + b - 1) / b : 1); }

}  // namespace
}  // namespace tsph

// the network, its gradients, Adam moments and activations for `cap` nodes
struct tsph_gnn {
    tsph::Layout L;
    int cap = 0;
    cudaStream_t st = nullptr;
    std::vector<void *> allocs;
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
    float *x = nullptr, *z0 = nullptr, *hs[tsph::NL + 1] = {}, *P[tsph::NL] = {}, *Q[tsph::NL] = {},
          *S[tsph::NL] = {}, *mm[tsph::NL] = {}, *u[tsph::NL] = {}, *t[tsph::NL] = {};
    float *y = nullptr, *dy = nullptr, *dh = nullptr, *dh2 = nullptr, *dhm = nullptr,
          *du = nullptr, *dP = nullptr, *dQ = nullptr, *dS = nullptr;
    float *part = nullptr, *epart = nullptr, *lpart = nullptr;
    float *ib[4] = {};  // inference activations h, P, Q, S (BF16, cap x 64 each)
    int adam_t = 0;
    tsph::GraphDev G{};
    ~tsph_gnn() {
        for (void *q : allocs) cudaFree(q);
    }
};

namespace {
using namespace tsph;

int galloc(tsph_gnn *n, float **q, size_t count) {
    void *x = nullptr;
    if (cudaMalloc(&x, sizeof(float) * (count ? count : 1)) != cudaSuccess) {
        cudaGetLastError();
        set_last_error("cudaMalloc failed for the network's buffers");
        return TSPH_ERR_NOMEM;
    }
    n->allocs.push_back(x);
    *q = static_cast<float *>(x);
    return 0;
}

LinArgs lin(const float *X1, int K1, int ld1, const float *W, int wm, int wk, float *Y, int n) {
    LinArgs a{};
    a.X1 = X1;
    a.K1 = K1;
    a.ld1 = ld1;
    a.X2 = nullptr;
    a.K2 = 0;
    a.ld2 = 0;
    a.W = W;
    a.wm = wm;
    a.wk = wk;
    a.Y = Y;
    a.n = n;
    return a;
}

int run_lin(tsph_gnn *N, int M, const LinArgs &a) {
    const int nb = std::min(gblocks(a.n, kLinTN), kLinBlocks);
    if (M == 128) k_linear<128><<<nb, kGB, 0, N->st>>>(a);
    else k_linear<64><<<nb, kGB, 0, N->st>>>(a);
    GCK(cudaGetLastError());
    return 0;
}

// dW from dY [n x M] and X = [X1 | X2], reduced into N->g
int run_wgrad(tsph_gnn *N, const float *dY, int ldy, int M, const float *X1, int K1, int ld1,
              const float *X2, int K2, int ld2, bool bias, const int32_t *deg, int n, int w_off,
              int b_off, int d_off) {
    WgArgs a{dY, ldy, M, X1, X2, K1, K2, ld1, ld2, bias ? 1 : 0, deg, n, N->part};
    k_wgrad<<<kWgBlocks, kGB, 0, N->st>>>(a);
    const int Kt = K1 + K2 + (bias ? 1 : 0) + (deg ? 1 : 0);
    k_wgrad_reduce<<<gblocks((long long)M * Kt), kGB, 0, N->st>>>(
        N->part, kWgBlocks, M, K1 + K2, bias ? 1 : 0, deg ? 1 : 0, N->g, w_off, b_off, d_off, 0);
    GCK(cudaGetLastError());
    return 0;
}

int forward(tsph_gnn *N) {
    const int n = N->G.n;
    const Layout &L = N->L;
    const float *p = N->p;
    k_node_inputs<<<gblocks(n), kGB, 0, N->st>>>(N->G, N->x);
    k_encode<<<gblocks((long long)n * H), kGB, 0, N->st>>>(N->G, p + L.A0, p + L.a0, N->z0, N->hs[0]);
    int rc;
    for (int l = 0; l < NL; l++) {
        const float *h = N->hs[l];
        if ((rc = run_lin(N, 64, lin(h, H, H, p + L.Wp[l], H, 1, N->P[l], n))) ||
            (rc = run_lin(N, 64, lin(h, H, H, p + L.Wq[l], H, 1, N->Q[l], n))))
            return rc;
        k_edge_forward<<<gblocks((long long)n * 32), kGB, 0, N->st>>>(
            N->G, N->P[l], N->Q[l], p + L.We[l], p + L.be[l], N->S[l]);
        LinArgs am = lin(N->S[l], H, H, p + L.W2[l], H, 1, N->mm[l], n);
        am.b2 = p + L.b2[l];
        am.deg = N->G.deg;
        if ((rc = run_lin(N, 64, am))) return rc;
        LinArgs au = lin(h, H, H, p + L.Wn1[l], 2 * H, 1, N->t[l], n);
        au.X2 = N->mm[l];
        au.K2 = H;
        au.ld2 = H;
        au.b = p + L.bn1[l];
        au.pre = N->u[l];
        au.act = 1;
        if ((rc = run_lin(N, 64, au))) return rc;
        LinArgs ah = lin(N->t[l], H, H, p + L.Wn2[l], H, 1, N->hs[l + 1], n);
        ah.b = p + L.bn2[l];
        ah.res = h;
        if ((rc = run_lin(N, 64, ah))) return rc;
    }
    k_decode<<<gblocks((long long)n * NOUT), kGB, 0, N->st>>>(N->hs[NL], n, p + L.Wd, p + L.bd, N->y);
    GCK(cudaGetLastError());
    return 0;
}

// gradients of the loss whose dL/dy is in N->dy (forward must have run)
int backward(tsph_gnn *N) {
    const int n = N->G.n;
    const Layout &L = N->L;
    const float *p = N->p;
    int rc;
    // decoder
    if ((rc = run_wgrad(N, N->dy, NOUT, NOUT, N->hs[NL], H, H, nullptr, 0, 0, true, nullptr, n,
                        L.Wd, L.bd, 0)))
        return rc;
    if ((rc = run_lin(N, 64, lin(N->dy, NOUT, NOUT, p + L.Wd, 1, H, N->dh, n)))) return rc;
    for (int l = NL - 1; l >= 0; l--) {
        const float *h = N->hs[l];
        // h_out = h + Wn2 t + bn2
        if ((rc = run_wgrad(N, N->dh, H, H, N->t[l], H, H, nullptr, 0, 0, true, nullptr, n,
                            L.Wn2[l], L.bn2[l], 0)))
            return rc;
        LinArgs a1 = lin(N->dh, H, H, p + L.Wn2[l], 1, H, N->du, n);
        a1.aux = N->u[l];
        if ((rc = run_lin(N, 64, a1))) return rc;
        // u = Wn1 [h, m] + bn1
        if ((rc = run_wgrad(N, N->du, H, H, h, H, H, N->mm[l], H, H, true, nullptr, n, L.Wn1[l],
                            L.bn1[l], 0)))
            return rc;
        if ((rc = run_lin(N, 128, lin(N->du, H, H, p + L.Wn1[l], 1, 2 * H, N->dhm, n)))) return rc;
        // m = W2 S + deg b2: dW2, db2 (degree column), dS = dm W2
        if ((rc = run_wgrad(N, N->dhm + H, 2 * H, H, N->S[l], H, H, nullptr, 0, 0, false,
                            N->G.deg, n, L.W2[l], 0, L.b2[l])))
            return rc;
        if ((rc = run_lin(N, 64, lin(N->dhm + H, H, 2 * H, p + L.W2[l], 1, H, N->dS, n)))) return rc;
        // edges: dP, dQ, dWe, dbe
        const int eb = gblocks((long long)n * 32);
        k_edge_backward<<<eb, kGB, 0, N->st>>>(N->G, N->P[l], N->Q[l], p + L.We[l], p + L.be[l],
                                               N->dS, N->dP, N->dQ, N->epart);
        k_edge_wgrad_reduce<<<gblocks(H * (EIN + 1)), kGB, 0, N->st>>>(N->epart, eb, N->g, L.We[l],
                                                                      L.be[l]);
        GCK(cudaGetLastError());
        if ((rc = run_wgrad(N, N->dP, H, H, h, H, H, nullptr, 0, 0, false, nullptr, n, L.Wp[l], 0,
                            0)) ||
            (rc = run_wgrad(N, N->dQ, H, H, h, H, H, nullptr, 0, 0, false, nullptr, n, L.Wq[l], 0,
                            0)))
            return rc;
        // dh_in = dh + dhm[:, :H] + dP Wp + dQ Wq
        k_add_strided<<<gblocks((long long)n * H), kGB, 0, N->st>>>(N->dh, N->dhm, 2 * H, n, N->dh2);
        LinArgs ad = lin(N->dP, H, H, p + L.Wp[l], 1, H, N->dh, n);
        ad.X2 = N->dQ;
        ad.K2 = H;
        ad.ld2 = H;  // [Wp; Wq] is contiguous: W(m, k) = Wp[k * H + m] for k < 2H
        ad.res = N->dh2;
        if ((rc = run_lin(N, 64, ad))) return rc;
    }
    // encoder
    k_mul_dsilu<<<gblocks((long long)n * H), kGB, 0, N->st>>>(N->dh, N->z0, n * H, N->dh2);
    if ((rc = run_wgrad(N, N->dh2, H, H, N->x, NIN, NIN, nullptr, 0, 0, true, nullptr, n, L.A0,
                        L.a0, 0)))
        return rc;
    GCK(cudaGetLastError());
    return 0;
}

int set_graph(tsph_gnn *N, const tsph_gnn_graph *gr) {
    if (!gr || gr->n_nodes < 0 || gr->n_nodes > N->cap || gr->k_slots < 1 || !gr->pos ||
        !gr->vel || !gr->srho || !gr->wall || !gr->deg || !gr->nbr || !(gr->h > 0) ||
        !(gr->u_scale > 0) || !(gr->s_scale > 0)) {
        set_last_error("bad graph");
        return TSPH_ERR_ARG;
    }
    const int n = gr->n_nodes;
    N->G = GraphDev{static_cast<const double2 *>(gr->pos), static_cast<const float2 *>(gr->vel),
                    gr->srho, gr->wall, gr->deg, gr->nbr, n, gr->k_slots,
                    (float)(1.0 / gr->h), (float)(1.0 / gr->u_scale), (float)(1.0 / gr->s_scale)};
    return 0;
}

// the BF16 tensor-core forward (the rollout's): y [n][3]
int infer(tsph_gnn *N, float *y) {
    const int n = N->G.n;
    if (n == 0) return 0;
    const Layout &L = N->L;
    bf16 *hb = reinterpret_cast<bf16 *>(N->ib[0]), *Pb = reinterpret_cast<bf16 *>(N->ib[1]),
         *Qb = reinterpret_cast<bf16 *>(N->ib[2]), *Sb = reinterpret_cast<bf16 *>(N->ib[3]);
    GCK(cudaFuncSetAttribute(k_inf_node<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, InfSmem<0>::bytes));
    GCK(cudaFuncSetAttribute(k_inf_node<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, InfSmem<1>::bytes));
    GCK(cudaFuncSetAttribute(k_inf_node<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, InfSmem<2>::bytes));
    const int nb = std::min(gblocks(n, 16 * kInfWarps), kInfBlocks);
    const int eb = gblocks((long long)n * 32);
    InfArgs a{};
    a.G = N->G;
    a.p = N->p;
    a.h = hb;
    a.P = Pb;
    a.Q = Qb;
    a.S = Sb;
    a.y = y;
    a.A0 = L.A0;
    a.a0 = L.a0;
    a.Wpq = L.Wp[0];
    a.be = L.be[0];
    k_inf_node<0><<<nb, 32 * kInfWarps, InfSmem<0>::bytes, N->st>>>(a);
    for (int l = 0; l < NL; l++) {
        k_inf_edge<<<eb, kGB, 0, N->st>>>(N->G, Pb, Qb, N->p + L.We[l], Sb);
        a.W2 = L.W2[l];
        a.b2 = L.b2[l];
        a.Wn1 = L.Wn1[l];
        a.bn1 = L.bn1[l];
        a.Wn2 = L.Wn2[l];
        a.bn2 = L.bn2[l];
        if (l + 1 < NL) {
            a.Wpq = L.Wp[l + 1];
            a.be = L.be[l + 1];
            k_inf_node<1><<<nb, 32 * kInfWarps, InfSmem<1>::bytes, N->st>>>(a);
        } else {
            a.Wd = L.Wd;
            a.bd = L.bd;
            k_inf_node<2><<<nb, 32 * kInfWarps, InfSmem<2>::bytes, N->st>>>(a);
        }
    }
    GCK(cudaGetLastError());
    return 0;
}

}  // namespace

extern "C" {

int tsph_gnn_n_params(void) { return tsph::Layout().total; }

int tsph_gnn_create(int capacity, void *stream, tsph_gnn **out) {
    if (!out || capacity < 1) {
        set_last_error("bad arguments");
        return TSPH_ERR_ARG;
    }
    *out = nullptr;
    tsph_gnn *N = new tsph_gnn();
    N->cap = capacity;
    N->st = static_cast<cudaStream_t>(stream);
    const size_t c = (size_t)capacity, P = (size_t)N->L.total;
    int rc = 0;
    auto A = [&](float **q, size_t count) {
        if (!rc) rc = galloc(N, q, count);
    };
    A(&N->p, P);
    A(&N->g, P);
    A(&N->m1, P);
    A(&N->m2, P);
    A(&N->x, NIN * c);
    A(&N->z0, H * c);
    for (int l = 0; l <= NL; l++) A(&N->hs[l], H * c);
    for (int l = 0; l < NL; l++) {
        A(&N->P[l], H * c);
        A(&N->Q[l], H * c);
        A(&N->S[l], H * c);
        A(&N->mm[l], H * c);
        A(&N->u[l], H * c);
        A(&N->t[l], H * c);
    }
    A(&N->y, NOUT * c);
    A(&N->dy, NOUT * c);
    A(&N->dh, H * c);
    A(&N->dh2, H * c);
    A(&N->dhm, 2 * H * c);
    A(&N->du, H * c);
    A(&N->dP, H * c);
    A(&N->dQ, H * c);
    A(&N->dS, H * c);
    A(&N->part, (size_t)kWgBlocks * kWgMaxOut);
    A(&N->epart, (size_t)gblocks((long long)c * 32) * H * (EIN + 1));
    A(&N->lpart, (size_t)gblocks((long long)c));
    for (int k = 0; k < 4; k++) A(&N->ib[k], (size_t)H / 2 * c);
    if (!rc && (cudaMemset(N->p, 0, 4 * P) != cudaSuccess || cudaMemset(N->m1, 0, 4 * P) != cudaSuccess ||
                cudaMemset(N->m2, 0, 4 * P) != cudaSuccess)) {
        set_last_error("cudaMemset failed");
        rc = TSPH_ERR_CUDA;
    }
    if (rc) {
        delete N;
        return rc;
    }
    *out = N;
    return TSPH_OK;
}

int tsph_gnn_destroy(tsph_gnn *N) {
    delete N;
    return TSPH_OK;
}

int tsph_gnn_set_params(tsph_gnn *N, const float *host) {
    if (!N || !host) return (set_last_error("null argument"), TSPH_ERR_ARG);
    GCK(cudaMemcpyAsync(N->p, host, 4 * (size_t)N->L.total, cudaMemcpyHostToDevice, N->st));
    GCK(cudaMemsetAsync(N->m1, 0, 4 * (size_t)N->L.total, N->st));
    GCK(cudaMemsetAsync(N->m2, 0, 4 * (size_t)N->L.total, N->st));
    GCK(cudaStreamSynchronize(N->st));
    N->adam_t = 0;
    return TSPH_OK;
}

int tsph_gnn_get_params(tsph_gnn *N, float *host) {
    if (!N || !host) return (set_last_error("null argument"), TSPH_ERR_ARG);
    GCK(cudaMemcpyAsync(host, N->p, 4 * (size_t)N->L.total, cudaMemcpyDeviceToHost, N->st));
    GCK(cudaStreamSynchronize(N->st));
    return TSPH_OK;
}

int tsph_gnn_get_grads(tsph_gnn *N, float *host) {
    if (!N || !host) return (set_last_error("null argument"), TSPH_ERR_ARG);
    GCK(cudaMemcpyAsync(host, N->g, 4 * (size_t)N->L.total, cudaMemcpyDeviceToHost, N->st));
    GCK(cudaStreamSynchronize(N->st));
    return TSPH_OK;
}

int tsph_gnn_forward(tsph_gnn *N, const tsph_gnn_graph *graph, float *y) {
    if (!N) return (set_last_error("null network"), TSPH_ERR_ARG);
    int rc;
    if ((rc = set_graph(N, graph)) || (rc = forward(N))) return rc;
    if (y) GCK(cudaMemcpyAsync(y, N->y, 4 * (size_t)NOUT * graph->n_nodes, cudaMemcpyDeviceToDevice, N->st));
    return TSPH_OK;
}

int tsph_gnn_infer(tsph_gnn *N, const tsph_gnn_graph *graph, float *y) {
    if (!N || !y) return (set_last_error("null argument"), TSPH_ERR_ARG);
    int rc;
    if ((rc = set_graph(N, graph)) || (rc = infer(N, y))) return rc;
    return TSPH_OK;
}

int tsph_gnn_loss_grad(tsph_gnn *N, const tsph_gnn_graph *graph, const float *target,
                       double *loss) {
    if (!N || !target) return (set_last_error("null argument"), TSPH_ERR_ARG);
    int rc;
    if ((rc = set_graph(N, graph)) || (rc = forward(N))) return rc;
    const int n = graph->n_nodes;
    std::vector<float> wall(n);
    GCK(cudaMemcpyAsync(wall.data(), graph->wall, 4 * (size_t)n, cudaMemcpyDeviceToHost, N->st));
    GCK(cudaStreamSynchronize(N->st));
    int nf = 0;
    for (float w : wall) nf += w == 0.f;
    const int nb = gblocks(n);
    k_loss<<<nb, kGB, 0, N->st>>>(N->y, target, graph->wall, n, 1.f / (float)(nf > 0 ? nf : 1),
                                  N->dy, N->lpart);
    GCK(cudaGetLastError());
    if ((rc = backward(N))) return rc;
    if (loss) {
        std::vector<float> lp(nb);
        GCK(cudaMemcpyAsync(lp.data(), N->lpart, 4 * (size_t)nb, cudaMemcpyDeviceToHost, N->st));
        GCK(cudaStreamSynchronize(N->st));
        double sum = 0;
        for (float v : lp) sum += v;
        *loss = sum / (nf > 0 ? nf : 1);
    }
    return TSPH_OK;
}

int tsph_gnn_adam(tsph_gnn *N, double lr, double beta1, double beta2, double eps) {
    if (!N) return (set_last_error("null network"), TSPH_ERR_ARG);
    N->adam_t++;
    const double c1 = 1.0 / (1.0 - std::pow(beta1, N->adam_t));
    const double c2 = 1.0 / (1.0 - std::pow(beta2, N->adam_t));
    k_adam<<<gblocks(N->L.total), kGB, 0, N->st>>>(N->p, N->g, N->m1, N->m2, N->L.total, (float)lr,
                                                   (float)beta1, (float)beta2, (float)eps,
                                                   (float)c1, (float)c2);
    GCK(cudaGetLastError());
    return TSPH_OK;
}

}  // extern "C"
