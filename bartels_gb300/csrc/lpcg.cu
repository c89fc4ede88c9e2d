// Learned PCG preconditioner: a 3-layer message-passing network over the mesh
// vertex graph (the Hessian's block pattern) that outputs a block-lower-
// triangular factor G on that pattern; PCG then uses M^-1 = G^T G.
//
// Coordinates. With L_v = chol(A_vv) and the block-diagonal L, the network sees
// the normalised Hessian  Ahat = L^-1 A L^-T  (Ahat_vv = I) and outputs Ghat;
// G = Ghat L^-1, so G A G^T = Ghat Ahat Ghat^T. Ghat = I is block-Jacobi, which
// is what the network starts from (zero output layers).
//
// Network (width H = 64, ReLU):
//   x_v   = [1, deg_v/14, mean_j |Ahat_vj|, max_j |Ahat_vj|]     (free neighbours j)
//   e_vj  = [Ahat_vj (row-major 9), |Ahat_vj|]
//   h^0   = relu(x W0 + b0)
//   layer l = 1..3:  [P | Q] = bf16(h) Wpq^T                    (tensor-core GEMM)
//                    m_vj = relu(P_v + Q_j + e_vj We + be)
//                    a_v  = (1/deg_v) sum_j m_vj
//                    h   <- h + relu(bf16([h | a]) Wu^T + bu)    (tensor-core GEMM)
//   head:            [S | T] = bf16(h) Wst^T                     (tensor-core GEMM)
//                    Ghat_vj = relu(S_v + T_j + e_vj Wf + bf) Wo + bo + e_vj Wskip   (j < v)
//                    d_v = h_v Wd + bd,  Ghat_vv = [[e^d0,0,0],[d3,e^d1,0],[d4,d5,e^d2]]
// Pinned vertices take no part: their rows and columns of G are zero.
//
// Training loss (log of Kaporin's condition number of G A G^T, up to a constant):
//   L = log( tr(Ghat Ahat Ghat^T) / N ) - (2/N) sum_v (d_v0 + d_v1 + d_v2)
// with the trace estimated from probe vectors w (Rademacher, plus an optional
// Newton residual): tr ~ (1/P) sum_p u_p^T Ahat u_p, u_p = Ghat^T w_p.
// Every kernel below has a hand-written backward; weight gradients are summed
// in a fixed order (block partials, then one ordered pass), Adam updates the
// FP32 master weights and refreshes the BF16 copies the GEMMs read.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "lpcg_internal.cuh"

namespace bartels {

constexpr int kH = 64;
constexpr int kLayers = 3;
constexpr int kDx = 4;
constexpr int kDe = 10;
constexpr int kFe = 12;  // row stride of the edge-feature array (10 used, padded for float4 loads)

// ------------------------------------------------------- parameter layout ---
struct Layout {
  int W0, b0;
  int Wpq[kLayers], We[kLayers], be[kLayers], Wu[kLayers], bu[kLayers];
  int Wst, Wf, bf, Wo, bo, Wd, bd, Wskip;
  int total;
};
static Layout make_layout() {
  Layout L{};
  int o = 0;
  auto take = [&](int n) {
    int r = o;
    o += n;
    return r;
  };
  L.W0 = take(kDx * kH);
  L.b0 = take(kH);
  for (int l = 0; l < kLayers; ++l) {
    L.Wpq[l] = take(2 * kH * kH);  // [128 out][64 in]
    L.We[l] = take(kDe * kH);      // [10][64]
    L.be[l] = take(kH);
    L.Wu[l] = take(kH * 2 * kH);   // [64 out][128 in]
    L.bu[l] = take(kH);
  }
  L.Wst = take(2 * kH * kH);       // [128 out][64 in]
  L.Wf = take(kDe * kH);
  L.bf = take(kH);
  L.Wo = take(kH * 9);             // [64][9]
  L.bo = take(9);
  L.Wd = take(kH * 6);             // [64][6]
  L.bd = take(6);
  L.Wskip = take(kDe * 9);         // [10][9]: linear path from e_vj to Ghat_vj
  L.total = o;
  return L;
}
static const Layout kL = make_layout();

// BF16 copies: forward (N x K as stored) and backward (transposed) operands
struct BfLayout {
  int pq[kLayers], u[kLayers], st, pqT[kLayers], uT[kLayers], stT, total;
};
static BfLayout make_bf() {
  BfLayout B{};
  int o = 0;
  for (int l = 0; l < kLayers; ++l) {
    B.pq[l] = o; o += 8192;
    B.u[l] = o; o += 8192;
    B.pqT[l] = o; o += 8192;
    B.uT[l] = o; o += 8192;
  }
  B.st = o; o += 8192;
  B.stT = o; o += 8192;
  B.total = o;
  return B;
}
static const BfLayout kB = make_bf();

}  // namespace bartels

struct bartels_lpcg_s {
  bartels_ctx ctx = nullptr;
  float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *wbf = nullptr;
  int *err = nullptr;
  double *scal = nullptr;  // device scalars: [0] trace, [1] logdiag sum, [2] n_free, [3] grad norm^2
  int64_t step = 0;
  bool bf_dirty = true;
  bartels::DevBuf part;    // reduction partials
};

namespace bartels {

// Per-plan buffers (sized for the plan; training buffers only when trained on).
struct LpcgPlanState {
  int nV = 0;
  int64_t nnzb = 0, nnzl = 0, nnzu = 0;
  bool train = false;
  float *fe = nullptr, *linv = nullptr, *xn = nullptr, *invdeg = nullptr;
  float *h[kLayers + 1] = {};      // FP32 h^0..h^3 (inference reuses two)
  __nv_bfloat16 *ha[kLayers + 1] = {};  // [h | a] BF16, per layer input; ha[3] left half = bf16(h^3)
  float *pq[kLayers] = {};          // [P | Q]
  float *upre[kLayers] = {};        // U pre-activation
  float *pre0 = nullptr;
  float *st = nullptr;              // [S | T]
  float *raw = nullptr;             // 9 per lower block: Ghat_vj or (d0..d5) at the diagonal
  __nv_bfloat16 *gl = nullptr, *gu = nullptr;  // the factor G, BF16 (lower and upper storage)
  // training
  float *dh = nullptr, *dha = nullptr, *du = nullptr, *dpq = nullptr, *dst = nullptr;
  __nv_bfloat16 *dbf = nullptr;     // BF16 copy of a backward GEMM input (V x 128)
  float *dpre_e = nullptr;          // per full-pattern position x 64
  float *dpre_h = nullptr, *z_h = nullptr, *e_h = nullptr, *dg = nullptr;  // per lower block
  float *dd = nullptr;              // V x 6
  float *wprobe = nullptr, *uprobe = nullptr, *vprobe = nullptr;
  int nprobe = 0;
  std::vector<void *> allocs;
};

// ---------------------------------------------------------------- helpers ---
__device__ __forceinline__ uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return h;
}

// value (k, l) of block b of vertex row v in scalar-CSR order
__device__ __forceinline__ float blk_val(const float *vals, int64_t base, int rs, int b, int k, int l) {
  return vals[base + (int64_t)k * rs + 3 * b + l];
}

// ------------------------------------------------------ input features ---
__global__ void k_lp_linv(int nV, const int *__restrict__ brp, const int *__restrict__ diag_pos,
                          const float *__restrict__ vals, const unsigned char *__restrict__ pinned,
                          float *__restrict__ linv) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    float *o = linv + 6ll * v;
    const bool pin = pinned && pinned[v];
    const int64_t base = 9ll * brp[v];
    const int rs = 3 * (brp[v + 1] - brp[v]);
    const int d = diag_pos[v];
    float a00 = blk_val(vals, base, rs, d, 0, 0), a10 = blk_val(vals, base, rs, d, 1, 0);
    float a11 = blk_val(vals, base, rs, d, 1, 1), a20 = blk_val(vals, base, rs, d, 2, 0);
    float a21 = blk_val(vals, base, rs, d, 2, 1), a22 = blk_val(vals, base, rs, d, 2, 2);
    float l00 = sqrtf(fmaxf(a00, 1e-30f));
    float l10 = a10 / l00, l20 = a20 / l00;
    float l11 = sqrtf(fmaxf(a11 - l10 * l10, 1e-30f));
    float l21 = (a21 - l20 * l10) / l11;
    float l22 = sqrtf(fmaxf(a22 - l20 * l20 - l21 * l21, 1e-30f));
    float i00 = 1.f / l00, i11 = 1.f / l11, i22 = 1.f / l22;
    float i10 = -l10 * i00 * i11;
    float i21 = -l21 * i11 * i22;
    float i20 = -(l20 * i00 + l21 * i10) * i22;
    if (pin) {
      i00 = i11 = i22 = 1.f;
      i10 = i20 = i21 = 0.f;
    }
    o[0] = i00; o[1] = i10; o[2] = i11; o[3] = i20; o[4] = i21; o[5] = i22;
  }
}

__device__ __forceinline__ void linv_mat(const float *li, float (&L)[3][3]) {
  L[0][0] = li[0]; L[0][1] = 0.f;  L[0][2] = 0.f;
  L[1][0] = li[1]; L[1][1] = li[2]; L[1][2] = 0.f;
  L[2][0] = li[3]; L[2][1] = li[4]; L[2][2] = li[5];
}

// Ahat_vj = Linv_v A_vj Linv_j^T for every block of the pattern, and node
// features. 16 lanes per vertex row (one block each, coalesced reads of the
// row's three scalar rows, 48-byte feature rows written as three float4).
__global__ void __launch_bounds__(256)
k_lp_feats(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const float *__restrict__ vals,
           const unsigned char *__restrict__ pinned, const float *__restrict__ linv, float *__restrict__ fe,
           float *__restrict__ xn, float *__restrict__ invdeg) {
  const int lane = threadIdx.x & 31, sl = lane & 15, half = lane >> 4;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int vb = 2 * warp; vb < nV; vb += 2 * nwarps) {
    const int v = vb + half;
    const bool active = v < nV;
    int deg = 0;
    float sum = 0.f, mx = 0.f;
    if (active) {
      const bool pv = pinned && pinned[v];
      const int rb = brp[v], nb = brp[v + 1] - rb;
      const int64_t base = 9ll * rb;
      const int rs = 3 * nb;
      float Li[3][3];
      linv_mat(linv + 6ll * v, Li);
      for (int b = sl; b < nb; b += 16) {
        const int j = __ldg(bcol + rb + b);
        float o[kFe];
#pragma unroll
        for (int k = 0; k < kFe; ++k) o[k] = 0.f;
        if (!(pv || (pinned && pinned[j]))) {
          float Lj[3][3], A[3][3], T[3][3];
          linv_mat(linv + 6ll * j, Lj);
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int l = 0; l < 3; ++l) A[k][l] = __ldg(vals + base + (int64_t)k * rs + 3 * b + l);
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int l = 0; l < 3; ++l) {
              float acc = 0.f;
#pragma unroll
              for (int m = 0; m <= k; ++m) acc += Li[k][m] * A[m][l];
              T[k][l] = acc;
            }
          float nrm = 0.f;
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int l = 0; l < 3; ++l) {
              float acc = 0.f;
#pragma unroll
              for (int m = 0; m <= l; ++m) acc += T[k][m] * Lj[l][m];  // (Linv_j^T)[m][l] = Lj[l][m]
              o[3 * k + l] = acc;
              nrm += acc * acc;
            }
          nrm = sqrtf(nrm);
          o[9] = nrm;
          if (j != v) {
            deg++;
            sum += nrm;
            mx = fmaxf(mx, nrm);
          }
        }
        float4 *dst = reinterpret_cast<float4 *>(fe + (int64_t)kFe * (rb + b));
        dst[0] = make_float4(o[0], o[1], o[2], o[3]);
        dst[1] = make_float4(o[4], o[5], o[6], o[7]);
        dst[2] = make_float4(o[8], o[9], o[10], o[11]);
      }
    }
    // reductions over the 16 lanes of the row (all lanes of the warp take part)
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
      deg += __shfl_xor_sync(0xffffffffu, deg, off);
      sum += __shfl_xor_sync(0xffffffffu, sum, off);
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (active && sl == 0) {
      float *x = xn + (int64_t)kDx * v;
      if (pinned && pinned[v]) {
        x[0] = x[1] = x[2] = x[3] = 0.f;
        invdeg[v] = 0.f;
      } else {
        x[0] = 1.f;
        x[1] = deg * (1.f / 14.f);
        x[2] = deg > 0 ? sum / deg : 0.f;
        x[3] = mx;
        invdeg[v] = deg > 0 ? 1.f / deg : 0.f;
      }
    }
  }
}

// h0 = relu(x W0 + b0): one warp per vertex, two channels per lane.
__global__ void k_lp_embed(int nV, const float *__restrict__ xn, const float *__restrict__ W0,
                           const float *__restrict__ b0, float *__restrict__ pre0, float *__restrict__ h,
                           __nv_bfloat16 *__restrict__ ha) {
  const int lane = threadIdx.x & 31;
  const int c = 2 * lane;
  for (int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nV; v += (gridDim.x * blockDim.x) >> 5) {
    const float *x = xn + (int64_t)kDx * v;
    float p0 = b0[c], p1 = b0[c + 1];
#pragma unroll
    for (int k = 0; k < kDx; ++k) {
      p0 += x[k] * W0[k * kH + c];
      p1 += x[k] * W0[k * kH + c + 1];
    }
    if (pre0) {
      pre0[(int64_t)kH * v + c] = p0;
      pre0[(int64_t)kH * v + c + 1] = p1;
    }
    const float h0 = fmaxf(p0, 0.f), h1 = fmaxf(p1, 0.f);
    h[(int64_t)kH * v + c] = h0;
    h[(int64_t)kH * v + c + 1] = h1;
    reinterpret_cast<__nv_bfloat162 *>(ha + 2ll * kH * v)[lane] = __floats2bfloat162_rn(h0, h1);
  }
}

// Weights of the edge term e We + be for one lane's two channels (c, c+1),
// held in registers for the whole edge loop.
struct EdgeW {
  float w0[kDe], w1[kDe], b0, b1;
  __device__ __forceinline__ EdgeW(const float *__restrict__ W, const float *__restrict__ b, int c) {
#pragma unroll
    for (int k = 0; k < kDe; ++k) {
      w0[k] = W[k * kH + c];
      w1[k] = W[k * kH + c + 1];
    }
    b0 = b[c];
    b1 = b[c + 1];
  }
  // e: one edge's feature row (kFe floats, 16-byte aligned): three float4 loads
  __device__ __forceinline__ void apply(const float *__restrict__ e, float &r0, float &r1) const {
    const float4 a = __ldg(reinterpret_cast<const float4 *>(e));
    const float4 bq = __ldg(reinterpret_cast<const float4 *>(e) + 1);
    const float4 cq = __ldg(reinterpret_cast<const float4 *>(e) + 2);
    const float ev[kDe] = {a.x, a.y, a.z, a.w, bq.x, bq.y, bq.z, bq.w, cq.x, cq.y};
    r0 = b0;
    r1 = b1;
#pragma unroll
    for (int k = 0; k < kDe; ++k) {
      r0 += ev[k] * w0[k];
      r1 += ev[k] * w1[k];
    }
  }
};

// a_v = (1/deg_v) sum_j relu(P_v + Q_j + e_vj We + be), written as BF16 into
// the right half of [h | a]. One warp per vertex.
__global__ void __launch_bounds__(256)
k_lp_msg(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const unsigned char *__restrict__ pinned,
         const float *__restrict__ fe, const float *__restrict__ invdeg, const float *__restrict__ pq,
         const float *__restrict__ We, const float *__restrict__ be, __nv_bfloat16 *__restrict__ ha) {
  const int lane = threadIdx.x & 31;
  const int c = 2 * lane;
  const EdgeW ew(We, be, c);
  for (int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nV; v += (gridDim.x * blockDim.x) >> 5) {
    float a0 = 0.f, a1 = 0.f;
    if (!(pinned && pinned[v])) {
      const float2 P = reinterpret_cast<const float2 *>(pq + 2ll * kH * v)[lane];
      const int rb = brp[v], re = brp[v + 1];
      // four edges per step: every load of the step is issued before any is
      // used (an edge past the row's end reads its own vertex's data and is
      // masked, as are the self edge and pinned neighbours); contributions are
      // added in edge order
      for (int p = rb; p < re; p += 4) {
        int j[4];
        bool ok[4];
        float2 Q[4];
        float r[4][2];
#pragma unroll
        for (int q = 0; q < 4; ++q) j[q] = p + q < re ? __ldg(bcol + p + q) : v;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          Q[q] = reinterpret_cast<const float2 *>(pq + 2ll * kH * j[q] + kH)[lane];
          ew.apply(fe + (int64_t)kFe * (p + q < re ? p + q : p), r[q][0], r[q][1]);
          ok[q] = p + q < re && j[q] != v && !(pinned && pinned[j[q]]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (ok[q]) {
            a0 += fmaxf(P.x + Q[q].x + r[q][0], 0.f);
            a1 += fmaxf(P.y + Q[q].y + r[q][1], 0.f);
          }
      }
      const float s = invdeg[v];
      a0 *= s;
      a1 *= s;
    }
    reinterpret_cast<__nv_bfloat162 *>(ha + 2ll * kH * v + kH)[lane] = __floats2bfloat162_rn(a0, a1);
  }
}

// Output head: Ghat for the lower blocks of row v, G = Ghat Linv_col in the
// lower storage (BF16, padded rows); raw network outputs kept for training.
// One thread per vertex row; the head's weights sit in shared memory and are
// read as broadcasts, so the per-edge 64 -> 9 projection needs no shuffles.
constexpr int kHeadThreads = 128;
__global__ void __launch_bounds__(kHeadThreads)
k_lp_head(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const int *__restrict__ diag_pos,
          const int *__restrict__ lrp, const int4 *__restrict__ meta, const unsigned char *__restrict__ pinned,
          const float *__restrict__ fe, const float *__restrict__ linv, const float *__restrict__ h,
          const float *__restrict__ st, const float *__restrict__ Wf, const float *__restrict__ bf,
          const float *__restrict__ Wo, const float *__restrict__ bo, const float *__restrict__ Wd,
          const float *__restrict__ bd, const float *__restrict__ Wskip, float *__restrict__ raw,
          __nv_bfloat16 *__restrict__ gl) {
  __shared__ float sWf[kDe * kH], sbf[kH], sWo[kH * 9], sbo[9], sWd[kH * 6], sbd[6], sWs[kDe * 9];
  for (int i = threadIdx.x; i < kDe * kH; i += blockDim.x) sWf[i] = Wf[i];
  for (int i = threadIdx.x; i < kH * 9; i += blockDim.x) sWo[i] = Wo[i];
  for (int i = threadIdx.x; i < kH * 6; i += blockDim.x) sWd[i] = Wd[i];
  for (int i = threadIdx.x; i < kDe * 9; i += blockDim.x) sWs[i] = Wskip[i];
  for (int i = threadIdx.x; i < kH; i += blockDim.x) sbf[i] = bf[i];
  if (threadIdx.x < 9) sbo[threadIdx.x] = bo[threadIdx.x];
  if (threadIdx.x < 6) sbd[threadIdx.x] = bd[threadIdx.x];
  __syncthreads();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const bool pv = pinned && pinned[v];
    const int rb = brp[v], d = diag_pos[v], nl = d + 1, lb = lrp[v];
    const int rs = padded_row(nl);
    __nv_bfloat16 *g = gl + meta[v].y;
    const float4 *S4 = reinterpret_cast<const float4 *>(st + 2ll * kH * v);
    for (int b = 0; b < nl; ++b) {
      const int j = __ldg(bcol + rb + b);
      const bool zero = pv || (pinned && pinned[j]);
      float out[9];
#pragma unroll
      for (int o = 0; o < 9; ++o) out[o] = 0.f;
      if (!zero && b < d) {
        const float4 *e4 = reinterpret_cast<const float4 *>(fe + (int64_t)kFe * (rb + b));
        const float4 ea = __ldg(e4), eb = __ldg(e4 + 1), ec = __ldg(e4 + 2);
        const float ev[kDe] = {ea.x, ea.y, ea.z, ea.w, eb.x, eb.y, eb.z, eb.w, ec.x, ec.y};
        const float4 *T4 = reinterpret_cast<const float4 *>(st + 2ll * kH * j + kH);
        for (int c4 = 0; c4 < kH / 4; ++c4) {
          const float4 s4 = __ldg(S4 + c4), t4 = __ldg(T4 + c4);
          const float sv[4] = {s4.x, s4.y, s4.z, s4.w}, tv[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int c = 4 * c4 + q;
            float pre = sv[q] + tv[q] + sbf[c];
#pragma unroll
            for (int k = 0; k < kDe; ++k) pre += ev[k] * sWf[k * kH + c];
            const float z = fmaxf(pre, 0.f);
#pragma unroll
            for (int o = 0; o < 9; ++o) out[o] += z * sWo[c * 9 + o];
          }
        }
#pragma unroll
        for (int o = 0; o < 9; ++o) {
          float a = out[o] + sbo[o];
#pragma unroll
          for (int k = 0; k < kDe; ++k) a += ev[k] * sWs[k * 9 + o];
          out[o] = a;
        }
      } else if (!zero) {
        const float4 *h4 = reinterpret_cast<const float4 *>(h + (int64_t)kH * v);
        for (int c4 = 0; c4 < kH / 4; ++c4) {
          const float4 hq = __ldg(h4 + c4);
          const float hv[4] = {hq.x, hq.y, hq.z, hq.w};
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int o = 0; o < 6; ++o) out[o] += hv[q] * sWd[(4 * c4 + q) * 6 + o];
        }
#pragma unroll
        for (int o = 0; o < 6; ++o) out[o] += sbd[o];
      }
      float *rw = raw + 9ll * (lb + b);
#pragma unroll
      for (int o = 0; o < 9; ++o) rw[o] = out[o];
      float Gh[3][3];
      if (b < d) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int l = 0; l < 3; ++l) Gh[k][l] = out[3 * k + l];
      } else {
        Gh[0][0] = expf(out[0]); Gh[0][1] = 0.f;          Gh[0][2] = 0.f;
        Gh[1][0] = out[3];       Gh[1][1] = expf(out[1]); Gh[1][2] = 0.f;
        Gh[2][0] = out[4];       Gh[2][1] = out[5];       Gh[2][2] = expf(out[2]);
      }
      float Lj[3][3];
      linv_mat(linv + 6ll * j, Lj);
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          float acc = 0.f;
#pragma unroll
          for (int m = 0; m < 3; ++m) acc += Gh[k][m] * Lj[m][l];
          g[k * rs + 3 * b + l] = __float2bfloat16_rn(zero ? 0.f : acc);
        }
    }
  }
}

// Transposed copy of the lower storage into the upper storage: lower block
// (v, j) becomes block (j, v) of row j, transposed (padded BF16 rows).
__global__ void k_factor_transpose(int nV, const int *__restrict__ bcol, const int4 *__restrict__ meta,
                                   const int *__restrict__ lrp, const int *__restrict__ urp,
                                   const int *__restrict__ low2up, const __nv_bfloat16 *__restrict__ gl,
                                   __nv_bfloat16 *__restrict__ gu) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int4 mv = meta[v];
    const int nl = (mv.w & 0xFFFF) + 1;
    const int rsl = padded_row(nl);
    const int lb = lrp[v];
    const __nv_bfloat16 *src = gl + mv.y;
    for (int b = 0; b < nl; ++b) {
      const int j = bcol[mv.x + b];
      const int4 mj = meta[j];
      const int dj = mj.w & 0xFFFF, nuj = (mj.w >> 16) - dj;
      const int rsu = padded_row(nuj);
      const int m = low2up[lb + b] - urp[j];
      __nv_bfloat16 *dst = gu + mj.z;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l) dst[l * rsu + 3 * m + k] = src[k * rsl + 3 * b + l];
    }
  }
}

// ============================================================ training ===
// Probes: Rademacher +-1 on free DOFs (probe p < nrand); the last probe may be
// the normalised residual Linv r (scaled to unit mean square).
__global__ void k_lp_probes(int nV, int nrand, uint32_t seed, const unsigned char *__restrict__ pinned,
                            float *__restrict__ w) {
  const int n = 3 * nV;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool pv = pinned && pinned[i / 3];
    for (int p = 0; p < nrand; ++p)
      w[(int64_t)p * n + i] = pv ? 0.f : ((hash3(seed, p, i) & 1u) ? 1.f : -1.f);
  }
}
__global__ void k_lp_resid_probe(int nV, const double *__restrict__ r, const float *__restrict__ linv,
                                 const unsigned char *__restrict__ pinned, float *__restrict__ w) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    float L[3][3];
    linv_mat(linv + 6ll * v, L);
    const bool pv = pinned && pinned[v];
    for (int k = 0; k < 3; ++k) {
      float s = 0.f;
      for (int m = 0; m <= k; ++m) s += L[k][m] * (float)r[3 * v + m];
      w[3 * v + k] = pv ? 0.f : s;
    }
  }
}

__device__ __forceinline__ void ghat_of(const float *rw, bool diag, float (&G)[3][3]) {
  if (!diag) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int l = 0; l < 3; ++l) G[k][l] = rw[3 * k + l];
  } else {
    G[0][0] = expf(rw[0]); G[0][1] = 0.f;         G[0][2] = 0.f;
    G[1][0] = rw[3];       G[1][1] = expf(rw[1]); G[1][2] = 0.f;
    G[2][0] = rw[4];       G[2][1] = rw[5];       G[2][2] = expf(rw[2]);
  }
}

// u_p = Ghat^T w_p: row j gathers the transposed blocks Ghat_ij, i >= j.
__global__ void k_lp_gt_apply(int nV, int np, const int *__restrict__ brp, const int *__restrict__ bcol,
                              const int *__restrict__ diag_pos, const int *__restrict__ urp,
                              const int *__restrict__ up2low, const unsigned char *__restrict__ pinned,
                              const float *__restrict__ raw, const float *__restrict__ w, float *__restrict__ u) {
  const int n = 3 * nV;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nV; j += gridDim.x * blockDim.x) {
    const int rb = brp[j], d = diag_pos[j], nb = brp[j + 1] - rb;
    const bool pj = pinned && pinned[j];
    for (int p = 0; p < np; ++p) {
      float s[3] = {0.f, 0.f, 0.f};
      if (!pj)
        for (int m = 0; m < nb - d; ++m) {
          const int i = bcol[rb + d + m];
          if (pinned && pinned[i]) continue;
          float G[3][3];
          ghat_of(raw + 9ll * up2low[urp[j] + m], m == 0, G);
          const float *wi = w + (int64_t)p * n + 3 * i;
#pragma unroll
          for (int c = 0; c < 3; ++c) s[c] += G[0][c] * wi[0] + G[1][c] * wi[1] + G[2][c] * wi[2];
        }
      for (int c = 0; c < 3; ++c) u[(int64_t)p * n + 3 * j + c] = s[c];
    }
  }
}

// v_p = Ahat u_p (rows of pinned vertices 0); partials of sum_p u_p.v_p and of
// the free log-diagonal sum.
__global__ void __launch_bounds__(256)
k_lp_ahat_apply(int nV, int np, const int *__restrict__ brp, const int *__restrict__ bcol,
                const int *__restrict__ diag_pos, const int *__restrict__ lrp,
                const unsigned char *__restrict__ pinned, const float *__restrict__ fe,
                const float *__restrict__ raw, const float *__restrict__ u, float *__restrict__ vv,
                double *__restrict__ part) {
  const int n = 3 * nV;
  double acc = 0.0, ld = 0.0, nf = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nV; i += gridDim.x * blockDim.x) {
    const bool pv = pinned && pinned[i];
    const int rb = brp[i], re = brp[i + 1];
    for (int p = 0; p < np; ++p) {
      float s[3] = {0.f, 0.f, 0.f};
      if (!pv)
        for (int q = rb; q < re; ++q) {
          const int j = bcol[q];
          const float *A = fe + (int64_t)kFe * q;
          const float *uj = u + (int64_t)p * n + 3 * j;
#pragma unroll
          for (int k = 0; k < 3; ++k) s[k] += A[3 * k] * uj[0] + A[3 * k + 1] * uj[1] + A[3 * k + 2] * uj[2];
        }
      const float *ui = u + (int64_t)p * n + 3 * i;
      for (int k = 0; k < 3; ++k) {
        vv[(int64_t)p * n + 3 * i + k] = s[k];
        acc += (double)ui[k] * s[k];
      }
    }
    if (!pv) {
      const float *rw = raw + 9ll * (lrp[i] + diag_pos[i]);
      ld += (double)rw[0] + rw[1] + rw[2];
      nf += 3.0;
    }
  }
  __shared__ double red[3][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double vals[3] = {acc, ld, nf};
  for (int k = 0; k < 3; ++k) {
    double x = vals[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) {
      double x = 0.0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) x += red[k][i];
      part[3ll * blockIdx.x + k] = x;
    }
  }
}

// fixed-order sum of the partials into scal[0..2] (trace, logdiag, n_free)
__global__ void k_lp_loss_sum(int nparts, int np, const double *__restrict__ part, double *__restrict__ scal) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = 0; i < nparts; ++i) {
      a += part[3 * i];
      b += part[3 * i + 1];
      c += part[3 * i + 2];
    }
    scal[0] = a / np;
    scal[1] = b;
    scal[2] = c;
  }
}

// dL/dGhat for every lower block (and dL/dd at the diagonal):
//   dGhat_ij = (2 / (P t)) sum_p w_p[i] (x) v_p[j]
__global__ void k_lp_dghat(int nV, int np, const int *__restrict__ brp, const int *__restrict__ bcol,
                           const int *__restrict__ diag_pos, const int *__restrict__ lrp,
                           const unsigned char *__restrict__ pinned, const float *__restrict__ raw,
                           const float *__restrict__ w, const float *__restrict__ vv, const double *__restrict__ scal,
                           float *__restrict__ dg, float *__restrict__ dd) {
  const int n = 3 * nV;
  const float ct = (float)(2.0 / (np * scal[0]));
  const float cl = (float)(2.0 / scal[2]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nV; i += gridDim.x * blockDim.x) {
    const bool pv = pinned && pinned[i];
    const int rb = brp[i], d = diag_pos[i], lb = lrp[i];
    for (int b = 0; b <= d; ++b) {
      const int j = bcol[rb + b];
      float D[3][3] = {};
      const bool zero = pv || (pinned && pinned[j]);
      if (!zero)
        for (int p = 0; p < np; ++p) {
          const float *wi = w + (int64_t)p * n + 3 * i;
          const float *vj = vv + (int64_t)p * n + 3 * j;
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int l = 0; l < 3; ++l) D[k][l] += wi[k] * vj[l];
        }
      float *o = dg + 9ll * (lb + b);
      if (b < d) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int l = 0; l < 3; ++l) o[3 * k + l] = ct * D[k][l];
      } else {
        const float *rw = raw + 9ll * (lb + b);
        float *q = dd + 6ll * i;
        if (zero) {
          for (int k = 0; k < 6; ++k) q[k] = 0.f;
        } else {
          q[0] = ct * D[0][0] * expf(rw[0]) - cl;
          q[1] = ct * D[1][1] * expf(rw[1]) - cl;
          q[2] = ct * D[2][2] * expf(rw[2]) - cl;
          q[3] = ct * D[1][0];
          q[4] = ct * D[2][0];
          q[5] = ct * D[2][1];
        }
        for (int k = 0; k < 9; ++k) o[k] = 0.f;
      }
    }
  }
}

// Head backward, rows: dS_v, dh_v from the diagonal head, and per lower block
// the edge input, z and dpre (for the weight gradients). One warp per vertex.
__global__ void __launch_bounds__(256)
k_lp_head_bwd(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const int *__restrict__ diag_pos,
              const int *__restrict__ lrp, const unsigned char *__restrict__ pinned, const float *__restrict__ fe,
              const float *__restrict__ st, const float *__restrict__ Wf, const float *__restrict__ bf,
              const float *__restrict__ Wo, const float *__restrict__ Wd, const float *__restrict__ dg,
              const float *__restrict__ dd, float *__restrict__ dst, float *__restrict__ dh,
              float *__restrict__ e_h, float *__restrict__ z_h, float *__restrict__ dpre_h) {
  const int lane = threadIdx.x & 31;
  const int c = 2 * lane;
  const EdgeW ew(Wf, bf, c);
  for (int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nV; v += (gridDim.x * blockDim.x) >> 5) {
    const bool pv = pinned && pinned[v];
    const int rb = brp[v], d = diag_pos[v], lb = lrp[v];
    const float2 S = reinterpret_cast<const float2 *>(st + 2ll * kH * v)[lane];
    float ds0 = 0.f, ds1 = 0.f;
    for (int b = 0; b <= d; ++b) {
      const int j = __ldg(bcol + rb + b);
      const int64_t l = lb + b;
      const bool zero = pv || (pinned && pinned[j]) || b == d;
      float z0 = 0.f, z1 = 0.f, q0 = 0.f, q1 = 0.f;
      if (!zero) {
        float r0, r1;
        ew.apply(fe + (int64_t)kFe * (rb + b), r0, r1);
        const float2 T = reinterpret_cast<const float2 *>(st + 2ll * kH * j + kH)[lane];
        const float p0 = S.x + T.x + r0, p1 = S.y + T.y + r1;
        z0 = fmaxf(p0, 0.f);
        z1 = fmaxf(p1, 0.f);
        const float *g = dg + 9 * l;
        float dz0 = 0.f, dz1 = 0.f;
#pragma unroll
        for (int o = 0; o < 9; ++o) {
          dz0 += Wo[c * 9 + o] * g[o];
          dz1 += Wo[(c + 1) * 9 + o] * g[o];
        }
        q0 = p0 > 0.f ? dz0 : 0.f;
        q1 = p1 > 0.f ? dz1 : 0.f;
        ds0 += q0;
        ds1 += q1;
      }
      z_h[kH * l + c] = z0;
      z_h[kH * l + c + 1] = z1;
      dpre_h[kH * l + c] = q0;
      dpre_h[kH * l + c + 1] = q1;
      if (lane < kDe) e_h[kDe * l + lane] = zero ? 0.f : fe[(int64_t)kFe * (rb + b) + lane];
    }
    dst[2ll * kH * v + c] = ds0;
    dst[2ll * kH * v + c + 1] = ds1;
    float h0 = 0.f, h1 = 0.f;
    if (!pv) {
      const float *q = dd + 6ll * v;
#pragma unroll
      for (int o = 0; o < 6; ++o) {
        h0 += Wd[c * 6 + o] * q[o];
        h1 += Wd[(c + 1) * 6 + o] * q[o];
      }
    }
    dh[(int64_t)kH * v + c] = h0;
    dh[(int64_t)kH * v + c + 1] = h1;
  }
}

// Head backward, columns: dT_j = sum over lower blocks (i, j), i > j, of dpre.
__global__ void __launch_bounds__(256)
k_lp_head_bwd_t(int nV, const int *__restrict__ brp, const int *__restrict__ diag_pos, const int *__restrict__ urp,
                const int *__restrict__ up2low, const float *__restrict__ dpre_h, float *__restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const int c = 2 * lane;
  for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < nV; j += (gridDim.x * blockDim.x) >> 5) {
    const int nu = brp[j + 1] - brp[j] - diag_pos[j];
    float t0 = 0.f, t1 = 0.f;
    for (int m = 1; m < nu; ++m) {
      const int64_t l = up2low[urp[j] + m];
      t0 += dpre_h[kH * l + c];
      t1 += dpre_h[kH * l + c + 1];
    }
    dst[2ll * kH * j + kH + c] = t0;
    dst[2ll * kH * j + kH + c + 1] = t1;
  }
}

// Message backward, rows: dm_v = da_v / deg_v, dpre per directed edge, dP_v.
__global__ void __launch_bounds__(256)
k_lp_msg_bwd(int nV, const int *__restrict__ brp, const int *__restrict__ bcol,
             const unsigned char *__restrict__ pinned, const float *__restrict__ fe, const float *__restrict__ invdeg,
             const float *__restrict__ pq, const float *__restrict__ We, const float *__restrict__ be,
             const float *__restrict__ dha, float *__restrict__ dpre_e, float *__restrict__ dpq) {
  const int lane = threadIdx.x & 31;
  const int c = 2 * lane;
  const EdgeW ew(We, be, c);
  for (int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nV; v += (gridDim.x * blockDim.x) >> 5) {
    const bool pv = pinned && pinned[v];
    const int rb = brp[v], re = brp[v + 1];
    const float2 P = reinterpret_cast<const float2 *>(pq + 2ll * kH * v)[lane];
    const float s = invdeg[v];
    const float dm0 = dha[2ll * kH * v + kH + c] * s, dm1 = dha[2ll * kH * v + kH + c + 1] * s;
    float dp0 = 0.f, dp1 = 0.f;
    for (int p = rb; p < re; ++p) {
      const int j = __ldg(bcol + p);
      float q0 = 0.f, q1 = 0.f;
      if (!pv && j != v && !(pinned && pinned[j])) {
        float r0, r1;
        ew.apply(fe + (int64_t)kFe * p, r0, r1);
        const float2 Q = reinterpret_cast<const float2 *>(pq + 2ll * kH * j + kH)[lane];
        q0 = (P.x + Q.x + r0) > 0.f ? dm0 : 0.f;
        q1 = (P.y + Q.y + r1) > 0.f ? dm1 : 0.f;
        dp0 += q0;
        dp1 += q1;
      }
      dpre_e[(int64_t)kH * p + c] = q0;
      dpre_e[(int64_t)kH * p + c + 1] = q1;
    }
    dpq[2ll * kH * v + c] = dp0;
    dpq[2ll * kH * v + c + 1] = dp1;
  }
}

// Message backward, columns: dQ_j = sum over directed edges (i -> j) of dpre.
__global__ void __launch_bounds__(256)
k_lp_msg_bwd_t(int nV, const int *__restrict__ brp, const int *__restrict__ rev, const float *__restrict__ dpre_e,
               float *__restrict__ dpq) {
  const int lane = threadIdx.x & 31;
  const int c = 2 * lane;
  for (int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < nV; j += (gridDim.x * blockDim.x) >> 5) {
    float q0 = 0.f, q1 = 0.f;
    for (int p = brp[j]; p < brp[j + 1]; ++p) {
      const int64_t r = rev[p];
      q0 += dpre_e[kH * r + c];
      q1 += dpre_e[kH * r + c + 1];
    }
    dpq[2ll * kH * j + kH + c] = q0;
    dpq[2ll * kH * j + kH + c + 1] = q1;
  }
}

// elementwise helpers
__global__ void k_lp_relu_mask(int64_t n, const float *__restrict__ pre, const float *__restrict__ g,
                               float *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = pre[i] > 0.f ? g[i] : 0.f;
}
__global__ void k_lp_to_bf16(int64_t n, const float *__restrict__ a, __nv_bfloat16 *__restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}
// FP32 copy of the lower storage without row padding (9 per lower block, three
// scalar rows of 3 nl entries per vertex)
__global__ void k_lp_unpad(int nV, const int4 *__restrict__ meta, const int *__restrict__ lrp,
                           const __nv_bfloat16 *__restrict__ gl, float *__restrict__ out) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int4 m = meta[v];
    const int nl = (m.w & 0xFFFF) + 1, rs = 3 * nl, rsp = padded_row(nl);
    float *o = out + 9ll * lrp[v];
    for (int k = 0; k < 3; ++k)
      for (int e = 0; e < rs; ++e) o[k * rs + e] = __bfloat162float(gl[m.y + k * rsp + e]);
  }
}
// dh += dha[:, 0:64]
__global__ void k_lp_add_left(int nV, const float *__restrict__ dha, float *__restrict__ dh) {
  const int64_t n = (int64_t)nV * kH;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dh[i] += dha[(i / kH) * 2 * kH + (i % kH)];
}

// Weight gradient partials: out[k][n] = sum_r A[r][k] * B[r][n] over the
// block's row range (A == nullptr means a column of ones: bias gradient).
template <class TB>
__global__ void __launch_bounds__(256)
k_lp_outer(int64_t R, int K, int N, const float *__restrict__ A, int lda, const TB *__restrict__ B, int ldb,
           int64_t rows_per_block, float *__restrict__ part) {
  const int64_t r0 = blockIdx.x * rows_per_block;
  const int64_t r1 = r0 + rows_per_block < R ? r0 + rows_per_block : R;
  const int KN = K * N;
  for (int o = threadIdx.x; o < KN; o += blockDim.x) {
    const int k = o / N, nn = o - k * N;
    float acc = 0.f;
    for (int64_t r = r0; r < r1; ++r) {
      const float a = A ? A[r * lda + k] : 1.f;
      acc += a * (float)B[r * ldb + nn];
    }
    part[(int64_t)blockIdx.x * KN + o] = acc;
  }
}
__global__ void k_lp_outer_sum(int nparts, int KN, const float *__restrict__ part, float *__restrict__ out) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < KN; o += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int g = 0; g < nparts; ++g) s += part[(int64_t)g * KN + o];
    out[o] = s;
  }
}

// gradient norm^2 (fixed order) and Adam with global-norm clipping
__global__ void k_lp_gnorm(int n, const float *__restrict__ g, double *__restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)g[i] * g[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}
__global__ void k_lp_adam(int n, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                          const double *__restrict__ gn2, float clip) {
  const double gn = sqrt(*gn2);
  const float sc = (clip > 0.f && gn > clip) ? (float)(clip / gn) : 1.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i] * sc;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_lp_scale_probe(int64_t n, const double *__restrict__ nrm2, float *__restrict__ w) {
  const float sc = *nrm2 > 0.0 ? (float)sqrt((double)n / *nrm2) : 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] *= sc;
}

// BF16 copies of the GEMM weights: forward (as stored, out x in) and transposed
__global__ void k_lp_weights_bf16(const float *__restrict__ P, __nv_bfloat16 *__restrict__ wb, int nmat,
                                  const int *__restrict__ src, const int *__restrict__ dst,
                                  const int *__restrict__ rows, const int *__restrict__ transpose) {
  for (int mtx = 0; mtx < nmat; ++mtx) {
    const int R = rows[mtx], C = 8192 / R;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 8192; i += gridDim.x * blockDim.x) {
      const int r = i / C, c = i - r * C;  // source element (r, c) of an R x C matrix
      const __nv_bfloat16 b = __float2bfloat16_rn(P[src[mtx] + i]);
      if (transpose[mtx]) wb[dst[mtx] + c * R + r] = b;
      else wb[dst[mtx] + i] = b;
    }
  }
}

// ================================================================= host ===
static int grid_for_n(bartels_ctx ctx, int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  int64_t cap = (int64_t)ctx->num_sms * 16;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}
static int grid_warps(bartels_ctx ctx, int64_t nwarps) { return grid_for_n(ctx, nwarps * 32, 256); }

template <class T>
static int lp_alloc(LpcgPlanState &s, T **p, size_t n) {
  void *q = nullptr;
  BT_CUDA(cudaMalloc(&q, sizeof(T) * std::max<size_t>(n, 1)));
  s.allocs.push_back(q);
  *p = static_cast<T *>(q);
  return BARTELS_OK;
}

static void lp_state_free(LpcgPlanState *s) {
  if (!s) return;
  for (void *p : s->allocs) cudaFree(p);
  delete s;
}

static int lp_state(bartels_mesh_plan plan, bool train, int nprobe, LpcgPlanState **out) {
  FactorPattern *fp;
  BT_CHECK(plan_factor_pattern(plan, &fp));
  LpcgPlanState *s = plan->lpcg;
  if (s && (s->train || !train) && (!train || s->nprobe >= nprobe)) {
    *out = s;
    return BARTELS_OK;
  }
  lp_state_free(s);
  plan->lpcg = nullptr;
  s = new LpcgPlanState();
  plan->lpcg = s;
  const size_t nV = plan->nV, nnzb = plan->nnzb, nnzl = fp->nnzl;
  s->nV = plan->nV;
  s->nnzb = plan->nnzb;
  s->nnzl = fp->nnzl;
  s->nnzu = fp->nnzu;
  s->train = train;
  s->nprobe = nprobe;
  BT_CHECK(lp_alloc(*s, &s->fe, kFe * nnzb));
  BT_CHECK(lp_alloc(*s, &s->linv, 6 * nV));
  BT_CHECK(lp_alloc(*s, &s->xn, kDx * nV));
  BT_CHECK(lp_alloc(*s, &s->invdeg, nV));
  const int nh = train ? kLayers + 1 : 2;
  for (int l = 0; l < nh; ++l) BT_CHECK(lp_alloc(*s, &s->h[l], kH * nV));
  for (int l = nh; l <= kLayers; ++l) s->h[l] = s->h[l % 2];
  const int na = train ? kLayers + 1 : 2;
  for (int l = 0; l < na; ++l) BT_CHECK(lp_alloc(*s, &s->ha[l], 2 * kH * nV));
  for (int l = na; l <= kLayers; ++l) s->ha[l] = s->ha[l % 2];
  const int np = train ? kLayers : 1;
  for (int l = 0; l < np; ++l) {
    BT_CHECK(lp_alloc(*s, &s->pq[l], 2 * kH * nV));
    BT_CHECK(lp_alloc(*s, &s->upre[l], kH * nV));
  }
  for (int l = np; l < kLayers; ++l) {
    s->pq[l] = s->pq[0];
    s->upre[l] = s->upre[0];
  }
  BT_CHECK(lp_alloc(*s, &s->pre0, kH * nV));
  BT_CHECK(lp_alloc(*s, &s->st, 2 * kH * nV));
  BT_CHECK(lp_alloc(*s, &s->raw, 9 * nnzl));
  BT_CHECK(lp_alloc(*s, &s->gl, (size_t)fp->lsize));
  BT_CHECK(lp_alloc(*s, &s->gu, (size_t)fp->usize));
  BT_CUDA(cudaMemsetAsync(s->gl, 0, 2 * (size_t)fp->lsize, plan->ctx->stream));  // padding stays zero
  BT_CUDA(cudaMemsetAsync(s->gu, 0, 2 * (size_t)fp->usize, plan->ctx->stream));
  if (train) {
    BT_CHECK(lp_alloc(*s, &s->dh, kH * nV));
    BT_CHECK(lp_alloc(*s, &s->dha, 2 * kH * nV));
    BT_CHECK(lp_alloc(*s, &s->du, kH * nV));
    BT_CHECK(lp_alloc(*s, &s->dpq, 2 * kH * nV));
    BT_CHECK(lp_alloc(*s, &s->dst, 2 * kH * nV));
    BT_CHECK(lp_alloc(*s, &s->dbf, 2 * kH * nV));
    BT_CHECK(lp_alloc(*s, &s->dpre_e, kH * nnzb));
    BT_CHECK(lp_alloc(*s, &s->dpre_h, kH * nnzl));
    BT_CHECK(lp_alloc(*s, &s->z_h, kH * nnzl));
    BT_CHECK(lp_alloc(*s, &s->e_h, kDe * nnzl));
    BT_CHECK(lp_alloc(*s, &s->dg, 9 * nnzl));
    BT_CHECK(lp_alloc(*s, &s->dd, 6 * nV));
    BT_CHECK(lp_alloc(*s, &s->wprobe, (size_t)nprobe * 3 * nV));
    BT_CHECK(lp_alloc(*s, &s->uprobe, (size_t)nprobe * 3 * nV));
    BT_CHECK(lp_alloc(*s, &s->vprobe, (size_t)nprobe * 3 * nV));
  }
  *out = s;
  return BARTELS_OK;
}

void lpcg_plan_release(bartels_mesh_plan plan) {
  lp_state_free(plan->lpcg);
  plan->lpcg = nullptr;
}

static int lp_refresh_bf16(bartels_lpcg net) {
  if (!net->bf_dirty) return BARTELS_OK;
  bartels_ctx ctx = net->ctx;
  // matrices: (source offset, destination offset, source rows, transpose)
  int src[4 * kLayers + 2], dst[4 * kLayers + 2], rows[4 * kLayers + 2], tr[4 * kLayers + 2];
  int k = 0;
  for (int l = 0; l < kLayers; ++l) {
    src[k] = kL.Wpq[l]; dst[k] = kB.pq[l]; rows[k] = 128; tr[k++] = 0;
    src[k] = kL.Wpq[l]; dst[k] = kB.pqT[l]; rows[k] = 128; tr[k++] = 1;
    src[k] = kL.Wu[l]; dst[k] = kB.u[l]; rows[k] = 64; tr[k++] = 0;
    src[k] = kL.Wu[l]; dst[k] = kB.uT[l]; rows[k] = 64; tr[k++] = 1;
  }
  src[k] = kL.Wst; dst[k] = kB.st; rows[k] = 128; tr[k++] = 0;
  src[k] = kL.Wst; dst[k] = kB.stT; rows[k] = 128; tr[k++] = 1;
  int *d = nullptr;
  BT_CHECK(ctx->scalars.ensure(sizeof(int) * 4 * k));
  d = ctx->scalars.as<int>();
  std::vector<int> h(4 * k);
  for (int i = 0; i < k; ++i) {
    h[i] = src[i];
    h[k + i] = dst[i];
    h[2 * k + i] = rows[i];
    h[3 * k + i] = tr[i];
  }
  BT_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(int) * 4 * k, cudaMemcpyHostToDevice, ctx->stream));
  BT_LAUNCH(ctx, k_lp_weights_bf16, 32, 256, 0, net->params, net->wbf, k, d, d + k, d + 2 * k, d + 3 * k);
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  net->bf_dirty = false;
  return BARTELS_OK;
}

static int lp_gemm(bartels_lpcg net, int M, int N, int K, const __nv_bfloat16 *x, int ldx, int wofs,
                   const float *bias, const float *resid, int ldr, int relu, float *ypre, int ldp, float *y, int ldy,
                   __nv_bfloat16 *y2, int ldy2) {
  GemmArgs g;
  g.M = M;
  g.N = N;
  g.K = K;
  g.x = x;
  g.ldx = ldx;
  g.w = net->wbf + wofs;
  g.bias = bias;
  g.resid = resid;
  g.ldr = ldr;
  g.relu = relu;
  g.ypre = ypre;
  g.ldp = ldp;
  g.y = y;
  g.ldy = ldy;
  g.y2 = y2;
  g.ldy2 = ldy2;
  g.err = net->err;
  return gemm_bf16(net->ctx, g);
}

// Forward pass on the plan's current Hessian values (scalar-CSR order, FP32):
// fills s->gl / s->gu with the factor G (lower and upper storage).
static int lp_forward(bartels_lpcg net, bartels_mesh_plan plan, LpcgPlanState *s, const float *vals) {
  bartels_ctx ctx = net->ctx;
  FactorPattern *fp = plan->factor;
  const int nV = plan->nV;
  const float *P = net->params;
  BT_CHECK(lp_refresh_bf16(net));
  const int gv = grid_for_n(ctx, nV, 256), gw = grid_warps(ctx, nV);
  BT_LAUNCH(ctx, k_lp_linv, gv, 256, 0, nV, plan->brp, plan->diag_pos, vals, plan->pinned, s->linv);
  BT_LAUNCH(ctx, k_lp_feats, grid_warps(ctx, (nV + 1) / 2), 256, 0, nV, plan->brp, plan->bcol, vals, plan->pinned,
            s->linv, s->fe, s->xn, s->invdeg);
  BT_LAUNCH(ctx, k_lp_embed, gw, 256, 0, nV, s->xn, P + kL.W0, P + kL.b0, s->train ? s->pre0 : nullptr, s->h[0],
            s->ha[0]);
  for (int l = 0; l < kLayers; ++l) {
    // [P | Q] = bf16(h) Wpq^T
    BT_CHECK(lp_gemm(net, nV, 128, 64, s->ha[l], 128, kB.pq[l], nullptr, nullptr, 0, 0, nullptr, 0, s->pq[l], 128,
                     nullptr, 0));
    BT_LAUNCH(ctx, k_lp_msg, gw, 256, 0, nV, plan->brp, plan->bcol, plan->pinned, s->fe, s->invdeg, s->pq[l],
              P + kL.We[l], P + kL.be[l], s->ha[l]);
    // U = bf16([h | a]) Wu^T + bu (pre-activation kept), h' = h + relu(U)
    BT_CHECK(lp_gemm(net, nV, 64, 128, s->ha[l], 128, kB.u[l], P + kL.bu[l], s->h[l], 64, 1,
                     s->train ? s->upre[l] : nullptr, 64, s->h[l + 1], 64, s->ha[l + 1], 128));
  }
  BT_CHECK(lp_gemm(net, nV, 128, 64, s->ha[kLayers], 128, kB.st, nullptr, nullptr, 0, 0, nullptr, 0, s->st, 128,
                   nullptr, 0));
  BT_LAUNCH(ctx, k_lp_head, grid_for_n(ctx, nV, kHeadThreads), kHeadThreads, 0, nV, plan->brp, plan->bcol,
            plan->diag_pos, fp->lrp, fp->meta, plan->pinned, s->fe,
            s->linv, s->h[kLayers], s->st, P + kL.Wf, P + kL.bf, P + kL.Wo, P + kL.bo, P + kL.Wd, P + kL.bd,
            P + kL.Wskip, s->raw, s->gl);
  BT_LAUNCH(ctx, k_factor_transpose, gv, 256, 0, nV, plan->bcol, fp->meta, fp->lrp, fp->urp, fp->low2up, s->gl,
            s->gu);
  return BARTELS_OK;
}

}  // namespace bartels

namespace bartels {

int lpcg_factor(bartels_lpcg net, bartels_mesh_plan plan, const float *values, const __nv_bfloat16 **gl,
                const __nv_bfloat16 **gu) {
  LpcgPlanState *s;
  BT_CHECK(lp_state(plan, false, 0, &s));
  BT_CHECK(lp_forward(net, plan, s, values));
  *gl = s->gl;
  *gu = s->gu;
  return BARTELS_OK;
}

template <class TB>
static int lp_outer(bartels_lpcg net, int64_t R, int K, int N, const float *A, int lda, const TB *B, int ldb,
                    float *out) {
  bartels_ctx ctx = net->ctx;
  const int64_t target = std::max<int64_t>(1, (R + 63) / 64);
  const int nparts = (int)std::min<int64_t>(target, 512);
  const int64_t rpb = (R + nparts - 1) / nparts;
  BT_CHECK(net->part.ensure(sizeof(float) * (size_t)nparts * K * N));
  float *part = net->part.as<float>();
  BT_LAUNCH(ctx, k_lp_outer<TB>, nparts, 256, 0, R, K, N, A, lda, B, ldb, rpb, part);
  BT_LAUNCH(ctx, k_lp_outer_sum, (K * N + 255) / 256, 256, 0, nparts, K * N, part, out);
  return BARTELS_OK;
}

static int lp_to_bf16(bartels_ctx ctx, int64_t n, const float *a, __nv_bfloat16 *b) {
  BT_LAUNCH(ctx, k_lp_to_bf16, grid_for_n(ctx, n, 256), 256, 0, n, a, b);
  return BARTELS_OK;
}

// Loss and gradient (net->grad) on one system; probes: nrand Rademacher vectors
// from `seed`, plus the residual r64 (device, FP64) when given.
static int lp_loss_grad(bartels_lpcg net, bartels_mesh_plan plan, const float *vals, const double *r64, int nrand,
                        uint32_t seed, double *loss, double *trace_out) {
  bartels_ctx ctx = net->ctx;
  const int np = nrand + (r64 ? 1 : 0);
  if (np < 1) return fail(BARTELS_E_INVALID_ARG, "at least one probe vector is needed");
  LpcgPlanState *s;
  BT_CHECK(lp_state(plan, true, np, &s));
  FactorPattern *fp = plan->factor;
  const int nV = plan->nV;
  const int64_t n3 = 3ll * nV;
  const float *P = net->params;
  float *G = net->grad;
  BT_CHECK(lp_forward(net, plan, s, vals));
  const int gv = grid_for_n(ctx, nV, 256), gw = grid_warps(ctx, nV);
  // probes
  BT_LAUNCH(ctx, k_lp_probes, grid_for_n(ctx, n3, 256), 256, 0, nV, nrand, seed, plan->pinned, s->wprobe);
  if (r64) {
    float *w = s->wprobe + (int64_t)nrand * n3;
    BT_LAUNCH(ctx, k_lp_resid_probe, gv, 256, 0, nV, r64, s->linv, plan->pinned, w);
    BT_LAUNCH(ctx, k_lp_gnorm, 1, 256, 0, (int)n3, w, net->scal + 4);
    BT_LAUNCH(ctx, k_lp_scale_probe, grid_for_n(ctx, n3, 256), 256, 0, n3, net->scal + 4, w);
  }
  // trace estimate and loss
  BT_LAUNCH(ctx, k_lp_gt_apply, gv, 256, 0, nV, np, plan->brp, plan->bcol, plan->diag_pos, fp->urp, fp->up2low,
            plan->pinned, s->raw, s->wprobe, s->uprobe);
  BT_CHECK(net->ctx->partials.ensure(sizeof(double) * 3 * (size_t)gv));
  double *lpart = net->ctx->partials.as<double>();
  BT_LAUNCH(ctx, k_lp_ahat_apply, gv, 256, 0, nV, np, plan->brp, plan->bcol, plan->diag_pos, fp->lrp, plan->pinned,
            s->fe, s->raw, s->uprobe, s->vprobe, lpart);
  BT_LAUNCH(ctx, k_lp_loss_sum, 1, 32, 0, gv, np, lpart, net->scal);
  BT_LAUNCH(ctx, k_lp_dghat, gv, 256, 0, nV, np, plan->brp, plan->bcol, plan->diag_pos, fp->lrp, plan->pinned, s->raw,
            s->wprobe, s->vprobe, net->scal, s->dg, s->dd);
  // head backward
  BT_LAUNCH(ctx, k_lp_head_bwd, gw, 256, 0, nV, plan->brp, plan->bcol, plan->diag_pos, fp->lrp, plan->pinned, s->fe,
            s->st, P + kL.Wf, P + kL.bf, P + kL.Wo, P + kL.Wd, s->dg, s->dd, s->dst, s->dh, s->e_h, s->z_h,
            s->dpre_h);
  BT_LAUNCH(ctx, k_lp_head_bwd_t, gw, 256, 0, nV, plan->brp, plan->diag_pos, fp->urp, fp->up2low, s->dpre_h, s->dst);
  const int64_t nl = s->nnzl;
  BT_CHECK(lp_outer<float>(net, nl, kDe, kH, s->e_h, kDe, s->dpre_h, kH, G + kL.Wf));
  BT_CHECK(lp_outer<float>(net, nl, 1, kH, nullptr, 0, s->dpre_h, kH, G + kL.bf));
  BT_CHECK(lp_outer<float>(net, nl, kH, 9, s->z_h, kH, s->dg, 9, G + kL.Wo));
  BT_CHECK(lp_outer<float>(net, nl, 1, 9, nullptr, 0, s->dg, 9, G + kL.bo));
  BT_CHECK(lp_outer<float>(net, nl, kDe, 9, s->e_h, kDe, s->dg, 9, G + kL.Wskip));
  BT_CHECK(lp_outer<float>(net, nV, kH, 6, s->h[kLayers], kH, s->dd, 6, G + kL.Wd));
  BT_CHECK(lp_outer<float>(net, nV, 1, 6, nullptr, 0, s->dd, 6, G + kL.bd));
  BT_CHECK(lp_outer<__nv_bfloat16>(net, nV, 2 * kH, kH, s->dst, 2 * kH, s->ha[kLayers], 2 * kH, G + kL.Wst));
  BT_CHECK(lp_to_bf16(ctx, 2ll * kH * nV, s->dst, s->dbf));
  BT_CHECK(lp_gemm(net, nV, 64, 128, s->dbf, 128, kB.stT, nullptr, s->dh, 64, 0, nullptr, 0, s->dh, 64, nullptr, 0));
  // message-passing layers, last to first
  for (int l = kLayers - 1; l >= 0; --l) {
    BT_LAUNCH(ctx, k_lp_relu_mask, grid_for_n(ctx, (int64_t)kH * nV, 256), 256, 0, (int64_t)kH * nV, s->upre[l], s->dh,
              s->du);
    BT_CHECK(lp_outer<__nv_bfloat16>(net, nV, kH, 2 * kH, s->du, kH, s->ha[l], 2 * kH, G + kL.Wu[l]));
    BT_CHECK(lp_outer<float>(net, nV, 1, kH, nullptr, 0, s->du, kH, G + kL.bu[l]));
    BT_CHECK(lp_to_bf16(ctx, (int64_t)kH * nV, s->du, s->dbf));
    BT_CHECK(lp_gemm(net, nV, 128, 64, s->dbf, 64, kB.uT[l], nullptr, nullptr, 0, 0, nullptr, 0, s->dha, 128, nullptr,
                     0));
    BT_LAUNCH(ctx, k_lp_add_left, grid_for_n(ctx, (int64_t)kH * nV, 256), 256, 0, nV, s->dha, s->dh);
    BT_LAUNCH(ctx, k_lp_msg_bwd, gw, 256, 0, nV, plan->brp, plan->bcol, plan->pinned, s->fe, s->invdeg, s->pq[l],
              P + kL.We[l], P + kL.be[l], s->dha, s->dpre_e, s->dpq);
    BT_LAUNCH(ctx, k_lp_msg_bwd_t, gw, 256, 0, nV, plan->brp, fp->rev, s->dpre_e, s->dpq);
    BT_CHECK(lp_outer<float>(net, s->nnzb, kDe, kH, s->fe, kFe, s->dpre_e, kH, G + kL.We[l]));
    BT_CHECK(lp_outer<float>(net, s->nnzb, 1, kH, nullptr, 0, s->dpre_e, kH, G + kL.be[l]));
    BT_CHECK(lp_outer<__nv_bfloat16>(net, nV, 2 * kH, kH, s->dpq, 2 * kH, s->ha[l], 2 * kH, G + kL.Wpq[l]));
    BT_CHECK(lp_to_bf16(ctx, 2ll * kH * nV, s->dpq, s->dbf));
    BT_CHECK(lp_gemm(net, nV, 64, 128, s->dbf, 128, kB.pqT[l], nullptr, s->dh, 64, 0, nullptr, 0, s->dh, 64, nullptr,
                     0));
  }
  // embedding
  BT_LAUNCH(ctx, k_lp_relu_mask, grid_for_n(ctx, (int64_t)kH * nV, 256), 256, 0, (int64_t)kH * nV, s->pre0, s->dh,
            s->du);
  BT_CHECK(lp_outer<float>(net, nV, kDx, kH, s->xn, kDx, s->du, kH, G + kL.W0));
  BT_CHECK(lp_outer<float>(net, nV, 1, kH, nullptr, 0, s->du, kH, G + kL.b0));
  // loss on the host
  double sc[3];
  BT_CUDA(cudaMemcpyAsync(sc, net->scal, sizeof(sc), cudaMemcpyDeviceToHost, ctx->stream));
  int gerr = 0;
  BT_CUDA(cudaMemcpyAsync(&gerr, net->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  if (gerr) return fail(BARTELS_E_TIMEOUT, "tensor-core GEMM: a bounded wait gave up");
  if (!(sc[0] > 0.0) || !(sc[2] > 0.0)) return fail(BARTELS_E_NONFINITE, "preconditioner loss: empty or invalid trace");
  *loss = std::log(sc[0] / sc[2]) - 2.0 * sc[1] / sc[2];
  if (trace_out) *trace_out = sc[0];
  return BARTELS_OK;
}

static int lp_adam(bartels_lpcg net, float lr, float clip) {
  bartels_ctx ctx = net->ctx;
  net->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)net->step), c2 = 1.f - std::pow(b2, (float)net->step);
  BT_LAUNCH(ctx, k_lp_gnorm, 1, 256, 0, kL.total, net->grad, net->scal + 3);
  BT_LAUNCH(ctx, k_lp_adam, grid_for_n(ctx, kL.total, 256), 256, 0, kL.total, net->params, net->grad, net->m, net->v,
            lr, b1, b2, 1e-8f, c1, c2, net->scal + 3, clip);
  net->bf_dirty = true;
  return BARTELS_OK;
}

}  // namespace bartels

using namespace bartels;

int lpcg_create(bartels_ctx ctx, bartels_lpcg *out) {
  bartels_lpcg n = new bartels_lpcg_s();
  n->ctx = ctx;
  const size_t P = kL.total;
  cudaError_t e = cudaSuccess;
  e = e == cudaSuccess ? cudaMalloc(&n->params, 4 * P) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->grad, 4 * P) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->m, 4 * P) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->v, 4 * P) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->wbf, 2 * (size_t)kB.total) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->err, sizeof(int)) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->scal, 8 * sizeof(double)) : e;
  if (e == cudaSuccess) e = cudaMemsetAsync(n->params, 0, 4 * P, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n->grad, 0, 4 * P, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n->m, 0, 4 * P, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n->v, 0, 4 * P, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n->err, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    lpcg_destroy(n);
    return fail(BARTELS_E_DEVICE, std::string("learned preconditioner allocation: ") + cudaGetErrorString(e));
  }
  *out = n;
  return BARTELS_OK;
}

void lpcg_destroy(bartels_lpcg n) {
  if (!n) return;
  void *ptrs[] = {n->params, n->grad, n->m, n->v, n->wbf, n->err, n->scal};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  n->part.release();
  delete n;
}

int lpcg_num_params() { return kL.total; }
bartels_ctx lpcg_ctx(bartels_lpcg n) { return n->ctx; }

int lpcg_set_params(bartels_lpcg n, const float *host) {
  BT_CUDA(cudaMemcpyAsync(n->params, host, 4 * (size_t)kL.total, cudaMemcpyHostToDevice, n->ctx->stream));
  BT_CUDA(cudaMemsetAsync(n->m, 0, 4 * (size_t)kL.total, n->ctx->stream));
  BT_CUDA(cudaMemsetAsync(n->v, 0, 4 * (size_t)kL.total, n->ctx->stream));
  BT_CUDA(cudaStreamSynchronize(n->ctx->stream));
  n->step = 0;
  n->bf_dirty = true;
  return BARTELS_OK;
}

int lpcg_get_params(bartels_lpcg n, float *host, float *grad_host) {
  if (host) BT_CUDA(cudaMemcpyAsync(host, n->params, 4 * (size_t)kL.total, cudaMemcpyDeviceToHost, n->ctx->stream));
  if (grad_host)
    BT_CUDA(cudaMemcpyAsync(grad_host, n->grad, 4 * (size_t)kL.total, cudaMemcpyDeviceToHost, n->ctx->stream));
  BT_CUDA(cudaStreamSynchronize(n->ctx->stream));
  return BARTELS_OK;
}

int lpcg_train_step(bartels_lpcg n, bartels_mesh_plan plan, const float *values_d, const double *resid_d, int nrand,
                    unsigned seed, float lr, float clip, double *loss) {
  BT_CHECK(lp_loss_grad(n, plan, values_d, resid_d, nrand, seed, loss, nullptr));
  if (lr > 0.f) BT_CHECK(lp_adam(n, lr, clip));
  return BARTELS_OK;
}

// Debug / test access: raw network outputs (9 per lower block) and G (lower storage).
int lpcg_outputs(bartels_lpcg n, bartels_mesh_plan plan, const float *values_d, float *raw_host, float *gl_host) {
  const __nv_bfloat16 *gl, *gu;
  BT_CHECK(lpcg_factor(n, plan, values_d, &gl, &gu));
  LpcgPlanState *s = plan->lpcg;
  bartels_ctx ctx = n->ctx;
  if (raw_host) BT_CUDA(cudaMemcpyAsync(raw_host, s->raw, 36 * (size_t)s->nnzl, cudaMemcpyDeviceToHost, ctx->stream));
  if (gl_host) {
    BT_CHECK(ctx->stage_d.ensure(36 * (size_t)s->nnzl));
    float *tmp = ctx->stage_d.as<float>();
    BT_LAUNCH(ctx, k_lp_unpad, grid_for_n(ctx, plan->nV, 256), 256, 0, plan->nV, plan->factor->meta,
              plan->factor->lrp, s->gl, tmp);
    BT_CUDA(cudaMemcpyAsync(gl_host, tmp, 36 * (size_t)s->nnzl, cudaMemcpyDeviceToHost, ctx->stream));
  }
  int gerr = 0;
  BT_CUDA(cudaMemcpyAsync(&gerr, n->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  if (gerr) return fail(BARTELS_E_TIMEOUT, "tensor-core GEMM: a bounded wait gave up");
  return BARTELS_OK;
}
