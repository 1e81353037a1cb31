// FP32 linear-elastic Hex8 residual / HVP on blocks of exact parallelepipeds:
// persistent CTAs, two-stage cp.async pipeline, two elements per thread in packed
// f32x2 arithmetic.
//
// Same mathematics, plan and summation order as the modal path of assemble.cu (the
// 2x2x2 Gauss sum evaluated exactly in the monomial basis of grad u through an
// 8-point Walsh-Hadamard transform); what changes is the schedule:
//   * each CTA walks its blocks b = blockIdx.x, blockIdx.x + gridDim.x, ...; while
//     block b is computed, the coordinates and the input vector of the next block
//     are gathered into the other shared-memory buffer with cp.async (4-byte
//     copies, one per value), and the node ids / partial slots of the block after
//     that are already in registers -- the HBM latency of the gathers is hidden
//     behind compute;
//   * every thread evaluates two elements at once, one per lane of f32x2 registers,
//     so each arithmetic instruction serves two elements;
//   * element results stay in registers until the colour-ordered shared-memory
//     accumulation (one barrier per colour), as in the scalar kernel.
#include "tg_common.cuh"
#include "tg_f32x2.cuh"
#include "tg_internal.h"

namespace tg {

constexpr int P5_THREADS = 128;
constexpr int P5_NPT = 6;  // staged nodes per thread per block
constexpr int P5_MAX_LOCAL = P5_THREADS * P5_NPT;

__device__ __forceinline__ int swz5(int l) { return l ^ ((l >> 3) & 7); }
__device__ __forceinline__ int hex_t5(int a) {
  return (a == 2) ? 3 : (a == 3) ? 2 : (a == 6) ? 7 : (a == 7) ? 6 : a;
}

__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait1() {
  asm volatile("cp.async.wait_group 1;" ::: "memory");
}

__device__ __forceinline__ void had8(f2 (&m)[8]) {
#pragma unroll
  for (int h = 1; h < 8; h <<= 1)
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (!(t & h)) {
        const f2 a = m[t], b = m[t | h];
        m[t] = b + a;
        m[t | h] = b - a;
      }
}
__device__ __forceinline__ void had8t(f2 (&m)[8]) {
#pragma unroll
  for (int h = 1; h < 8; h <<= 1)
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (!(t & h)) {
        const f2 a = m[t], b = m[t | h];
        m[t] = a - b;
        m[t | h] = a + b;
      }
}

__device__ __forceinline__ f2 dot3c(const f2 (&g)[3], const f2 (&R)[3][3], int c) {
  return fma2(g[2], R[2][c], fma2(g[1], R[1][c], g[0] * R[0][c]));
}

// two-direction monomial (directions P < Q), see le_two_dir in assemble.cu
template <int P, int Q>
__device__ __forceinline__ void le_two_dir2(const f2 (&R)[3][3], const f2 (&Gm)[3][3],
                                            const f2 (&gp)[3], const f2 (&gq)[3], f2 mu, f2 lam,
                                            f2 (&Fp)[3], f2 (&Fq)[3]) {
  const f2 a_pp = dot3c(gp, R, P), a_pq = dot3c(gp, R, Q);
  const f2 a_qp = dot3c(gq, R, P), a_qq = dot3c(gq, R, Q);
  const f2 lt = lam * (a_pp + a_qq);
  const f2 c1 = mu * Gm[P][P], c2 = mu * Gm[P][Q], c3 = fma2(mu, a_pp, lt), c4 = mu * a_qp;
  const f2 d2 = mu * Gm[Q][Q], d3 = mu * a_pq, d4 = fma2(mu, a_qq, lt);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Fp[j] = fma2(c4, R[j][Q], fma2(c3, R[j][P], fma2(c2, gq[j], c1 * gp[j])));
    Fq[j] = fma2(d4, R[j][Q], fma2(d3, R[j][P], fma2(d2, gq[j], c2 * gp[j])));
  }
}

// M: transformed nodal values (component j, monomial S); out: dE/dM_S (unscaled
// transform coefficients) for linear elasticity on a parallelepiped with
// R = inv(8 J) and detJm = det(8 J).
__device__ __forceinline__ void le_modal_pair(const f2 (&R)[3][3], f2 detJm, f2 mu, f2 lam,
                                              const f2 (&M)[3][8], f2 (&dM)[3][8]) {
  const float g2f = float(HEX_GAUSS) * float(HEX_GAUSS);
  const f2 s0 = detJm * f2_bcast(1.0f / 64);
  const f2 s1 = s0 * f2_bcast(g2f);
  const f2 s2 = s1 * f2_bcast(g2f);
  {  // constant monomial: directions (x, y, z) carry (M1, M2, M4)
    f2 H[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) H[j][k] = fma2(R[k][2], M[j][4], fma2(R[k][1], M[j][2], R[k][0] * M[j][1]));
    const f2 m0 = mu * s0;
    const f2 lt = (lam * s0) * (H[0][0] + H[1][1] + H[2][2]);
    f2 P[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      P[i][i] = fma2(m0, H[i][i] + H[i][i], lt);
#pragma unroll
      for (int j = i + 1; j < 3; ++j) {
        P[i][j] = m0 * (H[i][j] + H[j][i]);
        P[j][i] = P[i][j];
      }
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      dM[j][0] = f2_zero();
      dM[j][1] = fma2(P[j][2], R[2][0], fma2(P[j][1], R[1][0], P[j][0] * R[0][0]));
      dM[j][2] = fma2(P[j][2], R[2][1], fma2(P[j][1], R[1][1], P[j][0] * R[0][1]));
      dM[j][4] = fma2(P[j][2], R[2][2], fma2(P[j][1], R[1][2], P[j][0] * R[0][2]));
    }
  }
  f2 Gm[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = a; b < 3; ++b) {
      Gm[a][b] = fma2(R[2][a], R[2][b], fma2(R[1][a], R[1][b], R[0][a] * R[0][b]));
      Gm[b][a] = Gm[a][b];
    }
  const f2 mu1 = mu * s1, lam1 = lam * s1;
  f2 g12[3], g13[3], g23[3], g123[3], Fp[3], Fq[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    g12[j] = M[j][3];
    g13[j] = M[j][5];
    g23[j] = M[j][6];
    g123[j] = M[j][7];
  }
  le_two_dir2<1, 2>(R, Gm, g12, g13, mu1, lam1, Fp, Fq);  // monomial x
#pragma unroll
  for (int j = 0; j < 3; ++j) { dM[j][3] = Fp[j]; dM[j][5] = Fq[j]; }
  le_two_dir2<0, 2>(R, Gm, g12, g23, mu1, lam1, Fp, Fq);  // monomial y
#pragma unroll
  for (int j = 0; j < 3; ++j) { dM[j][3] = dM[j][3] + Fp[j]; dM[j][6] = Fq[j]; }
  le_two_dir2<0, 1>(R, Gm, g13, g23, mu1, lam1, Fp, Fq);  // monomial z
#pragma unroll
  for (int j = 0; j < 3; ++j) { dM[j][5] = dM[j][5] + Fp[j]; dM[j][6] = dM[j][6] + Fq[j]; }
  // monomials yz, xz, xy: mu tr(Gm) g + (mu + lam) R R^T g, g = M123
  const f2 mu2 = mu * s2, ml2 = (mu + lam) * s2;
  const f2 trG = Gm[0][0] + Gm[1][1] + Gm[2][2];
  f2 h[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) h[i] = dot3c(g123, R, i);
  const f2 a = mu2 * trG;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const f2 rh = fma2(R[j][2], h[2], fma2(R[j][1], h[1], R[j][0] * h[0]));
    dM[j][7] = fma2(ml2, rh, a * g123[j]);
  }
}

__device__ __forceinline__ f2 inv3_pair(const f2 (&J)[3][3], f2 (&Ji)[3][3]) {
  const f2 c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const f2 c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const f2 c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const f2 det = fma2(J[0][2], c02, fma2(J[0][1], c01, J[0][0] * c00));
  float dlo, dhi;
  f2_split(det, dlo, dhi);
  const f2 r = f2_make(__frcp_rn(dlo), __frcp_rn(dhi));
  Ji[0][0] = c00 * r;
  Ji[1][0] = c01 * r;
  Ji[2][0] = c02 * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  return det;
}

// shared-memory layout (floats), nl8 = node slots (multiple of 8):
//   buffer s (s = 0, 1) at s * 10 nl8: X (4 nl8) | W (4 nl8) | GID (nl8) | SLOT (nl8)
//   Y at 20 nl8 (4 nl8)
template <int MODE>
__global__ void __launch_bounds__(P5_THREADS, 3)
    hex_le_f32x2_kernel(const tg_block_plan p, int n_blocks, const float* __restrict__ coords,
                        const float* __restrict__ fin, const uint8_t* __restrict__ fixed,
                        const float* __restrict__ vin, float* __restrict__ y,
                        float* __restrict__ partials, float mu_s, float lam_s, int nl8) {
  extern __shared__ __align__(16) float sm[];
  float* const Ybuf = sm + 20 * nl8;
  const int tid = threadIdx.x;
  constexpr int NT = P5_THREADS;

  for (int l = tid; l < nl8; l += NT) {
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      sm[s * 10 * nl8 + l * 4 + 3] = 0.f;
      sm[s * 10 * nl8 + 4 * nl8 + l * 4 + 3] = 0.f;
    }
    reinterpret_cast<float4*>(Ybuf)[l] = make_float4(0.f, 0.f, 0.f, 0.f);
  }

  int G1[P5_NPT], S1[P5_NPT], G2[P5_NPT], S2[P5_NPT];
  auto load_gs = [&](int b, int (&G)[P5_NPT], int (&S)[P5_NPT]) {
    const int n0 = p.blk_node_ptr[b], nl = p.blk_node_ptr[b + 1] - n0;
#pragma unroll
    for (int k = 0; k < P5_NPT; ++k) {
      const int l = tid + k * NT;
      G[k] = (l < nl) ? __ldg(p.lnode_gid + n0 + l) : 0;
      S[k] = (l < nl) ? __ldg(p.lnode_slot + n0 + l) : 0;
    }
  };
  auto issue = [&](int b, int s, const int (&G)[P5_NPT], const int (&S)[P5_NPT]) {
    float* X = sm + s * 10 * nl8;
    float* W = X + 4 * nl8;
    int* GID = reinterpret_cast<int*>(X + 8 * nl8);
    int* SLOT = GID + nl8;
    const int nl = p.blk_node_ptr[b + 1] - p.blk_node_ptr[b];
#pragma unroll
    for (int k = 0; k < P5_NPT; ++k) {
      const int l = tid + k * NT;
      if (l < nl) {
        const int q = swz5(l);
        const int64_t g = G[k];
#pragma unroll
        for (int d = 0; d < 3; ++d) cp_async4(X + q * 4 + d, coords + g * 3 + d);
#pragma unroll
        for (int d = 0; d < 3; ++d) cp_async4(W + q * 4 + d, fin + g * 3 + d);
        GID[l] = G[k];
        SLOT[l] = S[k];
      }
    }
  };

  const int stride = gridDim.x;
  int b = blockIdx.x;
  if (b < n_blocks) {
    load_gs(b, G1, S1);
    issue(b, 0, G1, S1);
  }
  cp_async_commit();
  if (b + stride < n_blocks) load_gs(b + stride, G1, S1);

  const f2 mu = f2_bcast(mu_s), lam = f2_bcast(lam_s);
  for (int it = 0; b < n_blocks; ++it, b += stride) {
    const int s = it & 1;
    if (b + stride < n_blocks) issue(b + stride, s ^ 1, G1, S1);
    cp_async_commit();
    if (b + 2 * stride < n_blocks) load_gs(b + 2 * stride, G2, S2);
    cp_async_wait1();
    __syncthreads();

    const float* X = sm + s * 10 * nl8;
    float* W = const_cast<float*>(X) + 4 * nl8;
    const int* GID = reinterpret_cast<const int*>(X + 8 * nl8);
    const int* SLOT = GID + nl8;
    const int nl = p.blk_node_ptr[b + 1] - p.blk_node_ptr[b];
    if (MODE == TG_MODE_HVP && fixed) {
      for (int l = tid; l < nl; l += NT) {
        const int64_t g = GID[l];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          if (fixed[g * 3 + d]) W[swz5(l) * 4 + d] = 0.f;
      }
      __syncthreads();
    }

    const int e_base = p.blk_elem_ptr[b];
    const int ne = p.blk_elem_ptr[b + 1] - e_base;
    const int c_begin = p.blk_color_ptr[b];
    const int c_last = p.blk_color_ptr[b + 1] - 1;
    for (int k0 = 0; k0 < ne; k0 += 2 * NT) {
      const int kA = k0 + tid, kB = k0 + NT + tid;
      const bool actA = kA < ne, actB = kB < ne;
      float YA[8][3], YB[8][3];
      int qA[8], qB[8];
      if (actA) {
        int lcA[8], lcB[8];
        load_lconn<8>(p.lconn + (int64_t)(e_base + kA) * 8, lcA);
        load_lconn<8>(p.lconn + (int64_t)(e_base + (actB ? kB : kA)) * 8, lcB);
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          qA[a] = swz5(lcA[a]);
          qB[a] = swz5(lcB[a]);
        }
        f2 Jm[3][3], R[3][3];
        {
          const float4 a0 = reinterpret_cast<const float4*>(X)[qA[0]];
          const float4 b0 = reinterpret_cast<const float4*>(X)[qB[0]];
          const int ed[3] = {1, 3, 4};
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const float4 ai = reinterpret_cast<const float4*>(X)[qA[ed[i]]];
            const float4 bi = reinterpret_cast<const float4*>(X)[qB[ed[i]]];
            Jm[i][0] = f2_make(4.f * (ai.x - a0.x), 4.f * (bi.x - b0.x));
            Jm[i][1] = f2_make(4.f * (ai.y - a0.y), 4.f * (bi.y - b0.y));
            Jm[i][2] = f2_make(4.f * (ai.z - a0.z), 4.f * (bi.z - b0.z));
          }
        }
        const f2 detJm = inv3_pair(Jm, R);
        f2 M[3][8];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          const float4 wa = reinterpret_cast<const float4*>(W)[qA[a]];
          const float4 wb = reinterpret_cast<const float4*>(W)[qB[a]];
          M[0][hex_t5(a)] = f2_make(wa.x, wb.x);
          M[1][hex_t5(a)] = f2_make(wa.y, wb.y);
          M[2][hex_t5(a)] = f2_make(wa.z, wb.z);
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) had8(M[j]);
        f2 dM[3][8];
        le_modal_pair(R, detJm, mu, lam, M, dM);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          had8t(dM[j]);
#pragma unroll
          for (int a = 0; a < 8; ++a) f2_split(dM[j][hex_t5(a)], YA[a][j], YB[a][j]);
        }
      }
      for (int c = c_begin; c < c_last; ++c) {
        const int lo = max(p.color_ofs[c], k0);
        const int hi = min(p.color_ofs[c + 1], k0 + 2 * NT);
        if (lo >= hi) continue;  // uniform over the block
        if (actA && kA >= lo && kA < hi) {
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            float4* yp = reinterpret_cast<float4*>(Ybuf) + qA[a];
            const float4 o = *yp;
            *yp = make_float4(o.x + YA[a][0], o.y + YA[a][1], o.z + YA[a][2], 0.f);
          }
        }
        if (actB && kB >= lo && kB < hi) {
#pragma unroll
          for (int a = 0; a < 8; ++a) {
            float4* yp = reinterpret_cast<float4*>(Ybuf) + qB[a];
            const float4 o = *yp;
            *yp = make_float4(o.x + YB[a][0], o.y + YB[a][1], o.z + YB[a][2], 0.f);
          }
        }
        __syncthreads();
      }
    }

    // write back this block and clear the accumulator
    for (int l = tid; l < nl; l += NT) {
      const int q = swz5(l);
      float4* yp = reinterpret_cast<float4*>(Ybuf) + q;
      const float4 yv = *yp;
      *yp = make_float4(0.f, 0.f, 0.f, 0.f);
      const int64_t g = GID[l];
      const int slot = SLOT[l];
      const float vals[3] = {yv.x, yv.y, yv.z};
      if (slot < 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int64_t dof = g * 3 + d;
          float val = vals[d];
          if (fixed && fixed[dof]) val = (MODE == TG_MODE_HVP) ? vin[dof] : 0.f;
          y[dof] = val;
        }
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) partials[(int64_t)slot * 3 + d] = vals[d];
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < P5_NPT; ++k) {
      G1[k] = G2[k];
      S1[k] = S2[k];
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
}

int launch_hex_le_f32x2(const tg_block_plan* plan, int mode, const float* coords, const float* u,
                        const float* v, const uint8_t* fixed, float* y, float* partials,
                        float mu, float lam, cudaStream_t st) {
  const int n_aff = plan->n_affine_blocks;
  if (n_aff <= 0) return TG_OK;
  if (plan->max_local_nodes > P5_MAX_LOCAL) return TG_ERR_UNSUPPORTED;
  const int nl8 = (plan->max_local_nodes + 7) & ~7;
  const size_t smem = (size_t)24 * nl8 * sizeof(float);
  int dev = 0, sms = 0, per_sm = 0, optin = 0;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  TG_TRY(cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"));
  TG_TRY(cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                    "shared memory limit"));
  if (smem > (size_t)optin) return TG_ERR_UNSUPPORTED;
  if (mode == TG_MODE_HVP) {
    auto k = hex_le_f32x2_kernel<TG_MODE_HVP>;
    TG_TRY(cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "hex f32x2: shared memory attribute"));
    TG_TRY(cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, P5_THREADS, smem),
                      "hex f32x2: occupancy"));
    const int grid = std::max(1, std::min(n_aff, sms * std::max(per_sm, 1)));
    k<<<grid, P5_THREADS, smem, st>>>(*plan, n_aff, coords, v, fixed, v, y, partials, mu, lam, nl8);
  } else {
    auto k = hex_le_f32x2_kernel<TG_MODE_RESIDUAL>;
    TG_TRY(cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "hex f32x2: shared memory attribute"));
    TG_TRY(cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, P5_THREADS, smem),
                      "hex f32x2: occupancy"));
    const int grid = std::max(1, std::min(n_aff, sms * std::max(per_sm, 1)));
    k<<<grid, P5_THREADS, smem, st>>>(*plan, n_aff, coords, u, fixed, v, y, partials, mu, lam, nl8);
  }
  return launch_check("hex f32x2 kernel");
}

}  // namespace tg
