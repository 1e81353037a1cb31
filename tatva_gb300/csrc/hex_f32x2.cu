// FP32 linear-elastic Hex8 residual / HVP on blocks of exact parallelepipeds:
// persistent CTAs, cp.async pipeline, two elements per thread in packed f32x2
// arithmetic.  Two kernels: hex_le_f32x2_kernel (any box / parallelepiped block,
// colour-ordered shared-memory accumulation, described here) and
// hex_le_lattice_kernel (blocks that are 8 x 8 x 8 grids of boxes: register and
// lane-shuffle accumulation, described above its definition further down).
//
// Same mathematics, plan and summation order as the modal path of assemble.cu (the
// 2x2x2 Gauss sum evaluated exactly in the monomial basis of grad u through an
// 8-point Walsh-Hadamard transform); what changes is the schedule:
//   * each CTA walks its blocks b_0 = blockIdx.x, b_1 = b_0 + gridDim.x, ...; while
//     block b_i is computed, the coordinates and input vector of b_{i+1} are gathered
//     into the other shared-memory buffer (4-byte cp.async per value) and the node
//     ids of b_{i+2} are copied into a two-entry shared ring; the connectivity of
//     b_{i+1} is loaded into registers at the end of b_i's compute -- no global
//     load sits between a block's barrier and its arithmetic;
//   * every thread evaluates two elements at once, one per lane of f32x2 registers;
//   * element results stay in registers until the colour-ordered shared-memory
//     accumulation (one barrier per colour), as in the scalar kernel;
//   * DIAG instantiation: blocks whose elements are axis-aligned boxes (verified on
//     the host in FP32 and FP64) have a diagonal Jacobian, and the monomial terms
//     reduce to per-component products.
#include <map>
#include <mutex>
#include <tuple>

#include "tg_common.cuh"
#include "tg_dispatch.cuh"
#include "tg_f32x2.cuh"
#include "tg_internal.h"

namespace tg {

constexpr int P6_THREADS = 128;
constexpr int P6_NPT = 6;  // staged nodes per thread per block
constexpr int P6_EPT = 4;  // element positions per thread per block
constexpr int P6_MAX_LOCAL = P6_THREADS * P6_NPT;
constexpr int P6_MAX_ELEMS = P6_THREADS * P6_EPT;
constexpr int P6_CRING = 132;  // colour-offset ring entry (<= 128 colours + 1)

__device__ __forceinline__ int hex_t6(int a) {
  return (a == 2) ? 3 : (a == 3) ? 2 : (a == 6) ? 7 : (a == 7) ? 6 : a;
}

__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait0() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// L2 prefetch of the 128-byte lines that hold [p, p + bytes), spread over the CTA's
// threads.  Every line issued contains at least one byte of the range.
__device__ __forceinline__ void prefetch_l2_range(const void* p, size_t bytes, int tid, int nt) {
  if (bytes == 0) return;
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(127);
  const uintptr_t a1 = reinterpret_cast<uintptr_t>(p) + bytes;
  for (uintptr_t a = a0 + (uintptr_t)tid * 128; a < a1; a += (uintptr_t)nt * 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
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

// two-direction monomial (directions P < Q), general Jacobian (see le_two_dir)
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

// two-direction monomial with R = diag(r): the metric is diag(r^2) and R[j][P] = 0
// unless j == P
template <int P, int Q>
__device__ __forceinline__ void le_two_dir2_diag(const f2 (&r)[3], const f2 (&rr)[3],
                                                 const f2 (&gp)[3], const f2 (&gq)[3], f2 mu,
                                                 f2 lam, f2 (&Fp)[3], f2 (&Fq)[3]) {
  const f2 a_pp = gp[P] * r[P], a_pq = gp[Q] * r[Q];
  const f2 a_qp = gq[P] * r[P], a_qq = gq[Q] * r[Q];
  const f2 lt = lam * (a_pp + a_qq);
  const f2 c1 = mu * rr[P], d2 = mu * rr[Q];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Fp[j] = c1 * gp[j];
    Fq[j] = d2 * gq[j];
  }
  Fp[P] = fma2(fma2(mu, a_pp, lt), r[P], Fp[P]);
  Fp[Q] = fma2(mu * a_qp, r[Q], Fp[Q]);
  Fq[P] = fma2(mu * a_pq, r[P], Fq[P]);
  Fq[Q] = fma2(fma2(mu, a_qq, lt), r[Q], Fq[Q]);
}

// M: transformed nodal values (component j, monomial S); out: dE/dM_S for linear
// elasticity on a parallelepiped with R = inv(8 J), detJm = det(8 J).  DIAG: only
// the diagonal of R is read.
template <bool DIAG>
__device__ __forceinline__ void le_modal_pair(const f2 (&R)[3][3], f2 detJm, f2 mu, f2 lam,
                                              const f2 (&M)[3][8], f2 (&dM)[3][8]) {
  const float g2f = float(HEX_GAUSS) * float(HEX_GAUSS);
  const f2 s0 = detJm * f2_bcast(1.0f / 64);
  const f2 s1 = s0 * f2_bcast(g2f);
  const f2 s2 = s1 * f2_bcast(g2f);
  const f2 r[3] = {R[0][0], R[1][1], R[2][2]};
  {  // constant monomial: directions (x, y, z) carry (M1, M2, M4)
    f2 H[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if constexpr (DIAG) {
          H[j][k] = r[k] * M[j][1 << k];
        } else {
          H[j][k] = fma2(R[k][2], M[j][4], fma2(R[k][1], M[j][2], R[k][0] * M[j][1]));
        }
      }
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
      if constexpr (DIAG) {
        dM[j][1] = P[j][0] * r[0];
        dM[j][2] = P[j][1] * r[1];
        dM[j][4] = P[j][2] * r[2];
      } else {
        dM[j][1] = fma2(P[j][2], R[2][0], fma2(P[j][1], R[1][0], P[j][0] * R[0][0]));
        dM[j][2] = fma2(P[j][2], R[2][1], fma2(P[j][1], R[1][1], P[j][0] * R[0][1]));
        dM[j][4] = fma2(P[j][2], R[2][2], fma2(P[j][1], R[1][2], P[j][0] * R[0][2]));
      }
    }
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
  const f2 mu2 = mu * s2, ml2 = (mu + lam) * s2;
  if constexpr (DIAG) {
    const f2 rr[3] = {r[0] * r[0], r[1] * r[1], r[2] * r[2]};
    le_two_dir2_diag<1, 2>(r, rr, g12, g13, mu1, lam1, Fp, Fq);  // monomial x
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][3] = Fp[j]; dM[j][5] = Fq[j]; }
    le_two_dir2_diag<0, 2>(r, rr, g12, g23, mu1, lam1, Fp, Fq);  // monomial y
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][3] = dM[j][3] + Fp[j]; dM[j][6] = Fq[j]; }
    le_two_dir2_diag<0, 1>(r, rr, g13, g23, mu1, lam1, Fp, Fq);  // monomial z
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][5] = dM[j][5] + Fp[j]; dM[j][6] = dM[j][6] + Fq[j]; }
    // yz, xz, xy: (mu tr(Gm) + (mu + lam) r_j^2) g_j
    const f2 a = mu2 * (rr[0] + rr[1] + rr[2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) dM[j][7] = fma2(ml2, rr[j], a) * g123[j];
  } else {
    f2 Gm[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a; b < 3; ++b) {
        Gm[a][b] = fma2(R[2][a], R[2][b], fma2(R[1][a], R[1][b], R[0][a] * R[0][b]));
        Gm[b][a] = Gm[a][b];
      }
    le_two_dir2<1, 2>(R, Gm, g12, g13, mu1, lam1, Fp, Fq);
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][3] = Fp[j]; dM[j][5] = Fq[j]; }
    le_two_dir2<0, 2>(R, Gm, g12, g23, mu1, lam1, Fp, Fq);
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][3] = dM[j][3] + Fp[j]; dM[j][6] = Fq[j]; }
    le_two_dir2<0, 1>(R, Gm, g13, g23, mu1, lam1, Fp, Fq);
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][5] = dM[j][5] + Fp[j]; dM[j][6] = dM[j][6] + Fq[j]; }
    // yz, xz, xy: mu tr(Gm) g + (mu + lam) R R^T g, g = M123
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

__device__ __forceinline__ void unpack_lconn(uint4 v, int (&l)[8]) {
  l[0] = v.x & 0xffff; l[1] = v.x >> 16; l[2] = v.y & 0xffff; l[3] = v.y >> 16;
  l[4] = v.z & 0xffff; l[5] = v.z >> 16; l[6] = v.w & 0xffff; l[7] = v.w >> 16;
}

// Element kinds of the kernel: general parallelepipeds (Jacobian from staged
// coordinates), axis-aligned boxes with the edge lengths from staged coordinates, and
// axis-aligned boxes with the edge lengths from the plan's per-element box_geom32.
constexpr int P6_AFFINE = 0, P6_BOX = 1, P6_BOX_GEOM = 2;

// words of one data buffer per node slot: X (4) and W (4), or W only
__host__ __device__ constexpr int p6_buf_words(int kind) { return kind == P6_BOX_GEOM ? 4 : 8; }
__host__ __device__ constexpr int p6_smem_words_per_slot(int kind) {
  return 2 * p6_buf_words(kind) + 8;
}

// shared-memory layout (32-bit words), nl8 = node slots (multiple of 8), B = buffer
// words per slot (8: X | W, 4: W only):
//   data buffer s (s = 0, 1) at s * B nl8: [X (4 nl8)] | W (4 nl8)
//   node-id ring r (r = 0, 1) at 2B nl8 + r nl8, slot ring r at (2B + 2) nl8 + r nl8
//   Y at (2B + 4) nl8 (4 nl8)
//   colour-offset ring r at (2B + 8) nl8 + r P6_CRING     total (2B + 8) nl8 + 2 P6_CRING
template <int MODE, int KIND>
__global__ void __launch_bounds__(P6_THREADS, KIND == P6_AFFINE ? 3 : 4)
    hex_le_f32x2_kernel(const tg_block_plan p, int b_begin, int b_end,
                        const float* __restrict__ coords, const float* __restrict__ fin,
                        const uint8_t* __restrict__ fixed, const float* __restrict__ vin,
                        float* __restrict__ y, float* __restrict__ partials, float mu_s,
                        float lam_s, int nl8) {
  constexpr bool DIAG = KIND != P6_AFFINE;
  constexpr bool GEO = KIND == P6_BOX_GEOM;
  constexpr int BW = p6_buf_words(KIND);
  extern __shared__ __align__(16) float sm[];
  int* const ring = reinterpret_cast<int*>(sm + 2 * BW * nl8);
  int* const qring = reinterpret_cast<int*>(sm + (2 * BW + 2) * nl8);
  float* const Ybuf = sm + (2 * BW + 4) * nl8;
  int* const cring = reinterpret_cast<int*>(sm + (2 * BW + 8) * nl8);
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  constexpr int NT = P6_THREADS;
  const int nblk = b_end - b_begin;
  const int stride = gridDim.x;

  for (int l = tid; l < nl8; l += NT) {
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      sm[s * BW * nl8 + l * 4 + 3] = 0.f;
      if (!GEO) sm[s * BW * nl8 + 4 * nl8 + l * 4 + 3] = 0.f;
    }
    reinterpret_cast<float4*>(Ybuf)[l] = make_float4(0.f, 0.f, 0.f, 0.f);
  }

  // copy the node ids and shared-memory slots of block b into ring entry r (each
  // thread its own entries)
  auto issue_ids = [&](int b, int r) {
    const int n0 = __ldg(p.blk_node_ptr + b), nl = __ldg(p.blk_node_ptr + b + 1) - n0;
#pragma unroll
    for (int k = 0; k < P6_NPT; ++k) {
      const int l = tid + k * NT;
      if (l < nl) {
        cp_async4(ring + r * nl8 + l, p.lnode_gid + n0 + l);
        cp_async4(qring + r * nl8 + l, p.lnode_smem + n0 + l);
      }
    }
  };
  // colour offsets of block b (at most 129 values) into colour ring entry r
  auto issue_cofs = [&](int b, int r) {
    const int c0 = __ldg(p.blk_color_ptr + b), nc1 = __ldg(p.blk_color_ptr + b + 1) - c0;
    for (int l = tid; l < nc1; l += NT) cp_async4(cring + r * P6_CRING + l, p.color_ofs + c0 + l);
  };
  // gather coordinates and input values of block b (ids in ring slot r) into buffer s.
  // One warp instruction copies 8 consecutive local nodes x 3 components (lanes 0-23):
  // the plan puts such 8 nodes in distinct 16-byte bank quads, so the 24 shared-memory
  // words written land in 24 distinct banks, and the global reads stay contiguous.
  auto issue_data = [&](int b, int r, int s) {
    float* X = sm + s * BW * nl8;
    float* W = X + (BW - 4) * nl8;
    const int nl = __ldg(p.blk_node_ptr + b + 1) - __ldg(p.blk_node_ptr + b);
    const int sub = lane / 3, d = lane - 3 * sub;
    if (lane < 24) {
      for (int l = warp * 8 + sub; l < nl; l += (NT / 32) * 8) {
        const int q = qring[r * nl8 + l];
        const int64_t g = ring[r * nl8 + l];
        if (!GEO) cp_async4(X + q * 4 + d, coords + g * 3 + d);
        cp_async4(W + q * 4 + d, fin + g * 3 + d);
      }
    }
  };
  // the per-element and per-node plan arrays of block b that the compute reads with
  // plain loads (edge terms, local connectivity, partial slots): into L2 one block
  // ahead, so that those loads do not wait on DRAM
  auto prefetch_block = [&](int b) {
    const int e0 = __ldg(p.blk_elem_ptr + b), ne = __ldg(p.blk_elem_ptr + b + 1) - e0;
    const int n0 = __ldg(p.blk_node_ptr + b), nl = __ldg(p.blk_node_ptr + b + 1) - n0;
    if (GEO) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
        prefetch_l2_range(p.box_geom32 + (int64_t)c * p.n_elems + e0, (size_t)ne * 4, tid, NT);
    }
    prefetch_l2_range(reinterpret_cast<const uint4*>(p.lconn) + e0, (size_t)ne * 16, tid, NT);
    prefetch_l2_range(p.lnode_slot + n0, (size_t)nl * 4, tid, NT);
  };
  auto load_lconn4 = [&](int b, uint4 (&LC)[P6_EPT]) {
    const int e0 = __ldg(p.blk_elem_ptr + b), ne = __ldg(p.blk_elem_ptr + b + 1) - e0;
#pragma unroll
    for (int j = 0; j < P6_EPT; ++j) {
      const int k = tid + j * NT;
      LC[j] = (k < ne) ? __ldg(reinterpret_cast<const uint4*>(p.lconn) + e0 + k)
                       : make_uint4(0, 0, 0, 0);
    }
  };

  // prologue: ids of the first block, then its data and the ids of the second
  int bi = blockIdx.x;
  if (bi < nblk) issue_ids(b_begin + bi, 0);
  if (bi < nblk) issue_cofs(b_begin + bi, 0);
  cp_async_commit();
  if (bi < nblk) prefetch_block(b_begin + bi);
  cp_async_wait0();
  __syncthreads();
  if (bi < nblk) issue_data(b_begin + bi, 0, 0);
  if (bi + stride < nblk) issue_ids(b_begin + bi + stride, 1);
  if (bi + stride < nblk) issue_cofs(b_begin + bi + stride, 1);
  cp_async_commit();
  uint4 LC[P6_EPT];
  if (bi < nblk) load_lconn4(b_begin + bi, LC);

  const f2 mu = f2_bcast(mu_s), lam = f2_bcast(lam_s);
  for (int it = 0; bi < nblk; ++it, bi += stride) {
    const int b = b_begin + bi;
    const int s = it & 1;
    cp_async_wait0();
    __syncthreads();  // data of b in buffer s, ids of the next block in ring slot s ^ 1
    const int n0 = __ldg(p.blk_node_ptr + b);
    const int nl = __ldg(p.blk_node_ptr + b + 1) - n0;
    int Gwb[P6_NPT], Swb[P6_NPT], Qwb[P6_NPT];
#pragma unroll
    for (int k = 0; k < P6_NPT; ++k) {
      const int l = tid + k * NT;
      Gwb[k] = (l < nl) ? ring[s * nl8 + l] : 0;
      Qwb[k] = (l < nl) ? qring[s * nl8 + l] : 0;
      Swb[k] = (l < nl) ? __ldg(p.lnode_slot + n0 + l) : 0;
    }
    if (bi + stride < nblk) issue_data(b + stride, s ^ 1, s ^ 1);
    if (bi + 2 * stride < nblk) issue_ids(b + 2 * stride, s);
    cp_async_commit();
    if (bi + stride < nblk) prefetch_block(b + stride);

    const float* X = sm + s * BW * nl8;
    float* W = const_cast<float*>(X) + (BW - 4) * nl8;
    const int e_blk = __ldg(p.blk_elem_ptr + b);
    if (MODE == TG_MODE_HVP && fixed) {
#pragma unroll
      for (int k = 0; k < P6_NPT; ++k) {
        const int l = tid + k * NT;
        if (l < nl) {
#pragma unroll
          for (int d = 0; d < 3; ++d)
            if (fixed[(int64_t)Gwb[k] * 3 + d]) W[Qwb[k] * 4 + d] = 0.f;
        }
      }
      __syncthreads();
    }

    const int ne = __ldg(p.blk_elem_ptr + b + 1) - __ldg(p.blk_elem_ptr + b);
    const int n_col = __ldg(p.blk_color_ptr + b + 1) - 1 - __ldg(p.blk_color_ptr + b);
    const int* const cofs = cring + s * P6_CRING;
#pragma unroll
    for (int ch = 0; ch < P6_EPT / 2; ++ch) {
      const int k0 = ch * 2 * NT;
      if (k0 >= ne) break;  // uniform
      const int kA = k0 + tid, kB = k0 + NT + tid;
      const bool actA = kA < ne, actB = kB < ne;
      float YA[8][3], YB[8][3];
      int qA[8], qB[8];
      unpack_lconn(LC[2 * ch], qA);
      unpack_lconn(actB ? LC[2 * ch + 1] : LC[2 * ch], qB);
      if (actA) {
        f2 R[3][3], detJm;
        if constexpr (GEO) {
          const float* gp = p.box_geom32;
          const int64_t ng = p.n_elems;
          const int64_t iA = e_blk + kA, iB = e_blk + (actB ? kB : kA);
          const float jA0 = __ldg(gp + iA), jB0 = __ldg(gp + iB);
          const float jA1 = __ldg(gp + ng + iA), jB1 = __ldg(gp + ng + iB);
          const float jA2 = __ldg(gp + 2 * ng + iA), jB2 = __ldg(gp + 2 * ng + iB);
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) R[i][j] = f2_zero();
          R[0][0] = f2_make(__frcp_rn(jA0), __frcp_rn(jB0));
          R[1][1] = f2_make(__frcp_rn(jA1), __frcp_rn(jB1));
          R[2][2] = f2_make(__frcp_rn(jA2), __frcp_rn(jB2));
          detJm = f2_make(jA0 * jA1 * jA2, jB0 * jB1 * jB2);
        } else {
          const float4 a0 = reinterpret_cast<const float4*>(X)[qA[0]];
          const float4 b0 = reinterpret_cast<const float4*>(X)[qB[0]];
          const float4 a1 = reinterpret_cast<const float4*>(X)[qA[1]];
          const float4 b1 = reinterpret_cast<const float4*>(X)[qB[1]];
          const float4 a3 = reinterpret_cast<const float4*>(X)[qA[3]];
          const float4 b3 = reinterpret_cast<const float4*>(X)[qB[3]];
          const float4 a4 = reinterpret_cast<const float4*>(X)[qA[4]];
          const float4 b4 = reinterpret_cast<const float4*>(X)[qB[4]];
          if constexpr (DIAG) {
            const float jA0 = 4.f * (a1.x - a0.x), jB0 = 4.f * (b1.x - b0.x);
            const float jA1 = 4.f * (a3.y - a0.y), jB1 = 4.f * (b3.y - b0.y);
            const float jA2 = 4.f * (a4.z - a0.z), jB2 = 4.f * (b4.z - b0.z);
            R[0][0] = f2_make(__frcp_rn(jA0), __frcp_rn(jB0));
            R[1][1] = f2_make(__frcp_rn(jA1), __frcp_rn(jB1));
            R[2][2] = f2_make(__frcp_rn(jA2), __frcp_rn(jB2));
            detJm = f2_make(jA0 * jA1 * jA2, jB0 * jB1 * jB2);
          } else {
            f2 Jm[3][3];
            Jm[0][0] = f2_make(4.f * (a1.x - a0.x), 4.f * (b1.x - b0.x));
            Jm[0][1] = f2_make(4.f * (a1.y - a0.y), 4.f * (b1.y - b0.y));
            Jm[0][2] = f2_make(4.f * (a1.z - a0.z), 4.f * (b1.z - b0.z));
            Jm[1][0] = f2_make(4.f * (a3.x - a0.x), 4.f * (b3.x - b0.x));
            Jm[1][1] = f2_make(4.f * (a3.y - a0.y), 4.f * (b3.y - b0.y));
            Jm[1][2] = f2_make(4.f * (a3.z - a0.z), 4.f * (b3.z - b0.z));
            Jm[2][0] = f2_make(4.f * (a4.x - a0.x), 4.f * (b4.x - b0.x));
            Jm[2][1] = f2_make(4.f * (a4.y - a0.y), 4.f * (b4.y - b0.y));
            Jm[2][2] = f2_make(4.f * (a4.z - a0.z), 4.f * (b4.z - b0.z));
            detJm = inv3_pair(Jm, R);
          }
        }
        f2 M[3][8];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          const float4 wa = reinterpret_cast<const float4*>(W)[qA[a]];
          const float4 wb = reinterpret_cast<const float4*>(W)[qB[a]];
          M[0][hex_t6(a)] = f2_make(wa.x, wb.x);
          M[1][hex_t6(a)] = f2_make(wa.y, wb.y);
          M[2][hex_t6(a)] = f2_make(wa.z, wb.z);
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) had8(M[j]);
        f2 dM[3][8];
        le_modal_pair<DIAG>(R, detJm, mu, lam, M, dM);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          had8t(dM[j]);
#pragma unroll
          for (int a = 0; a < 8; ++a) f2_split(dM[j][hex_t6(a)], YA[a][j], YB[a][j]);
        }
      }
      for (int c = 0; c < n_col; ++c) {
        const int lo = max(cofs[c], k0);
        const int hi = min(cofs[c + 1], k0 + 2 * NT);
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
    if (bi + stride < nblk) load_lconn4(b + stride, LC);

    // write back this block and clear the accumulator
#pragma unroll
    for (int k = 0; k < P6_NPT; ++k) {
      const int l = tid + k * NT;
      if (l >= nl) continue;
      float4* yp = reinterpret_cast<float4*>(Ybuf) + Qwb[k];
      const float4 yv = *yp;
      *yp = make_float4(0.f, 0.f, 0.f, 0.f);
      const int64_t g = Gwb[k];
      const float vals[3] = {yv.x, yv.y, yv.z};
      if (Swb[k] < 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int64_t dof = g * 3 + d;
          float val = vals[d];
          if (fixed && fixed[dof]) val = (MODE == TG_MODE_HVP) ? vin[dof] : 0.f;
          y[dof] = val;
        }
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) partials[(int64_t)Swb[k] * 3 + d] = vals[d];
      }
    }
    __syncthreads();  // every read of colour ring entry s is done
    if (bi + 2 * stride < nblk) issue_cofs(b + 2 * stride, s);
    cp_async_commit();
  }
  asm volatile("griddepcontrol.launch_dependents;");
  cp_async_wait0();
}

// ------------------------------------------------------------------ lattice blocks
// Box blocks whose 512 elements form an 8 x 8 x 8 lattice over 9 x 9 x 9 local nodes
// numbered l = i + 9 j + 81 k (blocks [0, plan.n_lattice_blocks)).  Warp w = jh + 2 kh
// owns the element columns (i, j = 4 jh + jl), lane = i + 8 jl, and sweeps the element
// layers 4 kh .. 4 kh + 3 two at a time, one per f32x2 lane, with the box law of the
// kernel above (same inputs, same bits per element).  A node's sum over one warp's
// elements is formed in registers (the layer carried up the sweep) and by lane shuffles
// (along i, then along j) in a fixed order; the 153 nodes that two or four warps touch
// (row j = 4 and layer k = 4) go through shared memory and are added in warp order
// after the sweep.  No element colouring and no element connectivity: a block reads
// its 729 node ids and partial slots, the input vector at those nodes and the 27
// coordinates of its grid lines.  Barriers per block: data landed, mid-sweep (the next
// block's ids landed: start its input gather), merge parts in place, ring free (plus
// one after staging the Dirichlet bits when there is a mask).
constexpr int LT_THREADS = 128;
constexpr int LT_NODES = 729, LT_RING = 732, LT_MERGE = 153, LT_PARTS = 81;
// W [2][729] float4 | merge parts [4 warps][81] float4 | ids [2][732] | slots [2][732] |
// grid lines [2][32] | Dirichlet bits of the current block's nodes [732] bytes
constexpr size_t LT_SMEM =
    (2 * LT_NODES + 4 * LT_PARTS) * 16 + 4 * LT_RING * 4 + 2 * 32 * 4 + LT_RING;

// Index of node (ni, nj, L) among the 81 merge parts of warp (jh, kh): row j = 4 at the
// warp's layers 4 kh .. 4 kh + 4 first (45), then layer 4 at the warp's other rows (36).
__host__ __device__ __forceinline__ int lt_part(int jh, int kh, int ni, int nj, int L) {
  return (nj == 4) ? ni + 9 * (L - 4 * kh) : 45 + ni + 9 * (jh == 0 ? nj : nj - 5);
}

__device__ __forceinline__ void cp_async_wait1() {
  asm volatile("cp.async.wait_group 1;" ::: "memory");
}

template <int MODE>
__global__ void __launch_bounds__(LT_THREADS, 4)
    hex_le_lattice_kernel(const tg_block_plan p, const float* __restrict__ coords,
                          const float* __restrict__ fin, const uint8_t* __restrict__ fixed,
                          const float* __restrict__ vin, float* __restrict__ y,
                          float* __restrict__ partials, float mu_s, float lam_s) {
  extern __shared__ __align__(16) float sm[];
  float4* const W = reinterpret_cast<float4*>(sm);
  float4* const Pm = W + 2 * LT_NODES;
  int* const ids = reinterpret_cast<int*>(Pm + 4 * LT_PARTS);
  int* const slots = ids + 2 * LT_RING;
  float* const geo = reinterpret_cast<float*>(slots + 2 * LT_RING);
  uint8_t* const fbits = reinterpret_cast<uint8_t*>(geo + 2 * 32);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = p.n_lattice_blocks, stride = gridDim.x;
  const int64_t nbase = __ldg(p.blk_node_ptr);

  // node ids and partial slots of block b into ring entry r
  auto issue_meta = [&](int b, int r) {
    const int64_t n0 = nbase + (int64_t)LT_NODES * b;
#pragma unroll 3
    for (int l = tid; l < LT_NODES; l += LT_THREADS) {
      cp_async4(ids + r * LT_RING + l, p.lnode_gid + n0 + l);
      cp_async4(slots + r * LT_RING + l, p.lnode_slot + n0 + l);
    }
  };
  // input values of the block whose ids are in ring entry r into buffer r (8 nodes x 3
  // components per warp instruction), and its grid lines: x of nodes (i, 0, 0), y of
  // (0, j, 0), z of (0, 0, k)
  auto issue_data = [&](int r) {
    float* Wr = reinterpret_cast<float*>(W + r * LT_NODES);
    const int* id = ids + r * LT_RING;
    const int sub = lane / 3, d = lane - 3 * sub;
    if (lane < 24) {
#pragma unroll 4
      for (int l = warp * 8 + sub; l < LT_NODES; l += 32)
        cp_async4(Wr + l * 4 + d, fin + (int64_t)id[l] * 3 + d);
    }
    if (tid < 27) {
      const int a = tid / 9, q = tid - 9 * a;
      const int l = a == 0 ? q : (a == 1 ? 9 * q : 81 * q);
      cp_async4(geo + r * 32 + tid, coords + (int64_t)id[l] * 3 + a);
    }
  };

  int bi = blockIdx.x;
  if (bi < nblk) issue_meta(bi, 0);
  cp_async_commit();
  cp_async_wait0();
  __syncthreads();
  if (bi < nblk) issue_data(0);
  cp_async_commit();
  if (bi + stride < nblk) issue_meta(bi + stride, 1);
  cp_async_commit();

  const int jh = warp & 1, kh = warp >> 1;
  const int i = lane & 7, jl = lane >> 3, j = 4 * jh + jl, k0 = 4 * kh;
  const f2 mu = f2_bcast(mu_s), lam = f2_bcast(lam_s);
  for (int it = 0; bi < nblk; ++it, bi += stride) {
    const int s = it & 1;
    cp_async_wait1();  // this block's data (the newest group, the next block's ids, may pend)
    __syncthreads();
    const float4* Ws = W + s * LT_NODES;
    const int* id = ids + s * LT_RING;
    const int* sl = slots + s * LT_RING;
    if (fixed) {
      // the block's Dirichlet bits into shared memory (read once per node here, not at
      // every emission); HVP: fixed inputs read as 0
      float* Wf = reinterpret_cast<float*>(W + s * LT_NODES);
      constexpr int NQ = (LT_NODES + LT_THREADS - 1) / LT_THREADS;
      uint8_t f[NQ][3];  // all of this thread's mask bytes in flight at once
#pragma unroll
      for (int qn = 0; qn < NQ; ++qn) {
        const int l = tid + qn * LT_THREADS;
        const int64_t g = l < LT_NODES ? id[l] : 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) f[qn][d] = l < LT_NODES ? fixed[g * 3 + d] : 0;
      }
#pragma unroll
      for (int qn = 0; qn < NQ; ++qn) {
        const int l = tid + qn * LT_THREADS;
        if (l >= LT_NODES) continue;
        const int m = (f[qn][0] != 0) | (f[qn][1] != 0) << 1 | (f[qn][2] != 0) << 2;
        fbits[l] = (uint8_t)m;
        if (MODE == TG_MODE_HVP && m) {
#pragma unroll
          for (int d = 0; d < 3; ++d)
            if (m >> d & 1) Wf[l * 4 + d] = 0.f;
        }
      }
      __syncthreads();
    }

    // final block-local sum of node l: the node's own value if no other block touches it,
    // else its partial slot
    auto emit = [&](int l, float v0, float v1, float v2) {
      const int64_t g = id[l];
      const int q = sl[l];
      const float v[3] = {v0, v1, v2};
      if (q < 0) {
        const int m = fixed ? fbits[l] : 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int64_t dof = g * 3 + d;
          float val = v[d];
          if (m >> d & 1) val = (MODE == TG_MODE_HVP) ? vin[dof] : 0.f;
          y[dof] = val;
        }
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) partials[(int64_t)q * 3 + d] = v[d];
      }
    };
    // this warp's sum at node (ni, nj, L): emitted, or parked for the merge when another
    // warp also touches the node
    auto put = [&](int ni, int nj, int L, const float (&v)[3]) {
      if (nj == 4 || L == 4) {
        Pm[warp * LT_PARTS + lt_part(jh, kh, ni, nj, L)] = make_float4(v[0], v[1], v[2], 0.f);
      } else {
        emit(ni + 9 * nj + 81 * L, v[0], v[1], v[2]);
      }
    };
    // Q[t][c]: this lane's column values at the corners t = di + 2 dj of layer L
    auto reduce_put = [&](float (&Q)[4][3], int L) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float a = __shfl_up_sync(0xffffffffu, Q[1][c], 1);
        const float b = __shfl_up_sync(0xffffffffu, Q[3][c], 1);
        if (i > 0) {
          Q[0][c] += a;
          Q[2][c] += b;
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float a = __shfl_up_sync(0xffffffffu, Q[2][c], 8);
        const float b = __shfl_up_sync(0xffffffffu, Q[3][c], 8);
        if (jl > 0) {
          Q[0][c] += a;
          Q[1][c] += b;
        }
      }
      put(i, j, L, Q[0]);
      // the warp's 13 halo nodes in one pass: (8, j) from lanes i = 7, (i, j + 1) from
      // lanes jl = 3, and lane 31's second and third halo nodes handed to lanes 0, 1
      float X2[3], X3[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        X2[c] = __shfl_sync(0xffffffffu, Q[2][c], 31);
        X3[c] = __shfl_sync(0xffffffffu, Q[3][c], 31);
      }
      const int jt = 4 * jh + 4;
      int hi_ = -1, hj = 0;
      float hv[3];
      if (i == 7) {
        hi_ = 8; hj = j;
#pragma unroll
        for (int c = 0; c < 3; ++c) hv[c] = Q[1][c];
      } else if (jl == 3) {
        hi_ = i; hj = jt;
#pragma unroll
        for (int c = 0; c < 3; ++c) hv[c] = Q[2][c];
      } else if (lane < 2) {
        hi_ = 7 + lane; hj = jt;
#pragma unroll
        for (int c = 0; c < 3; ++c) hv[c] = lane == 0 ? X2[c] : X3[c];
      }
      if (hi_ >= 0) put(hi_, hj, L, hv);
    };
    auto load_layer = [&](int L, float (&o)[4][3]) {
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const float4 w = Ws[(i + (t & 1)) + 9 * (j + (t >> 1)) + 81 * L];
        o[t][0] = w.x;
        o[t][1] = w.y;
        o[t][2] = w.z;
      }
    };

    const float* G = geo + s * 32;
    const float hx = 4.f * (G[i + 1] - G[i]);
    const float hy = 4.f * (G[9 + j + 1] - G[9 + j]);
    const float rx = __frcp_rn(hx), ry = __frcp_rn(hy);
    const float hxy = hx * hy;
    float cur[4][3], C[4][3];
    load_layer(k0, cur);
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
      for (int c = 0; c < 3; ++c) C[t][c] = 0.f;
    // both pair steps in one scheduling region (measured 3 % faster than a loop)
#pragma unroll
    for (int ps = 0; ps < 2; ++ps) {
      const int k = k0 + 2 * ps;
      float mid[4][3], top[4][3];
      load_layer(k + 1, mid);
      load_layer(k + 2, top);
      f2 M[3][8];
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          M[c][t] = f2_make(cur[t][c], mid[t][c]);
          M[c][t + 4] = f2_make(mid[t][c], top[t][c]);
        }
#pragma unroll
      for (int c = 0; c < 3; ++c) had8(M[c]);
      const float hzA = 4.f * (G[18 + k + 1] - G[18 + k]);
      const float hzB = 4.f * (G[18 + k + 2] - G[18 + k + 1]);
      f2 R[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) R[a][b] = f2_zero();
      R[0][0] = f2_bcast(rx);
      R[1][1] = f2_bcast(ry);
      R[2][2] = f2_make(__frcp_rn(hzA), __frcp_rn(hzB));
      const f2 detJm = f2_make(hxy * hzA, hxy * hzB);
      f2 dM[3][8];
      le_modal_pair<true>(R, detJm, mu, lam, M, dM);
      float YA[8][3], YB[8][3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        had8t(dM[c]);
#pragma unroll
        for (int t = 0; t < 8; ++t) f2_split(dM[c][t], YA[t][c], YB[t][c]);
      }
      float Q[4][3];
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int c = 0; c < 3; ++c) Q[t][c] = C[t][c] + YA[t][c];
      reduce_put(Q, k);
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int c = 0; c < 3; ++c) Q[t][c] = YA[t + 4][c] + YB[t][c];
      reduce_put(Q, k + 1);
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          C[t][c] = YB[t + 4][c];
          cur[t][c] = top[t][c];
        }
      if (ps == 0) {  // the next block's ids have landed: start its data
        cp_async_wait0();
        __syncthreads();
        if (bi + stride < nblk) issue_data(s ^ 1);
        cp_async_commit();
      }
    }
    reduce_put(C, k0 + 4);
    __syncthreads();  // every warp's merge parts are in place

    for (int m = tid; m < LT_MERGE; m += LT_THREADS) {
      int ni, nj, L;
      float4 a;
      if (m < 81) {
        ni = m % 9;
        L = m / 9;
        nj = 4;
      } else {
        const int r = m - 81, jj = r / 9;
        ni = r - 9 * jj;
        nj = jj < 4 ? jj : jj + 1;
        L = 4;
      }
      if (nj == 4 && L == 4) {  // all four warps, in warp order
        const float4 a0 = Pm[lt_part(0, 0, ni, 4, 4)];
        const float4 a1 = Pm[LT_PARTS + lt_part(1, 0, ni, 4, 4)];
        const float4 a2 = Pm[2 * LT_PARTS + lt_part(0, 1, ni, 4, 4)];
        const float4 a3 = Pm[3 * LT_PARTS + lt_part(1, 1, ni, 4, 4)];
        a = make_float4(((a0.x + a1.x) + a2.x) + a3.x, ((a0.y + a1.y) + a2.y) + a3.y,
                        ((a0.z + a1.z) + a2.z) + a3.z, 0.f);
      } else {
        // row j = 4: warps jh = 0, 1 of the layer's half; layer 4: warps kh = 0, 1 of
        // the row's half
        const int kh0 = (nj == 4) ? (L < 4 ? 0 : 1) : 0, kh1 = (nj == 4) ? kh0 : 1;
        const int jh0 = (nj == 4) ? 0 : (nj < 4 ? 0 : 1), jh1 = (nj == 4) ? 1 : jh0;
        const float4 a0 = Pm[(jh0 + 2 * kh0) * LT_PARTS + lt_part(jh0, kh0, ni, nj, L)];
        const float4 a1 = Pm[(jh1 + 2 * kh1) * LT_PARTS + lt_part(jh1, kh1, ni, nj, L)];
        a = make_float4(a0.x + a1.x, a0.y + a1.y, a0.z + a1.z, 0.f);
      }
      emit(ni + 9 * nj + 81 * L, a.x, a.y, a.z);
    }
    __syncthreads();  // ring entry s and the merge parts are free
    if (bi + 2 * stride < nblk) issue_meta(bi + 2 * stride, s);
    cp_async_commit();
  }
  asm volatile("griddepcontrol.launch_dependents;");
  cp_async_wait0();
}

// Per (kernel, device, shared-memory size): SM count and resident CTAs per SM, set up
// once (the attribute call and the occupancy query cost more than a launch).
// The dynamic shared-memory attribute of a kernel only ever grows (to the largest size
// requested so far): lowering it would break launches of larger plans that reuse a
// cached shape, and CUDA graphs captured with them.
static int launch_shape(const void* k, size_t smem, int& sms, int& per_sm) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t>, std::pair<int, int>> cache;
  static std::map<std::pair<const void*, int>, size_t> attr;
  int dev = 0;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  std::lock_guard<std::mutex> g(mu);
  const auto key = std::make_tuple(k, dev, smem);
  auto it = cache.find(key);
  if (it == cache.end()) {
    int optin = 0, n_sm = 0, occ = 0;
    TG_TRY(cuda_check(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), "SM count"));
    TG_TRY(cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                      "shared memory limit"));
    if (smem <= (size_t)optin) {
      size_t& cur = attr[std::make_pair(k, dev)];
      if (smem > cur) {
        TG_TRY(cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                          "hex f32x2: shared memory attribute"));
        cur = smem;
      }
      TG_TRY(cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, P6_THREADS, smem),
                        "hex f32x2: occupancy"));
    }
    it = cache.emplace(key, std::make_pair(n_sm, occ)).first;
  }
  sms = it->second.first;
  per_sm = it->second.second;
  return TG_OK;
}

template <int MODE, int KIND>
static int launch6(const tg_block_plan* plan, int b0, int b1, const float* coords,
                   const float* fin, const uint8_t* fixed, const float* vin, float* y,
                   float* partials, float mu, float lam, int nl8, cudaStream_t st) {
  if (b1 <= b0) return TG_OK;
  auto k = hex_le_f32x2_kernel<MODE, KIND>;
  const size_t smem =
      ((size_t)p6_smem_words_per_slot(KIND) * nl8 + 2 * P6_CRING) * sizeof(float);
  int sms = 0, per_sm = 0;
  TG_TRY(launch_shape((const void*)k, smem, sms, per_sm));
  if (per_sm <= 0) return TG_ERR_UNSUPPORTED;
  const int grid = std::max(1, std::min(b1 - b0, sms * per_sm));
  k<<<grid, P6_THREADS, smem, st>>>(*plan, b0, b1, coords, fin, fixed, vin, y, partials, mu, lam,
                                    nl8);
  return launch_check("hex f32x2 kernel");
}

template <int MODE>
static int launch_lattice(const tg_block_plan* plan, const float* coords, const float* fin,
                          const uint8_t* fixed, const float* vin, float* y, float* partials,
                          float mu, float lam, cudaStream_t st) {
  const int n = plan->n_lattice_blocks;
  if (n <= 0) return TG_OK;
  auto k = hex_le_lattice_kernel<MODE>;
  int sms = 0, per_sm = 0;
  TG_TRY(launch_shape((const void*)k, LT_SMEM, sms, per_sm));
  if (per_sm <= 0) return TG_ERR_UNSUPPORTED;
  const int grid = std::max(1, std::min(n, sms * per_sm));
  k<<<grid, LT_THREADS, LT_SMEM, st>>>(*plan, coords, fin, fixed, vin, y, partials, mu, lam);
  return launch_check("hex lattice kernel");
}

template <int MODE>
static int launch_modes(const tg_block_plan* plan, const float* coords, const float* fin,
                        const uint8_t* fixed, const float* vin, float* y, float* partials,
                        float mu, float lam, int nl8, cudaStream_t st) {
  const int n_aff = plan->n_affine_blocks, n_diag = plan->n_diag_blocks;
  const int n_lat = plan->n_lattice_blocks;
  TG_TRY(launch_lattice<MODE>(plan, coords, fin, fixed, vin, y, partials, mu, lam, st));
  if (plan->box_geom32) {
    TG_TRY((launch6<MODE, P6_BOX_GEOM>(plan, n_lat, n_diag, coords, fin, fixed, vin, y, partials,
                                       mu, lam, nl8, st)));
  } else {
    TG_TRY((launch6<MODE, P6_BOX>(plan, n_lat, n_diag, coords, fin, fixed, vin, y, partials, mu,
                                  lam, nl8, st)));
  }
  return launch6<MODE, P6_AFFINE>(plan, n_diag, n_aff, coords, fin, fixed, vin, y, partials, mu,
                                  lam, nl8, st);
}

int launch_hex_le_f32x2(const tg_block_plan* plan, int mode, const float* coords, const float* u,
                        const float* v, const uint8_t* fixed, float* y, float* partials,
                        float mu, float lam, cudaStream_t st) {
  const int n_aff = plan->n_affine_blocks, n_diag = plan->n_diag_blocks;
  if (n_aff <= 0) return TG_OK;
  if (plan->max_local_nodes > P6_MAX_LOCAL || plan->max_block_elems > P6_MAX_ELEMS)
    return TG_ERR_UNSUPPORTED;
  if (n_diag < 0 || n_diag > n_aff) return set_error(TG_ERR_VALUE, "plan.n_diag_blocks out of range");
  if (plan->n_lattice_blocks < 0 || plan->n_lattice_blocks > n_diag)
    return set_error(TG_ERR_VALUE, "plan.n_lattice_blocks out of range");
  const int nl8 = (plan->max_local_nodes + 7) & ~7;
  // the general kernel needs the most shared memory: check it before launching anything
  int sms = 0, per_sm = 0;
  const size_t smem_aff =
      ((size_t)p6_smem_words_per_slot(P6_AFFINE) * nl8 + 2 * P6_CRING) * sizeof(float);
  TG_TRY(launch_shape((const void*)hex_le_f32x2_kernel<TG_MODE_HVP, P6_AFFINE>, smem_aff, sms,
                      per_sm));
  if (per_sm <= 0) return TG_ERR_UNSUPPORTED;
  if (mode == TG_MODE_HVP)
    return launch_modes<TG_MODE_HVP>(plan, coords, v, fixed, v, y, partials, mu, lam, nl8, st);
  return launch_modes<TG_MODE_RESIDUAL>(plan, coords, u, fixed, v, y, partials, mu, lam, nl8, st);
}

// Per-element box edge terms 4 (x1 - x0), 4 (y3 - y0), 4 (z4 - z0) in FP32, exactly as
// the box kernel computes them from staged coordinates, for element positions
// [0, blk_elem_ptr[n_diag_blocks]) of the plan; layout [3][n_elems].
__global__ void box_geometry_kernel(const tg_block_plan p, const float* __restrict__ coords,
                                    const int32_t* __restrict__ conn, float* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.n_elems) return;
  const int end = p.blk_elem_ptr[p.n_diag_blocks];
  if (k >= end) return;
  const int64_t e = p.elem_id[k];
  const int32_t* c = conn + e * 8;
  const float* x0 = coords + (int64_t)c[0] * 3;
  const float* x1 = coords + (int64_t)c[1] * 3;
  const float* x3 = coords + (int64_t)c[3] * 3;
  const float* x4 = coords + (int64_t)c[4] * 3;
  out[k] = 4.f * (x1[0] - x0[0]);
  out[p.n_elems + k] = 4.f * (x3[1] - x0[1]);
  out[2 * (int64_t)p.n_elems + k] = 4.f * (x4[2] - x0[2]);
}

}  // namespace tg

using namespace tg;

extern "C" int tg_plan_box_geometry(const tg_block_plan* plan, const float* coords,
                                    const int32_t* conn, float* out, void* stream) {
  if (!plan) return set_error(TG_ERR_VALUE, "plan must not be NULL");
  if (plan->nodes_per_elem_padded != 8)
    return set_error(TG_ERR_VALUE, "box geometry needs a Hex8 plan");
  if (plan->n_diag_blocks < 0 || plan->n_diag_blocks > plan->n_blocks)
    return set_error(TG_ERR_VALUE, "plan.n_diag_blocks out of range");
  if (plan->n_elems == 0 || plan->n_diag_blocks == 0) return TG_OK;
  TG_TRY(check_ptr(coords, "coords"));
  TG_TRY(check_ptr(conn, "conn"));
  TG_TRY(check_ptr(out, "out"));
  box_geometry_kernel<<<grid_for(plan->n_elems, 256), 256, 0, as_stream(stream)>>>(*plan, coords,
                                                                                  conn, out);
  return launch_check("tg_plan_box_geometry");
}
