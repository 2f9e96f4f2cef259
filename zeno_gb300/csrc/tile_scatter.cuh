// Shared-memory tile scatter of one particle block: the P2G phase used by
// P2G (momentum and mass) and by the G2P adjoint (node velocity adjoints).
//
// Each particle of a chunk stages (m, b, A, f) in shared memory: its
// contribution to stencil node o (node - x = (o - f) dx) is
//   mass channel W m,  vector channels W (b + A (o dx)),
// with W the quadratic B-spline weight.  Warp w takes cells w, w + 8, ...,
// w + 56 (three at a time, one per 9-lane slot); the particles of a cell are
// a contiguous range (sorted by cell).  Lane (slot, i, j) owns the three
// nodes (i, j, 0..2) of its slot's cell, so one weight product w_i w_j serves
// three nodes.  Sums go to the warp's private node array, slot by slot, so no
// two lanes update one word at the same time; the 8 warp arrays are added in
// warp order into the block's tile.  No atomics: the tile is reproducible.
#pragma once

#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {

constexpr int kNodes = 216;  // 6^3
constexpr int kP2GThreads = 256;
constexpr int kP2GWarps = kP2GThreads / 32;
constexpr int kP2GChunk = 384;
constexpr int kP2GSpdBytes = 4 * kP2GChunk * 16;
constexpr int kP2GAccBytes = kP2GWarps * 4 * kNodes * 4;
constexpr int kP2GSmem = kP2GSpdBytes + kP2GAccBytes + 65 * 4 + kP2GChunk;
static_assert(kP2GSpdBytes % 16 == 0 && kP2GAccBytes % 16 == 0,
              "spd (float4) and acc must stay 16-byte aligned");

// dynamic shared memory layout (kP2GSmem bytes):
//   spd   4 x kP2GChunk float4: (m,b0,b1,b2) (A00,A01,A02,A10) (A11,A12,A20,A21) (A22,f0,f1,f2)
//   acc   kP2GWarps x 4 x 216 floats: per-warp node sums
//   cst   65 ints: cell ranges of the chunk
//   scell kP2GChunk bytes: cell of each chunk particle
struct TileSmem {
  float4 (*spd)[kP2GChunk];
  float (*acc)[4][kNodes];
  int *cst;
  unsigned char *scell;
};

__device__ __forceinline__ TileSmem tile_smem(unsigned char *raw) {
  TileSmem t;
  t.spd = reinterpret_cast<float4(*)[kP2GChunk]>(raw);
  t.acc = reinterpret_cast<float(*)[4][kNodes]>(raw + kP2GSpdBytes);
  t.cst = reinterpret_cast<int *>(raw + kP2GSpdBytes + kP2GAccBytes);
  t.scell = raw + kP2GSpdBytes + kP2GAccBytes + 65 * sizeof(int);
  return t;
}

__device__ __forceinline__ void tile_zero(const TileSmem &t) {
  for (int i = threadIdx.x; i < kP2GWarps * 4 * kNodes; i += kP2GThreads)
    (&t.acc[0][0][0])[i] = 0.0f;
}

// particle j of the chunk: mass m, b, A (row-major), fractional position f
__device__ __forceinline__ void tile_stage(const TileSmem &t, int j, float m, const float (&b)[3],
                                           const float (&A)[9], const float (&f)[3], int cell) {
  t.spd[0][j] = make_float4(m, b[0], b[1], b[2]);
  t.spd[1][j] = make_float4(A[0], A[1], A[2], A[3]);
  t.spd[2][j] = make_float4(A[4], A[5], A[6], A[7]);
  t.spd[3][j] = make_float4(A[8], f[0], f[1], f[2]);
  t.scell[j] = (unsigned char)cell;
}

// cell ranges of the staged chunk (sorted by cell): first index with cell >= c
__device__ __forceinline__ void tile_cell_ranges(const TileSmem &t, int nc) {
  for (int c = threadIdx.x; c <= 64; c += kP2GThreads) {
    int lo = 0, hi = nc;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (t.scell[mid] < c)
        lo = mid + 1;
      else
        hi = mid;
    }
    t.cst[c] = lo;
  }
}

// the scatter of a staged chunk into the warp-private node sums; call after
// tile_cell_ranges and a __syncthreads
__device__ __forceinline__ void tile_scatter(const TileSmem &t, float dx) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // lane constants: slot, stencil column (i, j), weight polynomials
  // w_0(f) = (1.5-f)^2/2, w_1(f) = 3/4-(f-1)^2, w_2(f) = (f-1/2)^2/2 written as
  // c0 + f (c1 + f c2)
  const int slot = lane / 9, oi = (lane % 9) / 3, oj = lane % 3;
  auto coef = [](int o, float &c0, float &c1, float &c2) {
    c0 = o == 0 ? 1.125f : (o == 1 ? -0.25f : 0.125f);
    c1 = o == 0 ? -1.5f : (o == 1 ? 2.0f : -0.5f);
    c2 = o == 1 ? -1.0f : 0.5f;
  };
  float ci0, ci1, ci2, cj0, cj1, cj2;
  coef(oi, ci0, ci1, ci2);
  coef(oj, cj0, cj1, cj2);
  const float odx = oi * dx, ody = oj * dx;
  float *myacc = &t.acc[warp][0][0];
  const int *cst = t.cst;
  float4 (*spd)[kP2GChunk] = t.spd;
  // phase 2: 8 cells per warp, three per round (slots), 9 lanes per cell
  for (int round = 0; round < 3; ++round) {
    const int ct = 3 * round + slot;  // this lane's cell of the warp, 0..8
    const bool has = lane < 27 && ct < 8;
    const int cell = warp + 8 * ct;
    int q = 0, q1 = 0;
    if (has) {
      q = cst[cell];
      q1 = cst[cell + 1];
    }
    float am0 = 0.f, am1 = 0.f, am2 = 0.f;
    float a00 = 0.f, a01 = 0.f, a02 = 0.f, a10 = 0.f, a11 = 0.f, a12 = 0.f;
    float a20 = 0.f, a21 = 0.f, a22 = 0.f;
    for (; q < q1; ++q) {
      const float4 u0 = spd[0][q], u1 = spd[1][q], u2 = spd[2][q], u3 = spd[3][q];
      const float wx = fmaf(fmaf(ci2, u3.y, ci1), u3.y, ci0);
      const float wy = fmaf(fmaf(cj2, u3.z, cj1), u3.z, cj0);
      const float fz = u3.w;
      const float wz0 = fmaf(fmaf(0.5f, fz, -1.5f), fz, 1.125f);
      const float wz1 = fmaf(fmaf(-1.0f, fz, 2.0f), fz, -0.25f);
      const float wz2 = fmaf(fmaf(0.5f, fz, -0.5f), fz, 0.125f);
      const float wij = wx * wy;
      const float mw = u0.x * wij;
      // b + A (i dx, j dx, k dx) for k = 0, 1, 2
      const float p0 = fmaf(u1.y, ody, fmaf(u1.x, odx, u0.y));
      const float p1 = fmaf(u2.x, ody, fmaf(u1.w, odx, u0.z));
      const float p2 = fmaf(u2.w, ody, fmaf(u2.z, odx, u0.w));
      const float r0 = u1.z * dx, r1 = u2.y * dx, r2 = u3.x * dx;
      const float W0 = wij * wz0, W1 = wij * wz1, W2 = wij * wz2;
      am0 = fmaf(mw, wz0, am0);
      am1 = fmaf(mw, wz1, am1);
      am2 = fmaf(mw, wz2, am2);
      a00 = fmaf(W0, p0, a00);
      a01 = fmaf(W0, p1, a01);
      a02 = fmaf(W0, p2, a02);
      a10 = fmaf(W1, p0 + r0, a10);
      a11 = fmaf(W1, p1 + r1, a11);
      a12 = fmaf(W1, p2 + r2, a12);
      const float r02 = r0 + r0, r12 = r1 + r1, r22 = r2 + r2;
      a20 = fmaf(W2, p0 + r02, a20);
      a21 = fmaf(W2, p1 + r12, a21);
      a22 = fmaf(W2, p2 + r22, a22);
    }
    // slot by slot into the warp's private nodes (cells of one round may
    // share nodes, lanes of one slot own distinct nodes)
    // cell = sort_cell(l0, l1, l2) = (l2 << 4) | (l0 << 2) | l1
    const int nd0 = has ? (((((cell >> 2) & 3) + oi) * 6 + ((cell & 3) + oj)) * 6 + (cell >> 4))
                        : 0;
    for (int sl = 0; sl < 3; ++sl) {
      if (has && slot == sl && q1 > cst[cell]) {
        myacc[0 * kNodes + nd0] += am0;
        myacc[1 * kNodes + nd0] += a00;
        myacc[2 * kNodes + nd0] += a01;
        myacc[3 * kNodes + nd0] += a02;
        myacc[0 * kNodes + nd0 + 1] += am1;
        myacc[1 * kNodes + nd0 + 1] += a10;
        myacc[2 * kNodes + nd0 + 1] += a11;
        myacc[3 * kNodes + nd0 + 1] += a12;
        myacc[0 * kNodes + nd0 + 2] += am2;
        myacc[1 * kNodes + nd0 + 2] += a20;
        myacc[2 * kNodes + nd0 + 2] += a21;
        myacc[3 * kNodes + nd0 + 2] += a22;
      }
      __syncwarp();
    }
  }
}

// the 8 warp arrays, added per node in warp order, into a block's tile
__device__ __forceinline__ void tile_store(const TileSmem &t, float4 *tile) {
  for (int nd = threadIdx.x; nd < kNodes; nd += kP2GThreads) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int w = 0; w < kP2GWarps; ++w) {
      v.x += t.acc[w][0][nd];
      v.y += t.acc[w][1][nd];
      v.z += t.acc[w][2][nd];
      v.w += t.acc[w][3][nd];
    }
    tile[nd] = v;
  }
}

}  // namespace zsmpm
