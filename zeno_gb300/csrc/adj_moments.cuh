// Stencil moments of node values for the adjoint transfers.
//
// Both adjoint transfers need, for one particle and each channel c of a node
// field g (the grid velocities, or the node adjoints), sums over its 27
// stencil nodes n of g_c times the weight W_n, its position derivative
// dW_n / dx_a, and those times the node offset xx_n,b = (node - x_p)_b:
//   W[c]      = sum W g_c                 X[b][c]  = sum W xx_b g_c
//   D[a][c]   = sum dW_a g_c              DX[a][b][c] = sum dW_a xx_b g_c
// Every factor is a product of one function per axis (w, w xx, dw, dw xx of
// that axis's coordinate), so the sums are taken axis by axis: first over
// the z nodes of each (i, j) row (4 factors), then over y (the 9 factor
// pairs with at most one derivative and one offset), then over x (the 16
// triples) -- about 240 FMAs per channel instead of ~60 per node.
#pragma once

#include <cuda_runtime.h>

#include "mpm_math.cuh"

namespace zsmpm {

struct AdjMoments {
  float W[3];
  float X[3][3];      // [b][c]
  float D[3][3];      // [a][c]
  float DX[3][3][3];  // [a][b][c]
  float Dm[3];        // [a]: sum dW_a of the node field's .x (mass channel)
};

// per-axis factors of one particle: w, w xx, dw / dx, dw / dx xx at i = 0..2
struct AxisFactors {
  float w[3], x[3], d[3], dx[3];
};

__device__ __forceinline__ AxisFactors axis_factors(const Stencil1 &s, float dx, float inv_dx) {
  AxisFactors a;
  float dw[3];
  stencil_dw(s.f, dw);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float xx = ((float)i - s.f) * dx;
    a.w[i] = s.w[i];
    a.x[i] = s.w[i] * xx;
    a.d[i] = dw[i] * inv_dx;
    a.dx[i] = a.d[i] * xx;
  }
  return a;
}

// Moments of the channels .y .z .w (c = 0, 1, 2) of the staged 6^3 window
// `g` (node (i, j, k) of the stencil at ((l0 + i) * 6 + (l1 + j)) * 6 + l2 + k);
// with kMass also Dm from the .x channel.
template <bool kMass>
__device__ __forceinline__ void adj_moments(const float4 *__restrict__ g, int l0, int l1, int l2,
                                            const AxisFactors &A0, const AxisFactors &A1,
                                            const AxisFactors &A2, AdjMoments &M) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    M.W[c] = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      M.X[a][c] = M.D[a][c] = 0.f;
#pragma unroll
      for (int b = 0; b < 3; ++b) M.DX[a][b][c] = 0.f;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) M.Dm[a] = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    // y-level sums of this x layer: pairs (F1, F2) per channel
    float ww[3] = {0.f, 0.f, 0.f}, wx[3] = {0.f, 0.f, 0.f}, xw[3] = {0.f, 0.f, 0.f};
    float wd[3] = {0.f, 0.f, 0.f}, dw[3] = {0.f, 0.f, 0.f}, wdx[3] = {0.f, 0.f, 0.f};
    float dxw[3] = {0.f, 0.f, 0.f}, xd[3] = {0.f, 0.f, 0.f}, dx_[3] = {0.f, 0.f, 0.f};
    float mww = 0.f, mdw = 0.f, mwd = 0.f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float4 *row = g + ((l0 + i) * 6 + (l1 + j)) * 6 + l2;
      // z-level sums of this row: factors w, w xx, dw, dw xx per channel
      float tw[3] = {0.f, 0.f, 0.f}, tx[3] = {0.f, 0.f, 0.f}, td[3] = {0.f, 0.f, 0.f},
            tdx[3] = {0.f, 0.f, 0.f};
      float mw = 0.f, md = 0.f;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float4 v4 = row[k];
        const float v[3] = {v4.y, v4.z, v4.w};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          tw[c] = fmaf(A2.w[k], v[c], tw[c]);
          tx[c] = fmaf(A2.x[k], v[c], tx[c]);
          td[c] = fmaf(A2.d[k], v[c], td[c]);
          tdx[c] = fmaf(A2.dx[k], v[c], tdx[c]);
        }
        if (kMass) {
          mw = fmaf(A2.w[k], v4.x, mw);
          md = fmaf(A2.d[k], v4.x, md);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ww[c] = fmaf(A1.w[j], tw[c], ww[c]);
        wx[c] = fmaf(A1.w[j], tx[c], wx[c]);
        xw[c] = fmaf(A1.x[j], tw[c], xw[c]);
        wd[c] = fmaf(A1.w[j], td[c], wd[c]);
        dw[c] = fmaf(A1.d[j], tw[c], dw[c]);
        wdx[c] = fmaf(A1.w[j], tdx[c], wdx[c]);
        dxw[c] = fmaf(A1.dx[j], tw[c], dxw[c]);
        xd[c] = fmaf(A1.x[j], td[c], xd[c]);
        dx_[c] = fmaf(A1.d[j], tx[c], dx_[c]);
      }
      if (kMass) {
        mww = fmaf(A1.w[j], mw, mww);
        mdw = fmaf(A1.d[j], mw, mdw);
        mwd = fmaf(A1.w[j], md, mwd);
      }
    }
    const float w0 = A0.w[i], x0 = A0.x[i], d0 = A0.d[i], dx0 = A0.dx[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      M.W[c] = fmaf(w0, ww[c], M.W[c]);
      M.X[0][c] = fmaf(x0, ww[c], M.X[0][c]);
      M.X[1][c] = fmaf(w0, xw[c], M.X[1][c]);
      M.X[2][c] = fmaf(w0, wx[c], M.X[2][c]);
      M.D[0][c] = fmaf(d0, ww[c], M.D[0][c]);
      M.D[1][c] = fmaf(w0, dw[c], M.D[1][c]);
      M.D[2][c] = fmaf(w0, wd[c], M.D[2][c]);
      M.DX[0][0][c] = fmaf(dx0, ww[c], M.DX[0][0][c]);
      M.DX[0][1][c] = fmaf(d0, xw[c], M.DX[0][1][c]);
      M.DX[0][2][c] = fmaf(d0, wx[c], M.DX[0][2][c]);
      M.DX[1][0][c] = fmaf(x0, dw[c], M.DX[1][0][c]);
      M.DX[1][1][c] = fmaf(w0, dxw[c], M.DX[1][1][c]);
      M.DX[1][2][c] = fmaf(w0, dx_[c], M.DX[1][2][c]);
      M.DX[2][0][c] = fmaf(x0, wd[c], M.DX[2][0][c]);
      M.DX[2][1][c] = fmaf(w0, xd[c], M.DX[2][1][c]);
      M.DX[2][2][c] = fmaf(w0, wdx[c], M.DX[2][2][c]);
    }
    if (kMass) {
      M.Dm[0] = fmaf(d0, mww, M.Dm[0]);
      M.Dm[1] = fmaf(w0, mdw, M.Dm[1]);
      M.Dm[2] = fmaf(w0, mwd, M.Dm[2]);
    }
  }
}

}  // namespace zsmpm
