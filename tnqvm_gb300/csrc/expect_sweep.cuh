// Pauli-string expectation sweep, shared by the expectation kernel and the
// fused per-program observables of the persistent update kernel.
#pragma once
#include "mps_common.cuh"

namespace gbmps {

// Expectation sweep layout.  FP32 stages the site tensor, the partial
// product X and the environment E in shared memory (160 KiB, one CTA per SM);
// FP64 keeps E in shared memory and reads A and X through L1/L2.
template <typename T>
struct ExpLayout {
  static constexpr bool staged = sizeof(T) == 4;
  static constexpr size_t a_elems = (size_t)kChiLimit * 2 * kChiLimit;  // A or X: (l, s, r)
  static constexpr size_t e_elems = (size_t)kChiLimit * kChiLimit;
  static constexpr size_t smem = sizeof(cx<T>) * (e_elems + (staged ? 2 * a_elems : 0));
  static constexpr size_t scratch = staged ? 16 : sizeof(cx<T>) * a_elems;  // X per CTA (FP64)
};

// Transfer-matrix sweep of one Pauli string over one MPS (ITensor
// compute_expectation_z, ITensorMPSVisitor.cpp:173-250, for any Pauli
// letters): E <- sum_{l,s} A[l,s,:]^H (E P_s A)[l,s,:] site by site.  Step 1
// forms Y = E A (dl x 2dr) in 4(l) x 2(r) x 2(s) register tiles (a tile's two
// columns are strided by the tile count, so a warp reads contiguous shared
// memory without bank conflicts; 512 tiles at bond 64, one per thread) and
// applies the
// site's Pauli as the 2x2 mix X[l,s,r] = sum_s' P[s,s'] Y[l,s',r] in
// registers; step 2 forms E' = A_mat^H X (A_mat = A as a (2dl) x dr matrix) in
// 4 x 2 tiles.  E (ld kChiLimit) and X are work space; As receives the
// staged site when ExpLayout<T>::staged (else A is read from global memory).
// Any block size; thread 0 writes <P> (re, im) to out2.  Called by every
// thread of the block.
template <typename T>
__device__ void expect_sweep(const ExpTask& tk, cx<T>* E, cx<T>* As, cx<T>* X, double* out2) {
  const int tid = threadIdx.x, nt = blockDim.x;
  constexpr int LD = kChiLimit;
  constexpr bool staged = ExpLayout<T>::staged;
  __syncthreads();
  if (tid == 0) E[0] = mk<T>(1, 0);
  const cx<T>* sites = reinterpret_cast<const cx<T>*>(tk.sites);
  for (int i = 0; i < tk.n; ++i) {
    const int dl = tk.bond[i], dr = tk.bond[i + 1];
    const cx<T>* Ag = sites + tk.site_off[i];
    const int code = tk.codes[i];
    const cx<T>* A;
    if (staged) {
      for (int t = tid; t < dl * 2 * dr; t += nt) As[t] = Ag[t];
      A = As;
    } else {
      A = Ag;
    }
    __syncthreads();
    // step 1: X = P (E A), tiles of 4 rows l x 2 columns r x both s (512
    // tiles at bond 64: one per thread)
    {
      constexpr int TC = 2;
      const int nbl = (dl + 3) >> 2, nbr = (dr + TC - 1) / TC;
      for (int tt = tid; tt < nbl * nbr; tt += nt) {
        const int bl = tt / nbr, br = tt - bl * nbr;
        int el[4], ar[TC];
#pragma unroll
        for (int a = 0; a < 4; ++a) el[a] = min(4 * bl + a, dl - 1) * LD;
#pragma unroll
        for (int b = 0; b < TC; ++b) ar[b] = min(br + b * nbr, dr - 1);  // columns strided by nbr: a warp's loads are contiguous
        cx<T> y0[4][TC], y1[4][TC];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < TC; ++b) y0[a][b] = y1[a][b] = mk<T>(0, 0);
        for (int lp = 0; lp < dl; ++lp) {
          cx<T> e[4], a0[TC], a1[TC];
          const cx<T>* row0 = A + (lp * 2) * dr;
          const cx<T>* row1 = row0 + dr;
#pragma unroll
          for (int a = 0; a < 4; ++a) e[a] = E[el[a] + lp];
#pragma unroll
          for (int b = 0; b < TC; ++b) {
            a0[b] = row0[ar[b]];
            a1[b] = row1[ar[b]];
          }
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < TC; ++b) {
              fma_c(y0[a][b], e[a], a0[b]);
              fma_c(y1[a][b], e[a], a1[b]);
            }
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < TC; ++b) {
            const int l = 4 * bl + a, r = br + b * nbr;
            if (l < dl && r < dr) {
              cx<T> x0 = y0[a][b], x1 = y1[a][b];
              if (code == 1) {  // X
                x0 = y1[a][b];
                x1 = y0[a][b];
              } else if (code == 2) {  // Y = [[0,-i],[i,0]]
                x0 = mk<T>(y1[a][b].im, -y1[a][b].re);
                x1 = mk<T>(-y0[a][b].im, y0[a][b].re);
              } else if (code == 3) {  // Z
                x1 = mk<T>(-x1.re, -x1.im);
              }
              X[(l * 2) * dr + r] = x0;
              X[(l * 2 + 1) * dr + r] = x1;
            }
          }
      }
    }
    __syncthreads();
    // step 2: E'[r][r'] = sum_x conj(A[x][r]) X[x][r'], x = (l, s), in 4 (r)
    // x 2 (r') tiles (512 at bond 64)
    {
      constexpr int TC = 2;
      const int nbi = (dr + 3) >> 2, nbj = (dr + TC - 1) / TC;
      const int K = 2 * dl;
      for (int tt = tid; tt < nbi * nbj; tt += nt) {
        const int bi = tt / nbj, bj = tt - bi * nbj;
        int ri[4], rj[TC];
#pragma unroll
        for (int a = 0; a < 4; ++a) ri[a] = min(4 * bi + a, dr - 1);
#pragma unroll
        for (int b = 0; b < TC; ++b) rj[b] = min(bj + b * nbj, dr - 1);
        cx<T> acc[4][TC];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < TC; ++b) acc[a][b] = mk<T>(0, 0);
        for (int x = 0; x < K; ++x) {
          cx<T> av[4], xv[TC];
#pragma unroll
          for (int a = 0; a < 4; ++a) av[a] = A[x * dr + ri[a]];
#pragma unroll
          for (int b = 0; b < TC; ++b) xv[b] = X[x * dr + rj[b]];
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < TC; ++b) fma_cj(acc[a][b], av[a], xv[b]);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < TC; ++b) {
            const int r = 4 * bi + a, rp = bj + b * nbj;
            if (r < dr && rp < dr) E[r * LD + rp] = acc[a][b];
          }
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    out2[0] = (double)E[0].re;
    out2[1] = (double)E[0].im;
  }
  __syncthreads();
}

}  // namespace gbmps
