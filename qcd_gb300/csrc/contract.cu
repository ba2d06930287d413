// contract.cu -- proton two-point function on GPU-resident propagators, the
// contraction of twop.c (twop.c:219-226 boundary phases, :264-282 C g5 x
// bar C g5 entries, :324-399 block and Fourier sum).
//
// Propagators are 12 FP64 fields per flavour: column nu * 3 + c2 (source spin
// nu, source colour c2) holds the spinor (sink spin mu, sink colour c1), i.e.
// qcd_lib's D[v][mu][nu][c1][c2]. For every requested time-slice t (relative
// to the source) and spatial site x of slice (t + x_src,t) mod L_t:
//
//   block(x) = - f(t)^3 sum_{al,be} P13[al][be] sum_{mu nu ku lu} Cg5[mu][nu] barCg5[ku][lu]
//              sum_{eps, eps'} sgn sgn' [ u(mu,ku;c1,c1') d(nu,lu;c2,c2') u(be,al;c3,c3')
//                                        + u(mu,al;c1,c1') d(nu,lu;c2,c2') u(be,ku;c3,c3') ]
//
// with f(t) = exp(i pi t / L_t) (the antiperiodic-to-periodic phase twop.c
// multiplies into both propagators), and corr(t, p) = 1/2 sum_x block(x)
// exp(-2 pi i p.(x - x_src) / L). One thread per site computes block(x) in
// FP64; one CTA per (t, momentum) sums the sites in a fixed order.
#include <math.h>
#include <string.h>

#include <vector>

#include "dslash_args.h"

namespace qg {

using namespace qgd;

namespace {

// the tables of the contraction (kept identical to qcd_lib's qcd_EPS,
// qcd_SGN_EPS, qcd_CGAMMA[5], qcd_BAR_CGAMMA[5] and PROJECTOR[13])
__constant__ int c_eps[6][3] = {{0, 1, 2}, {2, 0, 1}, {1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {1, 0, 2}};
__constant__ int c_sgn[6] = {+1, +1, +1, -1, -1, -1};
// nonzero (mu, nu) of C g5 with its value; the same for bar C g5 (ku, lu)
__constant__ int c_cg5[4][3] = {{0, 1, 1}, {1, 0, -1}, {2, 3, 1}, {3, 2, -1}};
__constant__ int c_bcg5[4][3] = {{0, 1, -1}, {1, 0, 1}, {2, 3, -1}, {3, 2, 1}};
// nonzero (al, be) of PROJECTOR[13] with its value (re, im)
__constant__ int c_p13_idx[8][2] = {{0, 0}, {0, 2}, {1, 1}, {1, 3}, {2, 0}, {2, 2}, {3, 1}, {3, 3}};
__constant__ double c_p13_val[8][2] = {{0, .5}, {-.5, 0}, {0, .5}, {-.5, 0}, {-.5, 0}, {0, -.5}, {-.5, 0}, {0, -.5}};

struct Props {
  const double2 *u[12], *d[12];  // column nu * 3 + c2
  int64_t stride;
};

// u(mu, nu; c1, c2) at site v
__device__ __forceinline__ C<double> pr(const double2 *const *col, int64_t stride, int v, int mu, int nu, int c1,
                                         int c2)
{
  const double2 w = __ldg(col[nu * 3 + c2] + (int64_t)(mu * 3 + c1) * stride + v);
  return C<double>{w.x, w.y};
}

__global__ void __launch_bounds__(128) k_twop_block(Props p, Geom geo, int t0, int nt, int xsrc_t, double2 *block)
{
  const int V3 = geo.L[1] * geo.L[2] * geo.L[3];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V3 * nt) return;
  const int s = i % V3, t = t0 + i / V3;
  const int lt = (t + xsrc_t) % geo.L[0];
  const int v = lt + geo.L[0] * s;
  C<double> acc{0.0, 0.0};
  for (int ip = 0; ip < 8; ip++) {
    const int al = c_p13_idx[ip][0], be = c_p13_idx[ip][1];
    const C<double> P{c_p13_val[ip][0], c_p13_val[ip][1]};
    C<double> sp{0.0, 0.0};
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) {
        const int mu = c_cg5[a][0], nu = c_cg5[a][1], ku = c_bcg5[b][0], lu = c_bcg5[b][1];
        const double cval = (double)(c_cg5[a][2] * c_bcg5[b][2]);
        C<double> se{0.0, 0.0};
        for (int e1 = 0; e1 < 6; e1++)
          for (int e2 = 0; e2 < 6; e2++) {
            const int c1 = c_eps[e1][0], c2 = c_eps[e1][1], c3 = c_eps[e1][2];
            const int d1 = c_eps[e2][0], d2 = c_eps[e2][1], d3 = c_eps[e2][2];
            const C<double> dd = pr(p.d, p.stride, v, nu, lu, c2, d2);
            const C<double> t1 = pr(p.u, p.stride, v, mu, ku, c1, d1) * dd * pr(p.u, p.stride, v, be, al, c3, d3);
            const C<double> t2 = pr(p.u, p.stride, v, mu, al, c1, d1) * dd * pr(p.u, p.stride, v, be, ku, c3, d3);
            const double sg = (double)(c_sgn[e1] * c_sgn[e2]);
            se = C<double>{se.re + sg * (t1.re + t2.re), se.im + sg * (t1.im + t2.im)};
          }
        sp = C<double>{sp.re + cval * se.re, sp.im + cval * se.im};
      }
    acc = acc - P * sp;
  }
  // boundary phase of the three propagator factors: exp(3 i pi t / L_t)
  double sn, cs;
  sincospi(3.0 * (double)t / (double)geo.L[0], &sn, &cs);
  acc = acc * C<double>{cs, sn};
  block[(int64_t)(t - t0) * V3 + s] = make_double2(acc.re, acc.im);
}

// corr[t][j] = 1/2 sum_x block(x) exp(-2 pi i p_j.(x - x_src) / L); one CTA
// per (t, j), sites summed in a fixed order
__global__ void __launch_bounds__(256) k_twop_ft(const double2 *block, Geom geo, const int *mom, int nmom, int sx,
                                                 int sy, int sz, double2 *corr)
{
  const int t = blockIdx.x / nmom, j = blockIdx.x % nmom;
  const int Lx = geo.L[1], Ly = geo.L[2], Lz = geo.L[3], V3 = Lx * Ly * Lz;
  const double px = (double)mom[3 * j] / Lx, py = (double)mom[3 * j + 1] / Ly, pz = (double)mom[3 * j + 2] / Lz;
  double re = 0.0, im = 0.0;
  for (int s = threadIdx.x; s < V3; s += blockDim.x) {
    const int x = s % Lx, y = (s / Lx) % Ly, z = s / (Lx * Ly);
    double sn, cs;
    sincospi(2.0 * (px * (x - sx) + py * (y - sy) + pz * (z - sz)), &sn, &cs);
    const double2 b = block[(int64_t)t * V3 + s];
    re += b.x * cs + b.y * sn;  // b * (cos - i sin)
    im += b.y * cs - b.x * sn;
  }
  __shared__ double sr[256], si[256];
  sr[threadIdx.x] = re;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      si[threadIdx.x] += si[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) corr[blockIdx.x] = make_double2(0.5 * sr[0], 0.5 * si[0]);
}

}  // namespace

bool twop_proton(const qcdgpu_field *up, const qcdgpu_field *dn, const int xsrc[4], int t0, int t1, const int *mom,
                 int nmom, double *corr)
{
  if (!up || !dn || !xsrc || !mom || !corr || nmom < 1 || t0 < 0 || t1 < t0) {
    set_error("two-point function: 12 + 12 propagator columns, 0 <= t0 <= t1, at least one momentum");
    return false;
  }
  const qcdgpu_field f0 = up[0];
  if (!f0 || t1 >= f0->L[0]) {
    set_error("two-point function: time-slices beyond the lattice");
    return false;
  }
  Props p;
  for (int k = 0; k < 12; k++) {
    if (!up[k] || !dn[k] || up[k]->prec != QCDGPU_F64 || dn[k]->prec != QCDGPU_F64 || !same_shape(up[k], f0) ||
        !same_shape(dn[k], f0)) {
      set_error("two-point function: FP64 propagator columns of one lattice");
      return false;
    }
    p.u[k] = (const double2 *)up[k]->data;
    p.d[k] = (const double2 *)dn[k]->data;
  }
  for (int i = 0; i < 4; i++)
    if (xsrc[i] < 0 || xsrc[i] >= f0->L[i]) {
      set_error("two-point function: source outside the lattice");
      return false;
    }
  p.stride = f0->stride;
  Geom geo;
  for (int i = 0; i < 4; i++) geo.L[i] = f0->L[i];
  geo.st[0] = 1;
  geo.st[1] = f0->L[0];
  geo.st[2] = f0->L[0] * f0->L[1];
  geo.st[3] = f0->L[0] * f0->L[1] * f0->L[2];
  const int nt = t1 - t0 + 1, V3 = f0->L[1] * f0->L[2] * f0->L[3];
  double2 *block = nullptr, *dcorr = nullptr;
  int *dmom = nullptr;
  cudaStream_t st = stream();
  bool ok = QG_CUDA(cudaMalloc(&block, sizeof(double2) * (size_t)nt * V3)) &&
            QG_CUDA(cudaMalloc(&dcorr, sizeof(double2) * (size_t)nt * nmom)) &&
            QG_CUDA(cudaMalloc(&dmom, sizeof(int) * 3 * (size_t)nmom)) &&
            QG_CUDA(cudaMemcpyAsync(dmom, mom, sizeof(int) * 3 * (size_t)nmom, cudaMemcpyHostToDevice, st));
  if (ok) {
    const int n = nt * V3;
    k_twop_block<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(p, geo, t0, nt, xsrc[0], block);
    ok = QG_LAUNCHED("twop_block");
  }
  if (ok) {
    k_twop_ft<<<(unsigned)(nt * nmom), 256, 0, st>>>(block, geo, dmom, nmom, xsrc[1], xsrc[2], xsrc[3], dcorr);
    ok = QG_LAUNCHED("twop_ft") &&
         QG_CUDA(cudaMemcpyAsync(corr, dcorr, sizeof(double2) * (size_t)nt * nmom, cudaMemcpyDeviceToHost, st)) &&
         QG_CUDA(cudaStreamSynchronize(st));
  }
  cudaFree(block);
  cudaFree(dcorr);
  cudaFree(dmom);
  return ok;
}

}  // namespace qg

extern "C" {

int qcdgpu_twop_proton(const qcdgpu_field *up, const qcdgpu_field *dn, const int xsrc[4], int t0, int t1,
                       const int *mom, int nmom, double *corr)
{
  return qg::twop_proton(up, dn, xsrc, t0, t1, mom, nmom, corr) ? 0 : 1;
}

}  // extern "C"
