// Per-step right-hand-side kernels of the IMEX loop.
//
// k_carrier_rhs restates assemble_local_semiconductor_rhs /
// assemble_local_electrolyte_rhs plus the M u^{n-1} mat-vec of
// assemble_semiconductor_rhs / assemble_electrolyte_rhs (reference
// source/SolarCell.cpp:1037-1726): drift q/eps (p . D) u^{n-1} with D the RT
// field of the Poisson solution evaluated at the carrier quadrature points,
// SRH, the semiconductor--electrolyte interface Robin transfer and Schottky
// terms; generation and Dirichlet data are time independent and arrive
// pre-assembled in `bconst`.  One thread per (cell, carrier): a k=1 cell owns
// 4 density dofs and 4 field dofs (96 bytes), so a warp per cell would leave
// most lanes idle; neighbouring threads read neighbouring dof blocks, so the
// loads of a warp are contiguous.
//
// k_poisson_rhs restates assemble_local_Poisson_rhs_for_semiconductor /
// _for_electrolyte (SolarCell.cpp:487-815): -(v, sum q_i u_i) on the Phi rows
// of the matching Poisson cell plus the constant doping/Dirichlet part.
#pragma once
#include "fp_bits.cuh"
#include <type_traits>
#include <cuda_runtime.h>

namespace pecs {

struct Tables {
  const double* phi;   // n1*Q   carrier basis at cell qp
  const double* qw;    // Q
  const double* fphi;  // 4*n1*nq face values
  const double* fw;    // nq
  const double* psix;  // nrt*Q  RT basis x-component at cell qp
  const double* psiy;  // nrt*Q
  const double* phiP;  // nphi*Q Poisson DGQ_{k-1} basis at cell qp
  const double* mref;  // n1*n1  unit-square mass matrix
  // FP32 copies for the mixed-precision path
  const float *phi_f, *qw_f, *fphi_f, *fw_f, *psix_f, *psiy_f;
  // drift tensors of the current equations, sum_q phi_a phi_b psi_c w_q on
  // the unit square, over the RT basis functions with a non-zero x (y)
  // component only -- nrt/2 of them on rectangles: [a][b][j], n1*n1*(nrt/2)
  const double *drift_x, *drift_y;
  const int *drift_cx, *drift_cy;  // their RT indices, nrt/2 each
  // Poisson charge matrix sum_q phiP_a phi_b w_q on the unit square, nphi x n1
  const double* charge;
  // FP32-pair copies (hi, lo) of the drift tensors and the mass matrix for the
  // mixed-precision path
  const float2 *drift_x_ff, *drift_y_ff, *mref_ff;
};

struct RegionDev {
  int nc;              // cells
  int nd;              // dofs per carrier vector
  int field1;          // PECS_FIELD_N (semi) or PECS_FIELD_R (elec)
  int is_semi;
  int iface_face;      // face of this region's cells on the interface
  int partner_face;    // face of the partner cell
  double inv_eps;      // 1/permittivity of the region
  double inv_dt;
  const double2* h;    // (hx, hy) per cell
  const int4* bid;     // boundary id per face (-1 interior)
  const int* rt;       // nc*nrt Poisson RT dofs of the matching Poisson cell
  const int* phid;     // nc*nphi Poisson Phi dofs
  const int* partner;  // partner cell in the other region or -1
  const int* iface;    // interface index or -1
  const double2* ph;   // partner (hx, hy)
};

struct InstDev {
  double k_et, k_ht, tau_n, tau_p, n_i, s_n, s_p;
  int srh;
  int pad;
};

struct FieldPtrs {
  const double* u[5];   // state read (instance stride nd[f])
  double* out[5];       // written vectors (rhs)
  const double* bc[5];  // constant rhs parts
  int nd[5];
};

// K: LDG degree; KP - 1: degree of the Poisson element RT_{KP-1} x DGQ_{KP-1}
// (KP = K: the reference's pairing, SolarCell.cpp:23-24; KP = K + 1: the
// RT_K x DGQ_K pairing of the benchmark configurations)
template <int K, int KP>
struct Dims {
  static constexpr int n1 = (K + 1) * (K + 1);
  static constexpr int nq = K + 2;
  static constexpr int Q = nq * nq;
  static constexpr int nrt = 2 * KP * (KP + 1);
  static constexpr int nphi = KP * KP;
};

// state values into the quadrature type, and quadrature sums back: on the
// integer pipe for the FP32 path (fp_bits.cuh), plain for FP64
template <typename Tq>
__device__ __forceinline__ Tq to_q(double x) {
  if constexpr (sizeof(Tq) == 4) return d2f_trunc(x); else return x;
}
template <typename Tq>
__device__ __forceinline__ double from_q(Tq x) {
  if constexpr (sizeof(Tq) == 4) return f2d_exact(x); else return x;
}

template <typename Tq>
__device__ __forceinline__ const Tq* tab(const double* d, const float* f);
template <>
__device__ __forceinline__ const double* tab<double>(const double* d, const float*) { return d; }
template <>
__device__ __forceinline__ const float* tab<float>(const double*, const float* f) { return f; }

// grid: x over (cells of both regions) * 2 carriers, y over instances.
// Tq is the arithmetic type of the quadrature terms (SRH, interface, Schottky,
// and in the FP64 path the drift).  Tq = double is the FP64 path.  Tq = float
// is the mixed path: (1/dt) M u^{n-1} and the drift term of the current
// equations, (q/eps) u D, keep ~47-bit accuracy -- the drift is large (|D|/h
// relative to the density terms) and its rounding would leave a per-step
// noise of ~eps32 |D| dt / h in the densities, above a 1e-8 steady-state
// criterion -- but run in FP32-pair arithmetic on the FP32 pipe (fp_bits.cuh;
// inputs split on the integer pipe), the drift as the bilinear form
// sum_bc T_abc u_b D_c with precomputed tensors; the small recombination and
// interface terms run in plain FP32, and only the final additions to the
// constant part are FP64 (GB300 issues FP32 operations ~60x faster than FP64,
// conversions included).
template <int K, int KP, typename Tq>
__global__ void __launch_bounds__(128, (K == 1 && sizeof(Tq) == 4) ? 8 : 1)
    k_carrier_rhs(Tables T, RegionDev semi, RegionDev elec, int n_regions, FieldPtrs F,
                  const InstDev* __restrict__ inst, const double* __restrict__ iface_ne,
                  const double* __restrict__ iface_pe, int n_iface, const double* __restrict__ sch_ne,
                  const double* __restrict__ sch_pe, const int* __restrict__ active) {
  using D = Dims<K, KP>;
  constexpr int n1 = D::n1, nq = D::nq, Q = D::Q, nrt = D::nrt;
  const int i = blockIdx.y;
  if (active && !active[i]) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nsemi2 = 2 * semi.nc;
  const int ntot = nsemi2 + (n_regions > 1 ? 2 * elec.nc : 0);
  if (t >= ntot) return;
  const bool in_semi = t < nsemi2;
  const RegionDev& R = in_semi ? semi : elec;
  const RegionDev& O = in_semi ? elec : semi;
  if (!in_semi) t -= nsemi2;
  const int c = t >> 1, which = t & 1;  // which: 0 carrier_1, 1 carrier_2
  const int f1 = R.field1, f = f1 + which;
  const int nc = R.nc, nd = R.nd;
  const InstDev P = inst[i];
  const Tq* phi = tab<Tq>(T.phi, T.phi_f);
  const Tq* qw = tab<Tq>(T.qw, T.qw_f);
  const Tq* fphi = tab<Tq>(T.fphi, T.fphi_f);
  const Tq* fw = tab<Tq>(T.fw, T.fw_f);
  const Tq* psix = tab<Tq>(T.psix, T.psix_f);
  const Tq* psiy = tab<Tq>(T.psiy, T.psiy_f);
  const double* u1p = F.u[f1] + (size_t)i * F.nd[f1] + 2 * nc * n1 + c * n1;
  const double* u2p = F.u[f1 + 1] + (size_t)i * F.nd[f1 + 1] + 2 * nc * n1 + c * n1;
  double uown[n1];
  Tq u1[n1], u2[n1];
#pragma unroll
  for (int a = 0; a < n1; ++a) {
    const double x1 = u1p[a], x2 = u2p[a];
    uown[a] = which ? x2 : x1;
    u1[a] = to_q<Tq>(x1);
    u2[a] = to_q<Tq>(x2);
  }
  const double* Pv = F.u[4] + (size_t)i * F.nd[4];
  Tq Dd[nrt];
#pragma unroll
  for (int b = 0; b < nrt; ++b) Dd[b] = to_q<Tq>(Pv[R.rt[c * nrt + b]]);
  const double2 h = R.h[c];
  const Tq hxhy_q = std::is_same<Tq, double>::value ? (Tq)(h.x * h.y) : to_q<Tq>(h.x) * to_q<Tq>(h.y);
  const Tq charge = which ? Tq(1) : Tq(-1);
  const Tq inv_eps = to_q<Tq>(R.inv_eps);
  // quadrature-term accumulators: [Jx (n1) | Jy (n1) | u (n1)]
  Tq r[3 * n1];
  float2 drift_ff[2 * n1];  // mixed path: FP32-pair drift of the current rows
#pragma unroll
  for (int a = 0; a < 2 * n1; ++a) drift_ff[a] = make_float2(0.f, 0.f);
#pragma unroll
  for (int a = 0; a < 3 * n1; ++a) r[a] = Tq(0);
  const bool srh = in_semi && P.srh;
  const Tq ni = to_q<Tq>(P.n_i), taun = to_q<Tq>(P.tau_n), taup = to_q<Tq>(P.tau_p);
#pragma unroll 1
  for (int q = 0; q < Q; ++q) {
    const Tq JxW = qw[q] * hxhy_q;
    Tq n = 0, p = 0;
#pragma unroll
    for (int a = 0; a < n1; ++a) {
      const Tq ph = phi[a * Q + q];
      n += ph * u1[a];
      p += ph * u2[a];
    }
    const Tq uq = which ? p : n;
    Tq Ex = 0, Ey = 0;
#pragma unroll
    for (int b = 0; b < nrt; ++b) {
      Ex += psix[b * Q + q] * Dd[b];
      Ey += psiy[b * Q + q] * Dd[b];
    }
    const Tq w = charge * inv_eps * uq * JxW;
    Tq Rq = 0;
    if (srh) Rq = (ni * ni - n * p) / (taun * (n + ni) + taup * (p + ni)) * JxW;
#pragma unroll
    for (int a = 0; a < n1; ++a) {
      const Tq ph = phi[a * Q + q];
      if constexpr (std::is_same<Tq, double>::value) {
        r[a] += ph * Ex * w;
        r[n1 + a] += ph * Ey * w;
      }
      r[2 * n1 + a] += ph * Rq;
    }
  }
  float2 uff[n1];  // mixed path: the own density in FP32 pairs
  if constexpr (!std::is_same<Tq, double>::value) {
#pragma unroll
    for (int a = 0; a < n1; ++a) uff[a] = d2ff(uown[a]);
    // drift of the current equations: (q/eps) hx hy sum_bj T_abj u_b D_j, each
    // product u_b D_j formed once and added into every row a
    constexpr int NC = nrt / 2;
#pragma unroll 1
    for (int j = 0; j < NC; ++j) {
      const float2 dx = d2ff(Pv[R.rt[c * nrt + T.drift_cx[j]]]);
      const float2 dy = d2ff(Pv[R.rt[c * nrt + T.drift_cy[j]]]);
#pragma unroll
      for (int b = 0; b < n1; ++b) {
        const float2 px = ff_mul(uff[b], dx), py = ff_mul(uff[b], dy);
#pragma unroll
        for (int a = 0; a < n1; ++a) {
          drift_ff[a] = ff_fma(T.drift_x_ff[(a * n1 + b) * NC + j], px, drift_ff[a]);
          drift_ff[n1 + a] = ff_fma(T.drift_y_ff[(a * n1 + b) * NC + j], py, drift_ff[n1 + a]);
        }
      }
    }
    float2 sc = ff_mul(ff_mul(d2ff(R.inv_eps), d2ff(h.x)), d2ff(h.y));
    if (!which) sc = make_float2(-sc.x, -sc.y);
#pragma unroll
    for (int a = 0; a < 2 * n1; ++a) drift_ff[a] = ff_mul(sc, drift_ff[a]);
  }
  // interface Robin transfer (SolarCell.cpp:1265-1347, 1630-1716)
  const int4 bid = R.bid[c];
  const int bids[4] = {bid.x, bid.y, bid.z, bid.w};
  if (n_regions > 1 && R.iface[c] >= 0 && bids[R.iface_face] == 0) {
    const int pc = R.partner[c], ii = R.iface[c];
    const double* o1p = F.u[O.field1] + (size_t)i * F.nd[O.field1] + 2 * O.nc * n1 + pc * n1;
    const double* o2p = F.u[O.field1 + 1] + (size_t)i * F.nd[O.field1 + 1] + 2 * O.nc * n1 + pc * n1;
    const int ff = R.iface_face, pf = R.partner_face;
    const Tq flen = to_q<Tq>((ff == 0 || ff == 1) ? h.y : h.x);
    const Tq ket = to_q<Tq>(P.k_et), kht = to_q<Tq>(P.k_ht);
#pragma unroll 1
    for (int q = 0; q < nq; ++q) {
      Tq a1 = 0, a2 = 0, b1 = 0, b2 = 0;
#pragma unroll
      for (int a = 0; a < n1; ++a) {
        const Tq fo = fphi[(ff * n1 + a) * nq + q];
        const Tq fp = fphi[(pf * n1 + a) * nq + q];
        a1 += fo * u1[a];
        a2 += fo * u2[a];
        b1 += fp * to_q<Tq>(o1p[a]);
        b2 += fp * to_q<Tq>(o2p[a]);
      }
      // semiconductor-side values n, p and electrolyte-side r, o
      const Tq n = in_semi ? a1 : b1, p = in_semi ? a2 : b2;
      const Tq rr = in_semi ? b1 : a1, oo = in_semi ? b2 : a2;
      const Tq ne = to_q<Tq>(iface_ne[(size_t)i * n_iface * nq + ii * nq + q]);
      const Tq pe = to_q<Tq>(iface_pe[(size_t)i * n_iface * nq + ii * nq + q]);
      const Tq Jf = fw[q] * flen;
      const Tq tn = -ket * (n - ne) * oo * Jf;
      const Tq tp = kht * (p - pe) * rr * Jf;
      Tq coef;
      if (in_semi)
        coef = which ? tp : tn;
      else
        coef = which ? -(tn + tp) : (tn + tp);
#pragma unroll
      for (int a = 0; a < n1; ++a) r[2 * n1 + a] += fphi[(ff * n1 + a) * nq + q] * coef;
    }
  }
  // Schottky faces (SolarCell.cpp:1348-1404)
  if (in_semi && sch_ne) {
#pragma unroll 1
    for (int fc = 0; fc < 4; ++fc) {
      if (bids[fc] != 3) continue;
      const Tq flen = to_q<Tq>((fc == 0 || fc == 1) ? h.y : h.x);
      for (int q = 0; q < nq; ++q) {
        Tq val = 0;
#pragma unroll
        for (int a = 0; a < n1; ++a) val += fphi[(fc * n1 + a) * nq + q] * (which ? u2[a] : u1[a]);
        const size_t o = (size_t)i * nc * 4 * nq + (size_t)(c * 4 + fc) * nq + q;
        const Tq Jf = fw[q] * flen;
        const Tq coef = which ? to_q<Tq>(P.s_p) * (val - to_q<Tq>(sch_pe[o])) * Jf
                              : -to_q<Tq>(P.s_n) * (val - to_q<Tq>(sch_ne[o])) * Jf;
#pragma unroll
        for (int a = 0; a < n1; ++a) r[2 * n1 + a] += fphi[(fc * n1 + a) * nq + q] * coef;
      }
    }
  }
  // constant part + (1/dt) M u^{n-1} (FP64, or FP32 pairs in the mixed path),
  // then the quadrature terms
  const double* bcp = F.bc[f] + (size_t)i * nd;
  double* outp = F.out[f] + (size_t)i * nd;
#pragma unroll
  for (int comp = 0; comp < 2; ++comp)
#pragma unroll
    for (int a = 0; a < n1; ++a) {
      const size_t o = (size_t)comp * nc * n1 + c * n1 + a;
      if constexpr (std::is_same<Tq, double>::value)
        outp[o] = bcp[o] + (double)r[comp * n1 + a];
      else
        outp[o] = ff2d_i32(ff_add(d2ff(bcp[o]), drift_ff[comp * n1 + a]));
    }
  if constexpr (std::is_same<Tq, double>::value) {
#pragma unroll
    for (int a = 0; a < n1; ++a) {
      double s = 0.0;
#pragma unroll
      for (int b = 0; b < n1; ++b) s += T.mref[a * n1 + b] * uown[b];
      const size_t o = (size_t)2 * nc * n1 + c * n1 + a;
      outp[o] = bcp[o] + s * (h.x * h.y) * R.inv_dt + from_q<Tq>(r[2 * n1 + a]);
    }
  } else {
    const float2 md = ff_mul(ff_mul(d2ff(h.x), d2ff(h.y)), d2ff(R.inv_dt));
#pragma unroll
    for (int a = 0; a < n1; ++a) {
      float2 s = make_float2(0.f, 0.f);
#pragma unroll
      for (int b = 0; b < n1; ++b) s = ff_fma(T.mref_ff[a * n1 + b], uff[b], s);
      const size_t o = (size_t)2 * nc * n1 + c * n1 + a;
      outp[o] = ff2d_i32(ff_add(ff_add(d2ff(bcp[o]), ff_mul(s, md)), r[2 * n1 + a]));
    }
  }
}

// grid: x over max(n_rt_total, cells of both regions), y over instances
template <int K, int KP>
__global__ void __launch_bounds__(128)
    k_poisson_rhs(Tables T, RegionDev semi, RegionDev elec, int n_regions, FieldPtrs F,
                  int n_rt_total, const int* __restrict__ active) {
  using D = Dims<K, KP>;
  constexpr int n1 = D::n1, Q = D::Q, nphi = D::nphi;
  const int i = blockIdx.y;
  if (active && !active[i]) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double* bc = F.bc[4] + (size_t)i * F.nd[4];
  double* out = F.out[4] + (size_t)i * F.nd[4];
  if (t < n_rt_total) out[t] = bc[t];
  const int ntot = semi.nc + (n_regions > 1 ? elec.nc : 0);
  if (t >= ntot) return;
  const bool in_semi = t < semi.nc;
  const RegionDev& R = in_semi ? semi : elec;
  const int c = in_semi ? t : t - semi.nc;
  const int f1 = R.field1;
  const double* u1 = F.u[f1] + (size_t)i * F.nd[f1] + 2 * R.nc * n1 + c * n1;
  const double* u2 = F.u[f1 + 1] + (size_t)i * F.nd[f1 + 1] + 2 * R.nc * n1 + c * n1;
  const double2 h = R.h[c];
  // charge density (-u1 + u2) (charge numbers -1, +1) against the Poisson test
  // functions: the quadrature folded into the nphi x n1 matrix T.charge, so
  // each cell costs nphi * n1 FP64 FMAs
  double du[n1];
#pragma unroll
  for (int b = 0; b < n1; ++b) du[b] = u2[b] - u1[b];
  const double hxhy = h.x * h.y;
  double acc[nphi];
#pragma unroll
  for (int a = 0; a < nphi; ++a) {
    double t = 0.0;
#pragma unroll
    for (int b = 0; b < n1; ++b) t += T.charge[a * n1 + b] * du[b];
    acc[a] = t * hxhy;
  }
#pragma unroll
  for (int a = 0; a < nphi; ++a) {
    const int d = R.phid[c * nphi + a];
    out[d] = bc[d] - acc[a];
  }
}

}  // namespace pecs
