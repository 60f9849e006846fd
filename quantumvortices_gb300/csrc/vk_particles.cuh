// vk_particles.cuh -- Gaussian-particle coupling (src/gpe_particle.f90) on the GPU.
//
// Per RK4 stage the reference calls translate_particle_potential(0) for the
// RHS (V_tot = F^-1[V^ sum_i e^{-ik.q_i}], :327-374) and, per particle i in
// index order, translate_particle_potential(i) (:219-324): 4 FFTs to get the
// force -2 alpha dvol sum_x Re(d rho . V_i) plus the 1/r^12 repulsion, then
// the RK4 update of that particle (gp_particle_motion_rk4, :429-531).
//
// Here every particle's fluid force comes out of ONE pass over Fourier space
// (Parseval, in the Y1 kernel that already holds the masked rho^ rows):
//   sum_x d_x rho(x) V_i(x) = (1/N^2) sum_k (i k_x rho^(k)) conj(e^{-ik.q_i} V^(k))
//                           = -(1/N^2) sum_k k_x Im[rho^(k) conj(V^(k)) e^{ik.q_i}]
// summed over the half plane kx in [0,K] with weight 2 for kx > 0 (rho, V
// real).  e^{ik.q_i} = ex_i(kx) ey_i(ky) from FP64 tables rebuilt from the
// stage positions; the same products give V^_tot for the RHS.  The
// per-particle update (repulsion sees particles j < i at their new
// positions, :456-467) runs in one CTA in FP64: the new positions do not
// depend on the forces, so every particle's force is evaluated in parallel.
#pragma once
#include "vk_kernels.cuh"

namespace vk {

struct PartState {  // device-resident, FP64, [p][d] layout (Fortran (1:2,1:P))
  double* pos;
  double* vel;
  double* tpos;
  double* tvel;
  double* ku;   // [4][P][2]
  double* kq;   // [4][P][2]
  double* f0ext;
  double* frc;  // force at the last evaluation
  double* tab_x;  // [P][K+1] complex: e^{i kx qx}
  double* tab_y;  // [P][ny]  complex: e^{i ky qy}
  double* fpart;  // [nblk][P][2] Parseval partial sums
};

struct PartConsts {
  int np, K, nx, ny, nblk;
  double dt, mass, alpha, dvol, scale;  // scale = 1/(nx ny)
  double rep_factor;                    // 384 dE pi^12 r0^12 / L^12
};

// e^{i k qx} for kx in [0,K] and e^{i k qy} for ky in [0, ny) (kwn order).
__global__ void k_part_tables(PartState ps, PartConsts c);

// Y1 with particles: rows kx in [0,K], RP = R/2 logical rows per CTA; smem
// rows [0,RP) = rho spectrum, [RP, 2RP) = V^_tot.  Writes P_G rho^ rows to Tc
// and V^_tot rows to Tv (both [y][kx], pitch pk), optionally the masked rho^
// rows (rhohat), and with FORCE the per-CTA Parseval partial sums
// fpart[blk][p][d] of -w kx Im[rho^ conj(V^) e^{ik.q_p}] (w = 2 for kx > 0).
// Particles are taken 16 at a time with register accumulators.
template <typename T, int L, bool FORCE>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_y1_pot(const cplx<T>* __restrict__ Tb, const cplx<T>* __restrict__ vhat,
                                                       cplx<T>* __restrict__ Tc, cplx<T>* __restrict__ Tv,
                                                       cplx<T>* __restrict__ rhohat, PartState ps, PartConsts pc,
                                                       const cplx<T>* __restrict__ tw, StepConsts c) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  constexpr int RP = G::R / 2;
  constexpr int NW = G::NT / 32 > 0 ? G::NT / 32 : 1;
  // Particle grids are >= 32 points per side (checked at vk_init), where
  // every geometry has whole warps; smaller instantiations are empty.
  if constexpr (G::NT % 32 != 0) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  __shared__ double red[NW][32];
  const int l0 = blockIdx.x * RP;
  const int K = c.K, np = pc.np;
  for (int e = threadIdx.x; e < RP * L; e += G::NT) {
    const int r = e / L, y = e % L;
    C v = mkc<T>(T(0), T(0));
    if (l0 + r <= K) v = Tb[(size_t)(l0 + r) * L + y];
    s[r * G::LP + pidx(y)] = v;
  }
  __syncthreads();
  fft_rows<T, L, RP, G::NT, -1, G::NT>(s, tw);
  // mask rho^ in place, zero V^_tot
  for (int e = threadIdx.x; e < RP * L; e += G::NT) {
    const int r = e / L, ky = e % L;
    const int kx = l0 + r, k2 = kwn(ky, L);
    if (kx > K || kx * kx + k2 * k2 > c.k2max) s[r * G::LP + pidx(ky)] = mkc<T>(T(0), T(0));
    if (rhohat && kx <= K) rhohat[(size_t)kx * L + ky] = s[r * G::LP + pidx(ky)];
    s[(RP + r) * G::LP + pidx(ky)] = mkc<T>(T(0), T(0));
  }
  for (int p0 = 0; p0 < np; p0 += 16) {
    double acc[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) acc[q] = 0.0;
    for (int e = threadIdx.x; e < RP * L; e += G::NT) {
      const int r = e / L, ky = e % L;
      const int kx = l0 + r, k2 = kwn(ky, L);
      if (kx > K || kx * kx + k2 * k2 > c.k2max) continue;
      const C rh = s[r * G::LP + pidx(ky)];
      const C vh = vhat[(size_t)kx * L + ky];
      const double cr = (double)rh.x * vh.x + (double)rh.y * vh.y;  // rho^ conj(V^)
      const double ci = (double)rh.y * vh.x - (double)rh.x * vh.y;
      const double wx = (kx == 0 ? -1.0 : -2.0) * (double)kx, wy = (kx == 0 ? -1.0 : -2.0) * (double)k2;
      double sr = 0.0, si = 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int p = p0 + q;
        if (p < np) {
          const double* tx = ps.tab_x + 2 * ((size_t)p * (K + 1) + kx);
          const double* ty = ps.tab_y + 2 * ((size_t)p * L + ky);
          const double ax = tx[0], ay = tx[1], bx = ty[0], by = ty[1];
          const double er = ax * bx - ay * by, ei = ax * by + ay * bx;  // e^{ik.q_p}
          sr += er;
          si -= ei;  // sum_p e^{-ik.q_p}
          if (FORCE) {
            const double im = cr * ei + ci * er;  // Im[rho^ conj(V^) e^{ik.q}]
            acc[2 * q] += wx * im;
            acc[2 * q + 1] += wy * im;
          }
        }
      }
      C vt = s[(RP + r) * G::LP + pidx(ky)];
      vt.x += T(vh.x * sr - vh.y * si);
      vt.y += T(vh.x * si + vh.y * sr);
      s[(RP + r) * G::LP + pidx(ky)] = vt;
    }
    if (FORCE) {
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == q) red[wid][q] = v;
      }
      __syncthreads();
      if (threadIdx.x < 32) {
        double v = 0.0;
        for (int w = 0; w < NW; ++w) v += red[w][threadIdx.x];
        const int q = threadIdx.x >> 1, p = p0 + q;
        if (p < np) ps.fpart[(size_t)blockIdx.x * 2 * np + 2 * p + (threadIdx.x & 1)] = v;
      }
      __syncthreads();
    }
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  for (int e = threadIdx.x; e < RP * L; e += G::NT) {
    const int r = e % RP, y = e / RP;
    if (l0 + r <= K) {
      Tc[(size_t)y * c.pk + l0 + r] = s[r * G::LP + pidx(y)];
      Tv[(size_t)y * c.pk + l0 + r] = s[(RP + r) * G::LP + pidx(y)];
    }
  }
}

// X2 with particles: per row Z(kx) = P^(kx) + i V^(kx) (Hermitian halves
// extended to negative kx) -> F^-1_x -> P_G rho + i V_tot;
// N = SIGN*(g P_G rho psi + V_tot psi) -> F_x -> Td.  When VOUT is set the
// real V_tot rows are also stored (diagnostics).
template <typename T, int L, int SIGN, bool PRUNE_OUT>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_x2_pot(const cplx<T>* __restrict__ Tc, const cplx<T>* __restrict__ Tv,
                                                       const cplx<T>* __restrict__ psi, cplx<T>* __restrict__ Td,
                                                       const cplx<T>* __restrict__ tw, StepConsts c) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int y0 = blockIdx.x * G::R;
  const int K = c.K, ny = c.ny, pk = c.pk;
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, k = e % L;
    C v = mkc<T>(T(0), T(0));
    const size_t ro = (size_t)(y0 + r) * pk;
    if (k <= K) {
      const C a = Tc[ro + k], b = Tv[ro + k];
      v = mkc<T>(a.x - b.y, a.y + b.x);
    } else if (k >= L - K) {
      const C a = Tc[ro + (L - k)], b = Tv[ro + (L - k)];
      v = mkc<T>(a.x + b.y, b.x - a.y);
    }
    s[r * G::LP + pidx(k)] = v;
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  const T g = T(c.g), scale = T(c.scale), sg = T(SIGN);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, x = e % L;
    const C z = s[r * G::LP + pidx(x)];
    const T pg = z.x * scale, vt = z.y * scale;
    const C ps = psi[(size_t)(y0 + r) * L + x];
    const T gp = g * pg;
    // g*P*psi + V*psi (src/gpe.f90:585-589); ARGLE negates both (:107-111)
    C n = mkc<T>(sg * (gp * ps.x + vt * ps.x), sg * (gp * ps.y + vt * ps.y));
    s[r * G::LP + pidx(x)] = n;
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, -1>(s, tw);
  if (PRUNE_OUT) {
    const int ncol = 2 * K + 1;
    for (int e = threadIdx.x; e < G::R * ncol; e += G::NT) {
      const int r = e % G::R, l = e / G::R;
      const int k = pruned_row(l, K, L);
      Td[(size_t)k * ny + y0 + r] = s[r * G::LP + pidx(k)];
    }
  } else {
    for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
      const int r = e % G::R, k = e / G::R;
      Td[(size_t)k * ny + y0 + r] = s[r * G::LP + pidx(k)];
    }
  }
}

// Real V_tot rows (diagnostics): Z = V^ Hermitian-extended, F^-1_x, real part.
template <typename T, int L>
__global__ void __launch_bounds__(GeoX<T, L>::NT, GeoX<T, L>::MINB) k_vtot_x(const cplx<T>* __restrict__ Tv, T* __restrict__ vout,
                                                       const cplx<T>* __restrict__ tw, StepConsts c) {
  typedef GeoX<T, L> G;
  typedef cplx<T> C;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* s = reinterpret_cast<C*>(smraw);
  const int y0 = blockIdx.x * G::R;
  const int K = c.K, pk = c.pk;
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, k = e % L;
    C v = mkc<T>(T(0), T(0));
    const size_t ro = (size_t)(y0 + r) * pk;
    if (k <= K) v = Tv[ro + k];
    else if (k >= L - K) v = cconj(Tv[ro + (L - k)]);
    s[r * G::LP + pidx(k)] = v;
  }
  __syncthreads();
  fft_rows<T, L, G::R, G::NT, +1>(s, tw);
  const T scale = T(c.scale);
  for (int e = threadIdx.x; e < G::R * L; e += G::NT) {
    const int r = e / L, x = e % L;
    vout[(size_t)(y0 + r) * L + x] = s[r * G::LP + pidx(x)].x * scale;
  }
}

// Sequential particle update of one RK4 stage (gp_particle_motion_rk4,
// src/gpe_particle.f90:429-531), or with stage == 0 only the force evaluation
// at the current positions (diagnostics loop, src/diagnostics.f90:528-533).
// One thread.
constexpr int kPartThreads = 256;  // block size of k_part_update
constexpr int kPartSmemMax = 512;  // particles whose state k_part_update keeps in shared memory
// Dynamic shared memory of a k_part_update launch for np particles.
inline size_t part_update_smem(int np) { return np <= kPartSmemMax ? sizeof(double) * 14 * (size_t)np : 0; }
__global__ void k_part_update(PartState ps, PartConsts c, int stage);

}  // namespace vk
