// vk_common.cu -- small kernels shared by both precisions.
#include "vk_kernels.cuh"
#include "vk_particles.cuh"

namespace vk {

__global__ void k_chempot(const double* __restrict__ part, int nblk, double* __restrict__ omega, double dt,
                          double nun_area, double dvol, double nparticle) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double norm = 0.0;
  for (int i = 0; i < nblk; ++i) norm += part[i];
  norm = norm * dvol;
  *omega = *omega - dt * nun_area * (norm - nparticle);
}

// Fixed-order sum of per-CTA partials part[i*3 + j] -> out[j], j = 0..2.
// One block; each thread strides the partial list, then a fixed-shape tree.
__global__ void k_reduce_partials3(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  __shared__ double sh[3][256];
  double a = 0.0, b = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += part[3 * i + 0];
    b += part[3 * i + 1];
    c += part[3 * i + 2];
  }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = b;
  sh[2][threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
      sh[2][threadIdx.x] += sh[2][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sh[0][0];
    out[1] = sh[1][0];
    out[2] = sh[2][0];
  }
}

// spec[j*nsh + m] = sum_b hpart[b][j][m], fixed order over the CTAs b.
__global__ void k_spec_reduce(const double* __restrict__ hpart, int nblk, int nsh, double* __restrict__ spec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 6 * nsh) return;
  double a = 0.0;
  for (int b = 0; b < nblk; ++b) a += hpart[(size_t)b * 6 * nsh + i];
  spec[i] = a;
}

// e^{i k qx} for kx in [0,K] and e^{i k qy} for ky in [0, ny) (kwn order).
__global__ void k_part_tables(PartState ps, PartConsts c) {
  const int nx_tab = c.K + 1;
  const int tot = c.np * (nx_tab + c.ny);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += gridDim.x * blockDim.x) {
    double sn, cs;
    if (i < c.np * nx_tab) {
      const int p = i / nx_tab, k = i % nx_tab;
      sincos((double)k * ps.pos[2 * p], &sn, &cs);
      ps.tab_x[2 * i] = cs;
      ps.tab_x[2 * i + 1] = sn;
    } else {
      const int j = i - c.np * nx_tab;
      const int p = j / c.ny, k = j % c.ny;
      const int kw = k < c.ny / 2 ? k : k - c.ny;
      sincos((double)kw * ps.pos[2 * p + 1], &sn, &cs);
      ps.tab_y[2 * j] = cs;
      ps.tab_y[2 * j + 1] = sn;
    }
  }
}

// Particle update of one RK4 stage (gp_particle_motion_rk4), or with
// STAGE == 0 only the force evaluation at the current positions (the
// diagnostics loop, src/diagnostics.f90:528-533).  One CTA of kPartThreads.
//
// The reference updates the particles one after another, and particle i's
// repulsion sees particles j < i at their new positions (:456-467).  A
// particle's new position depends only on its velocity before the update
// (k_q = dt v), not on any force, so all new positions are computed first;
// then every particle's force is independent of the others' and one warp
// per particle evaluates it:
//  1. fluid forces: warp w sums the per-CTA Parseval partials of particles
//     w, w + nwarps, ...: lane l over blocks l, l + 32, ... in increasing
//     order, then a fixed shuffle tree (lane 0's sum is the same every run);
//  2. new positions of all particles;
//  3. per particle: the repulsion terms over j (new positions for j < i, the
//     old ones for j > i and for i itself) on the lanes and a shuffle tree,
//     then lane 0 adds the fluid and external forces and updates the velocity.
__device__ __forceinline__ double ipow_d(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kPartThreads) k_part_update(PartState ps, PartConsts c, int stage) {
  const int np = c.np;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  // Up to kPartSmemMax particles the state lives in shared memory (the launch
  // passes part_update_smem(np) bytes); above that in global memory, with
  // the new positions in the tab_x scratch (rebuilt from the positions
  // before every force pass).
  extern __shared__ double psm[];
  const bool sm = np <= kPartSmemMax;
  const size_t n2 = 2 * (size_t)np;
  double* pos = sm ? psm : ps.pos;
  double* vel = sm ? psm + n2 : ps.vel;
  double* tpos = sm ? psm + 2 * n2 : ps.tpos;
  double* tvel = sm ? psm + 3 * n2 : ps.tvel;
  double* f0 = sm ? psm + 4 * n2 : ps.f0ext;
  double* frc = sm ? psm + 5 * n2 : ps.frc;
  double* posn = sm ? psm + 6 * n2 : ps.tab_x;
  for (int i = threadIdx.x; i < 2 * np; i += blockDim.x) {
    if (sm) {
      pos[i] = ps.pos[i];
      vel[i] = ps.vel[i];
      f0[i] = ps.f0ext[i];
      if (stage != 1) {
        tpos[i] = ps.tpos[i];
        tvel[i] = ps.tvel[i];
      }
    }
    if (stage == 1) {
      tvel[i] = vel[i];
      tpos[i] = pos[i];
    }
  }
  const double fl = -2.0 * c.alpha * c.dvol * c.scale;  // -2 alpha dvol (1/N^2)
  for (int ip = warp; ip < np; ip += nwarp) {
    // sum_x d rho V_i = f/N^2 (Parseval); force = -2 alpha dvol * that
    double g0 = 0.0, g1 = 0.0;
    for (int b = lane; b < c.nblk; b += 32) {
      g0 += ps.fpart[(size_t)b * n2 + 2 * ip];
      g1 += ps.fpart[(size_t)b * n2 + 2 * ip + 1];
    }
    g0 = warp_sum_d(g0);
    g1 = warp_sum_d(g1);
    if (lane == 0) {
      frc[2 * ip] = g0 * fl;
      frc[2 * ip + 1] = g1 * fl;
    }
  }
  __syncthreads();
  // new positions (k_q = dt v with the velocity before this stage's update)
  for (int i = threadIdx.x; i < 2 * np; i += blockDim.x) {
    double q = pos[i];
    if (stage > 0) {
      const double kq = c.dt * vel[i];
      ps.kq[(stage - 1) * n2 + i] = kq;
      if (stage == 1 || stage == 2) q = tpos[i] + 0.5 * kq;
      else if (stage == 3) q = tpos[i] + kq;
      else {
        const double* Q1 = ps.kq;
        q = tpos[i] + (1.0 / 6.0) * (Q1[i] + 2.0 * Q1[n2 + i] + 2.0 * Q1[2 * n2 + i] + kq);
      }
    }
    posn[i] = q;
  }
  __syncthreads();
  for (int ip = warp; ip < np; ip += nwarp) {
    // short-range repulsion (shortrange_repulsion, :378-427): particles
    // j < ip at their new positions, the others and ip itself at the old ones
    double r0 = 0.0, r1 = 0.0;
    if (np > 1)
      for (int j = lane; j < np; j += 32) {
        if (j == ip) continue;
        const double* qj = j < ip ? posn : pos;
        const double x = pos[2 * ip] - qj[2 * j], y = pos[2 * ip + 1] - qj[2 * j + 1];
        const double den = ipow_d(-3.0 + cos(x) + cos(y), 7);
        r0 += -c.rep_factor * sin(x) / den;
        r1 += -c.rep_factor * sin(y) / den;
      }
    r0 = warp_sum_d(r0);
    r1 = warp_sum_d(r1);
    if (lane == 0) {
      const double rep[2] = {r0, r1};
      for (int d = 0; d < 2; ++d) {
        const int i = 2 * ip + d;
        const double ft = frc[i] + rep[d] + f0[i];
        frc[i] = ft;
        if (stage == 0) continue;
        const double ku = c.dt * ft / c.mass;
        ps.ku[(stage - 1) * n2 + i] = ku;
        if (stage == 1 || stage == 2) vel[i] = tvel[i] + 0.5 * ku;
        else if (stage == 3) vel[i] = tvel[i] + ku;
        else {
          const double* K1 = ps.ku;
          vel[i] = tvel[i] + (1.0 / 6.0) * (K1[i] + 2.0 * K1[n2 + i] + 2.0 * K1[2 * n2 + i] + ku);
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * np; i += blockDim.x) {
    ps.pos[i] = posn[i];
    if (sm) {
      ps.vel[i] = vel[i];
      ps.frc[i] = frc[i];
      if (stage == 1) {
        ps.tpos[i] = tpos[i];
        ps.tvel[i] = tvel[i];
      }
    }
  }
}

// Seeded neutral vortex state on the device (FP64), same mathematics as the
// host vk_ic_vortices: amplitude prod_j A(r_j) with the periodic minimum-image
// distance, phase prod_j theta_1((z - z_j)/2 | e^{-pi})^{q_j} / |..| times
// exp(-i y S/(2 pi)), S = sum_j q_j x_j.
__global__ void k_ic_vortices(double2* __restrict__ out, int nx, int ny, const double* __restrict__ vx,
                              const double* __restrict__ vy, const int* __restrict__ vq, int nv, double xi0,
                              double S) {
  const double two_pi = 6.283185307179586476925286766559, pi = two_pi / 2;
  const double qn = exp(-pi);
  double q2n[10];
  for (int n = 1; n <= 9; ++n) q2n[n] = pow(qn, 2.0 * n);
  const size_t np = (size_t)nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < np; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / nx), x = (int)(i % nx);
    const double xx = x * (two_pi / nx), yy = y * (two_pi / ny);
    double amp = 1.0, pr = 1.0, pim = 0.0;
    for (int j = 0; j < nv; ++j) {
      const double ddx = xx - vx[j], ddy = yy - vy[j];
      double wx = fmod(ddx, two_pi), wy = fmod(ddy, two_pi);
      if (wx > pi) wx -= two_pi;
      if (wx <= -pi) wx += two_pi;
      if (wy > pi) wy -= two_pi;
      if (wy <= -pi) wy += two_pi;
      const double r = sqrt(wx * wx + wy * wy) / xi0;
      amp *= r / sqrt(2.0 + r * r);
      const double a = 0.5 * ddx, b = 0.5 * ddy;
      double sa, ca;
      sincos(a, &sa, &ca);
      double fr = sa * cosh(b), fi = ca * sinh(b);
      double s2, c2;
      sincos(ddx, &s2, &c2);
      const double em = exp(-ddy), ep = exp(ddy);
      for (int n = 1; n <= 9; ++n) {
        const double r1 = q2n[n] * em, r2 = q2n[n] * ep;
        const double ar = 1.0 - r1 * c2, ai = -r1 * s2;
        const double br = 1.0 - r2 * c2, bi = r2 * s2;
        const double tr = ar * br - ai * bi, ti = ar * bi + ai * br;
        const double nr = fr * tr - fi * ti, ni = fr * ti + fi * tr;
        fr = nr;
        fi = ni;
      }
      const double m = hypot(fr, fi);
      if (m > 0) {
        fr /= m;
        fi /= m;
      } else {
        fr = 1.0;
        fi = 0.0;
      }
      if (vq[j] < 0) fi = -fi;
      const double nr = pr * fr - pim * fi, ni = pr * fi + pim * fr;
      pr = nr;
      pim = ni;
    }
    double sl, cl;
    sincos(-yy * S / two_pi, &sl, &cl);
    const double fr = pr * cl - pim * sl, fi = pr * sl + pim * cl;
    const double m = hypot(fr, fi);
    out[i] = make_double2(amp * fr / m, amp * fi / m);
  }
}

}  // namespace vk
