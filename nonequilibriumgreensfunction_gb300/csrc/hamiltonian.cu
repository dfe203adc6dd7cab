// On-device Build_Hamiltonian (Source/Build_Hamiltonian.F90:1-303, open boundaries): one
// slot's Htotd (npx slices of M x M, column-major) is written in HBM from a table of
// norb x norb site blocks (norb <= 4: the channel models 0-4 of :13-47 have 4, 4, 1, 2 and 2
// orbitals), so a request ships a few hundred bytes instead of npx*M^2*16.
//
// The host computes the blocks that involve rounding (the y hop times its Landau-gauge
// phase, one block per z, Source/Build_Hamiltonian.F90:186-207); the kernel only places
// them, conjugates the lower triangle and adds the on-site potential, so the device result
// equals a host build with the same arithmetic bit for bit.  The Anderson potential comes
// from a counter-based stream (the i-th SplitMix64 output for site i), generated in the
// kernel where it is needed.
#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.h"

namespace negf {

namespace {

constexpr double kPi = 3.14159265358979323846;

// SplitMix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014): output i of the generator seeded with `seed`.
__host__ __device__ __forceinline__ unsigned long long splitmix64(unsigned long long seed, unsigned long long i) {
  unsigned long long z = seed + i * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Anderson potential of site (x, y, z): (u - 1/2) W on slices 2..npx-1, u in [0, 1) with 53 bits
__host__ __device__ __forceinline__ double anderson(unsigned long long seed, double W, int npx, int npy, int x, int y,
                                                    int z) {
  if (x == 0 || x == npx - 1) return 0.0;
  const unsigned long long i = (unsigned long long)x + (unsigned long long)npx * (y + (unsigned long long)npy * z);
  const double u = (double)(splitmix64(seed, i + 1) >> 11) * 0x1.0p-53;
  return (u - 0.5) * W;
}

// tab: [0..15] on-site block, [16..31] hop_z, [32 + 16 z ..] hop_y times the phase of layer z;
// each block row-major [a][b] with a row stride of 4 whatever norb.  The on-site potential
// of a site is V (npx*npy*npz, column-major, may be null) plus the counter-based Anderson
// potential, on each of its norb orbitals (Insert_Impurity, :154-165).
__global__ void build_h_kernel(int npx, int npy, int npz, int norb, const double2* __restrict__ tab,
                               const double* __restrict__ V, unsigned long long seed, double W, double2* H) {
  const int x = blockIdx.y;
  const int nsite = npy * npz;
  const int n = norb * nsite;
  const long long nn = (long long)n * n;
  double2* Hx = H + (long long)x * nn;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x) {
    const int col = (int)(e / n), row = (int)(e % n);
    const int rs = row / norb, ra = row - rs * norb, cs = col / norb, ca = col - cs * norb;
    double2 v = make_double2(0.0, 0.0);
    if (rs == cs) {
      v = tab[ra * 4 + ca];
      if (ra == ca) {
        const int y = rs % npy, z = rs / npy;
        const double vext = V ? V[x + (long long)npx * (y + (long long)npy * z)] : 0.0;
        v.x += vext + anderson(seed, W, npx, npy, x, y, z);
      }
    } else if (cs == rs + 1 && rs % npy + 1 < npy) {          // H(s, s + e_y)
      v = tab[32 + 16 * (rs / npy) + ra * 4 + ca];
    } else if (rs == cs + 1 && cs % npy + 1 < npy) {          // H(s + e_y, s) = H(s, s + e_y)^H
      const double2 t = tab[32 + 16 * (cs / npy) + ca * 4 + ra];
      v = make_double2(t.x, -t.y);
    } else if (cs == rs + npy) {                               // H(s, s + e_z)
      v = tab[16 + ra * 4 + ca];
    } else if (rs == cs + npy) {                               // H(s + e_z, s)
      const double2 t = tab[16 + ca * 4 + ra];
      v = make_double2(t.x, -t.y);
    }
    Hx[e] = v;
  }
}

double2 block_entry(const double (*b)[4][2], int r, int c) { return make_double2(b[r][c][0], b[r][c][1]); }

}  // namespace

int Engine::build_hamiltonian(int slot, const negf_wire_model& m) {
  // a plain (not BdG) Hamiltonian of at most 4 orbitals per site
  const int no = p_.norb;
  if (slot < 0 || slot >= p_.n_hamiltonians || no > 4 || sc_()) return NEGF_EINVAL;
  for (int i = 0; i < 8; ++i)
    if (m.reserved[i] != 0) return NEGF_EINVAL;
  NEGF_CUDA_TRY(cudaSetDevice(p_.device));
  const int npx = p_.npx, npy = p_.npy, npz = p_.npz;
  // block table: on-site, hop_z, then hop_y e^{i 2 pi z flux / ((npy-1)(npz-1))} per layer z
  std::vector<double2> tab((size_t)16 * (2 + npz));
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      // entries outside the leading norb x norb block must be zero
      if (a >= no || b >= no) {
        for (const double (*blk)[4][2] : {m.onsite, m.hop[0], m.hop[1], m.hop[2]})
          if (blk[a][b][0] != 0.0 || blk[a][b][1] != 0.0) return NEGF_EINVAL;
      }
      tab[a * 4 + b] = block_entry(m.onsite, a, b);
      tab[16 + a * 4 + b] = block_entry(m.hop[2], a, b);
    }
  const bool phased = m.flux != 0.0 && npy > 1 && npz > 1;
  for (int z = 0; z < npz; ++z) {
    double c = 1.0, s = 0.0;
    if (phased) {
      const double th = 2.0 * kPi * z * m.flux / (double)((npy - 1) * (npz - 1));
      c = std::cos(th);
      s = std::sin(th);
    }
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) {
        const double2 h = block_entry(m.hop[1], a, b);
        tab[32 + 16 * z + a * 4 + b] = phased ? make_double2(h.x * c - h.y * s, h.x * s + h.y * c) : h;
      }
  }
  // HopX: hop_x on every site (Source/Build_Hamiltonian.F90:59-64)
  std::vector<double2> hx((size_t)MM_, make_double2(0.0, 0.0));
  for (int st = 0; st < nsite_; ++st)
    for (int a = 0; a < no; ++a)
      for (int b = 0; b < no; ++b) hx[(size_t)(st * no + b) * M_ + st * no + a] = block_entry(m.hop[0], a, b);
  NEGF_TRY(set_hopx(hx.data()));

  const long long total = nsite_total();
  double2* Hs = dH_ + (long long)slot * npx * MM_;
  NEGF_CUDA_TRY(cudaMemcpyAsync(dHtab_, tab.data(), sizeof(double2) * tab.size(), cudaMemcpyHostToDevice, st_));
  if (m.V) NEGF_CUDA_TRY(cudaMemcpyAsync(dVext_, m.V, sizeof(double) * total, cudaMemcpyHostToDevice, st_));
  const long long per = (MM_ + 255) / 256;
  dim3 grid((unsigned)std::min<long long>(per, 1024), npx);
  build_h_kernel<<<grid, 256, 0, st_>>>(npx, npy, npz, no, dHtab_, m.V ? dVext_ : nullptr, (unsigned long long)m.seed, m.W,
                                        Hs);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  // host copies of the end slices decide which slots share a Sancho-Rubio decimation
  end_h1_[slot].resize(MM_);
  end_hn_[slot].resize(MM_);
  NEGF_CUDA_TRY(cudaMemcpyAsync(end_h1_[slot].data(), Hs, sizeof(double2) * MM_, cudaMemcpyDeviceToHost, st_));
  NEGF_CUDA_TRY(cudaMemcpyAsync(end_hn_[slot].data(), Hs + (long long)(npx - 1) * MM_, sizeof(double2) * MM_,
                                cudaMemcpyDeviceToHost, st_));
  NEGF_CUDA_TRY(cudaStreamSynchronize(st_));
  slot_set_[slot] = 1;
  recompute_lead_classes();
  sr_valid_ = rgf_valid_ = dens_valid_ = false;
  return NEGF_OK;
}

}  // namespace negf
