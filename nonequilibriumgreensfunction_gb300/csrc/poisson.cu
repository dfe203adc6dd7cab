// Electrostatics of the self-consistent bias point on the device: the role of SIP_V1
// (Source/SIP_Solver.F90:36-201) in the Poisson <-> NEGF loop of Source/NEGF_Main.F90:7-38.
//
// The system is the 7-point Laplacian on the npx x npy x npz site grid with Dirichlet
// values outside it (contacts at x = -1 and x = npx, a gate on every y and z face):
//     6 U_i - sum_{in-grid neighbours j} U_j = kappa rho_i + (boundary values next to i).
// It is symmetric positive definite, so it is solved by conjugate gradients instead of the
// reference's strongly implicit procedure, whose recurrences run along all three axes and
// leave a GPU idle.  A grid has at most a few 10^4 sites, so one CTA solves one grid with
// its four vectors in global memory (they stay in L2), and the dot products are block
// reductions in a fixed order: the result is deterministic.  Grids of different disorder
// samples are independent CTAs of one launch.
#include <algorithm>
#include <cmath>
#include <vector>

#include "negf_internal.cuh"

namespace negf {

namespace {

constexpr int PCG_THREADS = 1024;

__device__ __forceinline__ double apply_a(const double* v, int i, int nx, int ny, int nz) {
  const int x = i % nx, yz = i / nx, y = yz % ny, z = yz / ny;
  double s = 6.0 * v[i];
  if (x > 0) s -= v[i - 1];
  if (x < nx - 1) s -= v[i + 1];
  if (y > 0) s -= v[i - nx];
  if (y < ny - 1) s -= v[i + nx];
  if (z > 0) s -= v[i - nx * ny];
  if (z < nz - 1) s -= v[i + nx * ny];
  return s;
}

// sum over the CTA in a fixed order; every thread gets the result
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (l == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// b: right-hand sides, u: initial guesses -> solutions, work: 3 vectors per grid.
// Stops when ||b - A u|| <= tol ||b|| or after max_iter steps (a bounded loop).
__global__ void __launch_bounds__(PCG_THREADS) poisson_cg_kernel(int nx, int ny, int nz, const double* b, double* u,
                                                                 double* work, double tol, int max_iter, int* iters,
                                                                 double* rel) {
  __shared__ double red[33];
  const int n = nx * ny * nz;
  const long long g = blockIdx.x;
  const double* bg = b + g * n;
  double* ug = u + g * n;
  double* r = work + g * 3LL * n;
  double* p = r + n;
  double* q = p + n;
  double rr = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double ri = bg[i] - apply_a(ug, i, nx, ny, nz);
    r[i] = ri;
    p[i] = ri;
    rr += ri * ri;
    bb += bg[i] * bg[i];
  }
  rr = block_sum(rr, red);
  bb = block_sum(bb, red);
  const double thr = tol * tol * bb;
  int it = 0;
  for (; it < max_iter && rr > thr; ++it) {
    double pq = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double qi = apply_a(p, i, nx, ny, nz);
      q[i] = qi;
      pq += p[i] * qi;
    }
    pq = block_sum(pq, red);
    if (!(pq > 0.0)) break;             // breakdown (cannot happen for an SPD operator)
    const double alpha = rr / pq;
    double rn = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      ug[i] += alpha * p[i];
      const double ri = r[i] - alpha * q[i];
      r[i] = ri;
      rn += ri * ri;
    }
    rn = block_sum(rn, red);
    const double beta = rn / rr;
    rr = rn;
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = r[i] + beta * p[i];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    iters[g] = it;
    rel[g] = bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
  }
}

// b = kappa rho + the Dirichlet values of the neighbours outside the grid
__global__ void poisson_rhs_kernel(int nx, int ny, int nz, int grids, const double* rho, double kappa, double ul,
                                   double ur, double ug, double* b) {
  const long long n = (long long)nx * ny * nz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n * grids;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n);
    const int x = i % nx, yz = i / nx, y = yz % ny, z = yz / ny;
    double v = kappa * rho[e];
    if (x == 0) v += ul;
    if (x == nx - 1) v += ur;
    if (y == 0) v += ug;
    if (y == ny - 1) v += ug;
    if (z == 0) v += ug;
    if (z == nz - 1) v += ug;
    b[e] = v;
  }
}

struct DevMem {
  void* p = nullptr;
  ~DevMem() { if (p) cudaFree(p); }
  int alloc(size_t bytes) { return cudaMalloc(&p, bytes) == cudaSuccess ? NEGF_OK : NEGF_ENOMEM; }
};

}  // namespace

}  // namespace negf

extern "C" int negf_poisson_solve(int32_t npx, int32_t npy, int32_t npz, int32_t n_grids, const double* rho,
                                  const double* bc, double kappa, double* U, double tol, int32_t max_iter,
                                  int32_t* iters) {
  using namespace negf;
  if (npx < 1 || npy < 1 || npz < 1 || n_grids < 1 || !rho || !bc || !U || !(tol >= 0.0) || max_iter < 0)
    return NEGF_EINVAL;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NEGF_ENODEV;
  const long long n = (long long)npx * npy * npz;
  if (n > (1LL << 28)) return NEGF_EINVAL;
  const size_t vec = sizeof(double) * n * n_grids;
  for (long long i = 0; i < n * n_grids; ++i)
    if (!std::isfinite(rho[i])) return NEGF_ENAN;
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(bc[i])) return NEGF_EINVAL;
  DevMem dRho, dB, dU, dW, dIt, dRel;
  NEGF_TRY(dRho.alloc(vec));
  NEGF_TRY(dB.alloc(vec));
  NEGF_TRY(dU.alloc(vec));
  NEGF_TRY(dW.alloc(3 * vec));
  NEGF_TRY(dIt.alloc(sizeof(int) * n_grids));
  NEGF_TRY(dRel.alloc(sizeof(double) * n_grids));
  NEGF_CUDA_TRY(cudaMemcpy(dRho.p, rho, vec, cudaMemcpyHostToDevice));
  NEGF_CUDA_TRY(cudaMemcpy(dU.p, U, vec, cudaMemcpyHostToDevice));
  const long long total = n * n_grids;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 1024);
  poisson_rhs_kernel<<<blocks, 256>>>(npx, npy, npz, n_grids, (const double*)dRho.p, kappa, bc[0], bc[1], bc[2],
                                      (double*)dB.p);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  poisson_cg_kernel<<<n_grids, PCG_THREADS>>>(npx, npy, npz, (const double*)dB.p, (double*)dU.p, (double*)dW.p, tol,
                                              max_iter, (int*)dIt.p, (double*)dRel.p);
  NEGF_CUDA_TRY(cudaGetLastError());
  count_launch();
  NEGF_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<int> it(n_grids);
  std::vector<double> rel(n_grids);
  NEGF_CUDA_TRY(cudaMemcpy(it.data(), dIt.p, sizeof(int) * n_grids, cudaMemcpyDeviceToHost));
  NEGF_CUDA_TRY(cudaMemcpy(rel.data(), dRel.p, sizeof(double) * n_grids, cudaMemcpyDeviceToHost));
  NEGF_CUDA_TRY(cudaMemcpy(U, dU.p, vec, cudaMemcpyDeviceToHost));
  int worst = 0;
  bool ok = true;
  for (int g = 0; g < n_grids; ++g) {
    worst = std::max(worst, it[g]);
    if (!(rel[g] <= tol)) ok = false;
  }
  if (iters) *iters = worst;
  return ok ? NEGF_OK : NEGF_EREFINE;
}
