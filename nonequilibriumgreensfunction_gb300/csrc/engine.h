// Host-side engine: owns the device state of one negf_handle and orchestrates the
// per-energy solve as batched device kernels.
#pragma once

#include <array>
#include <map>
#include <vector>

#include "negf_internal.cuh"
#include "zgemm_tc.h"

namespace negf {

// Energy- and orbital-resolved arrays of a batched solve (Source/Calculate_Observables.F90:
// 124-160, Source/Calculate_Gnp.F90:125-129); every pointer may be null, values are added.
struct ResolvedOut {
  double* er[4] = {nullptr, nullptr, nullptr, nullptr};  // ERJx, ERJy, ERJz, ERRhon: nsite_total x n
  double* orj[3] = {nullptr, nullptr, nullptr};          // ORJx/y/z: nsite_total x norb^2 x slots
  double* orrho = nullptr;                               // ORRhon: nsite_total x norb x slots
  bool any_er() const { return er[0] || er[1] || er[2] || er[3]; }
  bool any_or() const { return orj[0] || orj[1] || orj[2] || orrho; }
};

struct SrJob {          // one Sancho-Rubio problem
  double energy;
  int slot;             // device end slice comes from this slot
  int use_last;         // alpha from H_N (1) or H_1 (0)
  int want_l, want_r;   // which lead outputs are used
};

class Engine {
 public:
  ~Engine();
  int init(const negf_params& p);
  // device bytes an engine with these parameters allocates at init (< 0: invalid
  // parameters); the serving layer admits engines by it
  static long long estimate_bytes(const negf_params& p);
  int set_hamiltonian(int slot, const double* Htotd, const double* HopX);
  // Htotd of `slot` generated on the device from a wire model (Build_Hamiltonian)
  int build_hamiltonian(int slot, const negf_wire_model& m);

  // Sancho-Rubio for a list of problems; outputs into sr_* buffers (index = problem)
  int solve_sr(const std::vector<SrJob>& jobs, std::vector<int>& status, std::vector<int>& iters);
  // RGF + Gn site blocks + traces for a batch of items (Sigma/Gamma gathered from SR)
  int solve_rgf(const std::vector<Item>& items, bool keep_columns);
  // densities/spin for the current batch (after solve_rgf) with the items' f1,f2,dE
  int densities(const std::vector<Item>& items, std::vector<double>& edens, std::vector<double>& hdens);

  // outs[8] = RhoN, RhoP, SigX, SigY, SigZ, Jx, Jy, Jz (each may be null).  site_items
  // (optional): n x nf_ x nsite_total per-request dE-weighted site arrays, so a caller can
  // sum energies in its own fixed order.  ro (optional, needs calc_currents): the energy-
  // and orbital-resolved arrays.
  int batch_solve(const negf_request* req, int n, negf_result* res, double* const* outs,
                  double* site_items = nullptr, const ResolvedOut* ro = nullptr);
  // energy- and orbital-resolved outputs of the batch in dItems_ (after densities): er_out
  // per item when `er`, or_acc += the batch's sums for slots 0..nslots-1 when `orb`
  int resolved(int batch, bool er, bool orb, int nslots);

  // accessors used by the per-energy API
  int M() const { return M_; }
  int npx() const { return p_.npx; }
  int nsite_total() const { return p_.npx * p_.npy * p_.npz; }
  long long bytes() const { return bytes_; }

  negf_params p_{};
  int M_ = 0, nsite_ = 0, B_ = 0, S_ = 0;
  long long MM_ = 0;
  cudaStream_t st_ = nullptr;       // stream the work runs on
  cudaStream_t own_st_ = nullptr;   // the handle's own stream
  long long bytes_ = 0;

  // Hamiltonian
  double2* dH_ = nullptr;
  double2* dHop_ = nullptr;
  double2* dHopBD_ = nullptr;
  bool hop_bd_ = false;
  // every site's HopX block is the same 4 x 4 block: compact terms of op(H) for each side,
  // hop_rows_[left][op == OP_C]
  bool hop_uniform_ = false;
  HopRows hop_rows_[2][2]{};
  bool hop_set_ = false;
  std::vector<int> slot_set_;
  // Slots whose end slices H_1 / H_N are bitwise identical share the Sancho-Rubio
  // decimation at a given energy: slot_rep_[s] is the first such slot.  slot_joint_[s]
  // is set when H_1 == H_N, so one decimation gives both leads.
  std::vector<std::vector<double2>> end_h1_, end_hn_;
  std::vector<int> slot_rep_, slot_joint_;
  void recompute_lead_classes();
  double2* dSpin_ = nullptr;
  double2* dHtab_ = nullptr;   // build_hamiltonian: site-block table (16 * (2 + npz))
  double* dVext_ = nullptr;    // build_hamiltonian: caller's potential (npx*npy*npz)

  // batch workspace
  double2 *dG_ = nullptr, *dC1_ = nullptr, *dCN_ = nullptr, *dZ_ = nullptr, *dY_ = nullptr, *dQ_ = nullptr;
  double2 *dSigL_ = nullptr, *dSigR_ = nullptr, *dGamL_ = nullptr, *dGamR_ = nullptr;
  double2 *dP1_ = nullptr, *dP2_ = nullptr;
  double2 *dCol1_ = nullptr, *dColN_ = nullptr;  // optional full columns for item 0
  // bond currents (calc_currents): +x/+y/+z neighbour site blocks of each lead, and second
  // buffers for Y = G(:,1) Gamma_L and G(:,N) so that slices x and x+1 are both at hand
  bool currents_ = false;
  int nh_ = 4;            // electron orbitals per site (norb, or norb / 2 with SC contacts)
  // model contacts (contact_type 1..3): Sigma from closed forms instead of Sancho-Rubio;
  // with SC contacts the G(1,1) site blocks are kept for the supercurrent trace
  int solve_contact_model(const std::vector<SrJob>& jobs, std::vector<int>& status, std::vector<int>& iters);
  double2* dContactCoef_ = nullptr;   // [S_][2][3]
  double2* dG11_ = nullptr;           // [B_][M][norb], SC contacts only
  double* dTrJ_ = nullptr;            // [B_] supercurrent transmission, SC contacts only
  bool sc_() const { return p_.contact_type == NEGF_CONTACT_SC; }
  int nf_ = 5;   // site fields per item: RhoN, RhoP, SigX, SigY, SigZ (+ Jx, Jy, Jz)
  double2 *dPx1_ = nullptr, *dPy1_ = nullptr, *dPz1_ = nullptr;
  double2 *dPx2_ = nullptr, *dPy2_ = nullptr, *dPz2_ = nullptr;
  double2 *dYalt_ = nullptr, *dCNalt_ = nullptr;
  // energy/orbital-resolved outputs, allocated on first use: dEr_ [B_][4][nsite_total],
  // dOrAcc_ [slots][3 norb^2 + norb][nsite_total]
  double* dEr_ = nullptr;
  double* dOrAcc_ = nullptr;
  int ensure_resolved();
  int n_or_fields() const { return 3 * p_.norb * p_.norb + p_.norb; }
  double* dSite_ = nullptr;
  double* dSums_ = nullptr;
  double* dTr_ = nullptr;
  double* dAcc_ = nullptr;  // slots * 5 * nsite_total
  int* dStatus_ = nullptr;
  Item* dItems_ = nullptr;
  int sums_blocks_ = 0;

  // Sancho-Rubio workspace (S_ problems)
  double2* dSr_ = nullptr;  // kSrBlocks * S_ blocks
  double2 *dSrSigL_ = nullptr, *dSrSigR_ = nullptr, *dSrGamL_ = nullptr, *dSrGamR_ = nullptr;
  double* dSrCmax_ = nullptr;
  double* dSrDos_ = nullptr;
  int* dSrActive_ = nullptr;
  double* dSrE_ = nullptr;
  const double2** dSrHend_ = nullptr;
  int* dSrStatus_ = nullptr;

  // pinned host staging
  double* hPin_ = nullptr;
  size_t hPinBytes_ = 0;

  InvWork inv_;

  // mixed form (NEGF_PREC_MIXED): tensor-core GEMMs on S integer BF16 slices, inverses as
  // FP32 Gauss-Jordan + Newton-Schulz steps with the residual at s_res_ slices
  bool mixed_ = false;
  int s_rgf_ = 5;      // RGF block products
  int s_sr_ = 8;       // Sancho-Rubio products: 2^-56, the decimation is ill-conditioned near band edges
  int s_res_ = 7;      // Newton-Schulz residual W X (2^-49, FP64-class)
  int s_res0_ = 5;     // the first residual (2^-35: the second step squares its error)
  int s_upd_ = 3;      // Newton-Schulz update X R: its error, ~sqrt(M) 2^-7S of |X||R|, must stay
                       // well below |R| for quadratic convergence; 2 slices (~1e-3 at M = 400)
                       // broke the mixed-form tolerance, 3 slices (~1e-5) keep it
  int ns_steps_ = 2;        // Newton-Schulz steps always taken
  int ns_max_steps_ = 4;    // more while the latest residual norm is above ns_tol_
  double ns_tol_ = 1e-5;     // residual norm before the last update; that update squares it
  double ns_accept_ = 0.5;   // first residual norm above this -> FP64 inverse for that matrix
  int cur_slices_ = 4;       // slices for the GEMMs issued now (set per phase)
  double2* dWinv_ = nullptr; // copy of the matrix being inverted (FP64)
  float2* dW32_ = nullptr;
  double2* dT_ = nullptr;
  SlicedOperand sa_, sb_, sw_;   // sw_: slices of the matrix under inversion (kept across NS steps)
  SlicedOperand sgl_, sgr_;      // Gamma_L, Gamma_R as B operands, sliced once per sweep
  unsigned long long* dRnorm_ = nullptr;
  int* dNsIdx_ = nullptr;     // matrices still taking Newton-Schulz steps beyond ns_steps_
  double2 *dNsX_ = nullptr, *dNsW_ = nullptr;   // their X and W, gathered into a compact batch
  long long ns_extra_ = 0;    // matrix-steps taken beyond ns_steps_ (statistics)
  long long ns_unconverged_ = 0;   // matrices still above ns_tol_ after ns_max_steps_ (redone in FP64)
  double last_rk_max_ = 0.0;       // largest residual norm before the last update of an accepted matrix
  int* dTcErr_ = nullptr;
  long long fallbacks_ = 0;
  double last_rnorm_max_ = 0.0;
  // Newton-Schulz policy of the mixed form (negf_set_refinement); <= 0 restores a default
  int set_refinement(int max_steps, double tol, double accept);
  int invert(double2* A, long long sA, int batch, int* status_dev);
  // FP32 Gauss-Jordan form per batch (rounded up to a power of two): 0 three launches per
  // panel, 1 fused; chosen by timing both on the first inverse of that batch size
  std::map<int, int> gj_form_;
  int invert_f32(int batch);
  int invert_impl(double2* A, long long sA, int batch, int* status_dev);
  int solve_sr_impl(const std::vector<SrJob>& jobs, std::vector<int>& status, std::vector<int>& iters);
  int solve_rgf_impl(const std::vector<Item>& items, bool keep_columns);
  int densities_impl(const std::vector<Item>& items, std::vector<double>& edens, std::vector<double>& hdens);
  HopBD hop() const {
    HopBD h;
    h.hb = dHopBD_;
    h.norb = p_.norb;
    h.nsite = nsite_;
    return h;
  }

  // per-energy API state
  bool sr_valid_ = false, rgf_valid_ = false, dens_valid_ = false;
  double cur_energy_ = 0.0;
  std::array<double, 2> cur_dos_{};
  int cur_sr_status_ = 0;
  int cur_sr_iters_ = 0;
  int cur_rgf_status_ = 0;
  std::vector<double> last_site_;  // nf_ * nsite_total for item 0
  double last_edens_ = 0.0, last_hdens_ = 0.0;
  bool keep_columns_ = false;

 private:
  int configure(const negf_params& p);   // validation and derived sizes, no CUDA calls
  bool dry_ = false;                      // alloc() counts bytes without allocating
  cudaMemPool_t pool_ = nullptr;          // the library's stream-ordered pool on p_.device
  int alloc();
  // Y = op(H) X (left) or X op(H) (right) for every block of a strided batch
  int hop_mul(int left, Op op, const double2* X, long long sX, double2* Y, long long sY, int batch);
  int gemm(int batch, Op opA, const double2* A, long long sA, Op opB, const double2* B, long long sB, double2* C,
           long long sC, double2 alpha, double2 beta);
  int gemm_tc_nn(int batch, const double2* A, long long sA, const double2* B, long long sB, double2* C, long long sC,
                 double2 alpha, double2 beta, int slices);
  int gemm_gamma(int batch, const double2* A, long long sA, const double2* G, const SlicedOperand& sg, double2* C,
                 long long sC);
  int merge_info(int batch);
  // upload HopX (M x M) and its site-block form; a changed HopX invalidates every slot
  int set_hopx(const double2* hx);
};

int merge_info_kernel_launch(int batch, const int* info, int* status, cudaStream_t st);
// release the unused blocks of the library's memory pool on `device` to the device
int pool_trim(int device);

}  // namespace negf
