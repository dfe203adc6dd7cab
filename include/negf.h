/*
 * negf.h - C ABI of libnegf_gb300.so, the GB300 (sm_103a) implementation of the
 * per-energy NEGF solve of brian-dellabetta/nonEquilibriumGreensFunction.
 *
 * The reference's hot path is four argument-less Fortran subroutines that read and
 * write NEGF_Module globals, called once per energy point by Energy_Sweep
 * (Source/Energy_Sweep.F90:28,40,42,45).  This header replaces them with calls that
 * take the same data explicitly: plain pointers to the caller's column-major arrays,
 * sizes, and an opaque handle that owns every device buffer.
 *
 * Conventions
 *  - Complex arrays are interleaved (re, im) doubles, i.e. the memory layout of Fortran
 *    COMPLEX(8) / C double _Complex.  A "block" is an M x M column-major complex
 *    matrix, M = norb*npy*npz (NNz in Source/Read_In_Allocate.F90:96-97).
 *  - Htotd is M x M x npx (Source/NEGF_Module.F90:56), HopX is M x M (:57) and is the
 *    coupling H(x, x+1); H(x+1, x) = HopX^H (Source/Recursive_Greens.F90:6).
 *  - Site arrays (RhoN, RhoP, SigXExp, ...) are npx x npy x npz, column-major
 *    (x fastest), as Source/NEGF_Module.F90:51-52.  In-slice orbital index is
 *    orb + y*norb + z*norb*npy (Source/Calculate_Gnp.F90:122).
 *  - Every entry point returns int: 0 = success; > 0 = LAPACK-style INFO (1-based
 *    index of the first exactly-zero pivot of an inverse, as ZGETRF/ZGETRI report it
 *    through Invert_Matrix, Source/MKL_Routines_Cluster.F90:17-28); < 0 = NEGF_E*.
 *    No entry point aborts, exits or traps.
 *  - A handle is used by one host thread at a time; separate handles are independent.
 *  - There is no CPU fallback: if no CUDA device is present, negf_create returns
 *    NEGF_ENODEV.
 */
#ifndef NEGF_GB300_H
#define NEGF_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define NEGF_API __attribute__((visibility("default")))
#else
#define NEGF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define NEGF_OK            0
#define NEGF_EINVAL       (-1)   /* bad argument or size                                 */
#define NEGF_ENOMEM       (-2)   /* device allocation failed                             */
#define NEGF_ECUDA        (-3)   /* a CUDA runtime call failed                           */
#define NEGF_ESR_NOCONV   (-4)   /* Sancho-Rubio hit sr_max_iter (Contact_Self_Energy.F90:202-205) */
#define NEGF_ENAN         (-5)   /* NaN in the Sancho-Rubio update (Contact_Self_Energy.F90:182-191) */
#define NEGF_ESTATE       (-6)   /* call order violated (e.g. Greens before self-energy) */
#define NEGF_EADMIT       (-7)   /* request larger than the handle's admission budget    */
#define NEGF_ETIMEDOUT    (-8)   /* bounded device wait ran out                          */
#define NEGF_EREFINE      (-9)   /* mixed form: refinement residual above bound          */
#define NEGF_ENODEV      (-10)   /* no CUDA device                                       */
#define NEGF_ENOHAM      (-11)   /* Hamiltonian slot never set                           */
#define NEGF_ESCRATCH    (-12)   /* negf_zgemm_noalloc: sizes exceed its static scratch  */

/* ---- arithmetic form ------------------------------------------------------------- */
#define NEGF_PREC_FP64     0     /* plain FP64 complex throughout                        */
#define NEGF_PREC_MIXED    1     /* tcgen05 BF16 sliced products, FP64 refinement        */

typedef struct negf_params {
    int32_t npx, npy, npz;   /* lattice (Source/NEGF_Module.F90:27)                      */
    int32_t norb;            /* orbitals per site (<= 8); 4 for the TI models, 8 for their
                                BdG form with superconducting contacts                  */
    int32_t n_hamiltonians;  /* Htotd slots held on the device (e.g. disorder seeds)     */
    int32_t max_batch;       /* energy points solved together by negf_solve_batch        */
    double  eta;             /* eta_sigma, Source/Constants.F90:7 (reference 1e-4)       */
    double  sr_tol;          /* Sancho-Rubio stop: max|change| <= sr_tol (ref. 1e-8)      */
    int32_t sr_max_iter;     /* Sancho-Rubio iteration cap (reference 20000)             */
    int32_t calc_spin;       /* calcSigExp, Source/Read_In_Allocate.F90:93               */
    int32_t precision;       /* NEGF_PREC_*                                              */
    int32_t device;          /* CUDA device ordinal                                      */
    int32_t mixed_slices;    /* NEGF_PREC_MIXED: BF16 slices per operand (0 = default)   */
    int32_t keep_g_columns;  /* 1: keep G(:,1), G(:,N) of the per-energy call for
                                negf_copy_g_columns (2*Npx*M^2*16 extra device bytes)    */
    int32_t residual_slices; /* NEGF_PREC_MIXED: slices of the Newton-Schulz residual W X
                                (0 = default 7; 5..8 allowed)                            */
    int32_t sr_slices;       /* NEGF_PREC_MIXED: slices of the Sancho-Rubio products
                                (0 = default 8; 5..8 allowed)                            */
    int32_t calc_currents;   /* 1: bond currents Jx/Jy/Jz (Source/Calculate_Observables.F90:
                                110-169); keeps the +x/+y/+z site blocks of Gn/Gp
                                (6*npx*M*norb*16 bytes per batch entry)                  */
    int32_t reserved[3];     /* must be zero                                             */
    double  spin_ops[3][4][4][2]; /* gMx, gMy, gMz (row-major [row][col][re,im]) used by
                                     the spin reduction, Source/Read_In_Allocate.F90:183-196;
                                     all zero = the reference's own for the nh electron
                                     orbitals: tau0 (x) sigma_j (nh = 4), the Pauli
                                     matrices (nh = 2, :205-216), zero (nh = 1)           */
    /* Contacts (contactType, Source/Read_In_Allocate.F90:19, Contact_Self_Energy.F90:19-92):
     *   NEGF_CONTACT_LEADS   semi-infinite leads, Sancho-Rubio decimation (default);
     *   NEGF_CONTACT_PBIG    phenomenological: Sigma = -i rate on every orbital of the end
     *                        slice (:19-23);
     *   NEGF_CONTACT_PSMALL  the same on the first npy*norb orbitals only (:24-28);
     *   NEGF_CONTACT_SC      superconducting contacts (:29-67) on a BdG Hamiltonian: norb =
     *                        2 nh, each site block holds the nh electron orbitals first and
     *                        their holes after them (Read_In_Allocate.F90:69-71,
     *                        Build_Hamiltonian.F90:52-56).  T12 is then the supercurrent
     *                        transmission of Calculate_Observables.F90:60-81, and EDensity,
     *                        HDensity, spin and bond currents run over the electron orbitals
     *                        (:14-15, :37-39, :114-115).                                  */
    int32_t contact_type;
    int32_t reserved1;       /* must be zero                                             */
    double  tunneling_rate;  /* phenomenological and SC contacts (Contact_Self_Energy.F90:10);
                                0 = the reference's 1                                    */
    double  delta_sc[2];     /* DeltaSCL, DeltaSCR in eV (Read_In_Allocate.F90:74-75)    */
    double  chi_lr;          /* Josephson phase of the left contact (Read_In_Allocate.F90:72) */
    double  gds[4][4][2];    /* gDS, the nh x nh pairing structure of the SC contacts
                                (Read_In_Allocate.F90:199-202, 214-215), row-major; all zero
                                = the four-orbital models' gDS                           */
    int32_t reserved2[8];    /* must be zero                                             */
} negf_params;

#define NEGF_CONTACT_LEADS   0
#define NEGF_CONTACT_PBIG    1
#define NEGF_CONTACT_PSMALL  2
#define NEGF_CONTACT_SC      3

typedef struct negf_handle negf_handle;

/* ---- lifetime -------------------------------------------------------------------- */
NEGF_API int  negf_create(const negf_params* p, negf_handle** out);
NEGF_API int  negf_destroy(negf_handle* h);
NEGF_API const char* negf_strerror(int code);
/* bytes of device memory the handle holds (for admission / reporting) */
NEGF_API int  negf_device_bytes(const negf_handle* h, int64_t* bytes);
/* bytes of device memory negf_create would allocate for these parameters, computed on the
 * host without a device (the admission unit of the serving layer: the Npx*M^2*16-byte
 * block store per batch entry plus the Hamiltonian slots and work buffers).  No reference
 * counterpart: the reference allocates its arrays per rank at start-up
 * (Source/Read_In_Allocate.F90:104-238).  NEGF_EINVAL for parameters negf_create refuses. */
NEGF_API int  negf_estimate_device_bytes(const negf_params* p, int64_t* bytes);

/* Run the handle's work on a caller-owned CUDA stream (cudaStream_t passed as void*);
 * NULL restores the handle's own stream.  Calls still return only after their results
 * are on the host.                                                                     */
NEGF_API int negf_set_stream(negf_handle* h, void* stream);

/* Instrumentation: launch counts and CUDA-event timings of the dense kernels.  Enabling
 * resets the counters; timing adds one event pair per timed launch.                    */
typedef struct negf_stats {
    int64_t launches;        /* kernels launched by the library since the last reset       */
    int64_t gemm_launches;   /* complex GEMM launches (also those inside the inverses)     */
    double  gemm_ms;         /* summed device time of those launches (profiling on)        */
    double  gemm_flops;      /* their real flops, 8*m*n*k per complex GEMM                 */
    int64_t panel_launches;  /* Gauss-Jordan panel factorisations                          */
    double  panel_ms;
    int64_t tc_launches;     /* tcgen05 sliced-BF16 GEMM launches (mixed form)             */
    double  tc_ms;
    double  tc_flops;        /* BF16 tensor flops issued: S(S+1)/2 slice pairs x 8*m*n*k   */
    double  tc_complex_flops;/* the complex products they compute, 8*m*n*k                 */
    int64_t fallbacks;       /* mixed form: inverses redone in FP64 (residual too large)   */
    double  ns_residual_max; /* mixed form: largest accepted first Newton-Schulz residual  */
    double  f32_gemm_ms;     /* FP32 Gauss-Jordan rank-nb updates (mixed form)             */
    double  slice_ms;        /* operand slicing kernels (mixed form)                       */
    double  phase_sr_ms;     /* whole Sancho-Rubio phases                                  */
    double  phase_rgf_ms;    /* whole RGF sweeps (including their inverses)                */
    double  phase_inv_ms;    /* all inverses (Sancho-Rubio and RGF)                        */
    double  phase_dens_ms;   /* density / spin reductions                                  */
    int64_t ns_extra_steps;  /* mixed form: Newton-Schulz matrix-steps beyond the two fixed
                                ones (matrices whose residual was still above ns_tol)      */
    int64_t ns_unconverged;  /* mixed form: matrices still above ns_tol after ns_max_steps
                                steps; each was inverted again in FP64 (also counted in
                                fallbacks)                                                  */
    double  ns_final_residual_max; /* mixed form: largest residual norm before the last
                                update among the accepted inverses (<= ns_tol; the last
                                update squares it)                                          */
} negf_stats;
NEGF_API int negf_profile(negf_handle* h, int enable);
NEGF_API int negf_get_stats(negf_handle* h, negf_stats* out);

/* Newton-Schulz policy of the mixed form's inverses (no reference counterpart: the
 * reference's Invert_Matrix, Source/MKL_Routines_Cluster.F90:2-33, is a direct LU; its
 * errorFlag contract is kept by redoing in FP64 any inverse this policy cannot certify).
 * Each block is inverted in FP32 and refined by X <- X + X (I - W X); two steps always,
 * more (up to ns_max_steps in all, 2..16) while the row-sum norm of I - W X before the
 * latest update is above ns_tol.  A block is inverted again in FP64 when its first
 * residual norm is above ns_accept (< 1), its FP32 factorisation met a zero pivot, or it
 * is still above ns_tol after ns_max_steps steps.  Values <= 0 select the defaults
 * (4, 1e-5, 0.5).  NEGF_ESTATE on an FP64 handle.                                      */
NEGF_API int negf_set_refinement(negf_handle* h, int32_t ns_max_steps, double ns_tol, double ns_accept);

/* ---- Hamiltonian upload ------------------------------------------------------------
 * Replaces the broadcast of Build_Hamiltonian's output to the solvers
 * (Source/MPI_Routines.F90:19-30).  Htotd: M x M x npx complex, HopX: M x M complex.
 * HopX is shared by all slots: the call with slot 0 sets it, other slots must pass the
 * same HopX (or NULL).  Detects whether HopX is block diagonal in norb x norb site
 * blocks (true for every channel of Source/Build_Hamiltonian.F90:59-64) and then
 * applies it as a site-local operator instead of a dense product.                     */
NEGF_API int negf_set_hamiltonian(negf_handle* h, int32_t slot, const double* Htotd, const double* HopX);

/* ---- on-device Hamiltonian ----------------------------------------------------------
 * Build_Hamiltonian (Source/Build_Hamiltonian.F90:1-303, open boundaries) on the device:
 * the slot's Htotd is generated in HBM from norb x norb site blocks instead of being
 * copied from the host (npx*M^2*16 bytes, 256 MB at M = 400, npx = 100).  Every slice holds
 * the on-site block on each site, hop_y between (y, z) and (y+1, z) times the Landau-gauge
 * phase exp(i 2 pi z flux / ((npy-1)(npz-1))) (:186-207), hop_z between (y, z) and (y, z+1),
 * their Hermitian conjugates below the diagonal, and the potential V(x, y, z) on the
 * diagonal.  HopX is hop_x on every site (:59-64).  V is the caller's array (an
 * electrostatic potential, :104-112; NULL = 0) plus Anderson disorder U[-W/2, W/2) on
 * slices 2..npx-1 only (:279-296) from a counter-based stream: (u - 1/2) W with
 * u = (s >> 11) 2^-53 and s the i-th output of SplitMix64 seeded with `seed` (Steele, Lea,
 * Flood 2014), i = x + npx (y + npy z) + 1; the site's potential is V + that.  The
 * reference's RANDOM_NUMBER stream is compiler-specific (:230-241); this one is
 * reproducible bit for bit on any host.  The blocks are norb x norb, norb <= 4 (the
 * channel models of :13-47: the TI and Bi2Se3 wires 4, the one-band metal 1, the TI
 * surface and the 1-D spin-orbit wire 2), in the leading rows and columns of the 4 x 4
 * arrays, whose other entries must be zero; not with superconducting contacts (a BdG
 * Hamiltonian).  HopX is shared by all slots, as in negf_set_hamiltonian.               */
typedef struct negf_wire_model {
    double   onsite[4][4][2];  /* row-major [row][col][re, im]                           */
    double   hop[3][4][4][2];  /* hop_x, hop_y, hop_z = H(site, site + e_j)              */
    double   flux;             /* Aharonov-Bohm flux through the cross-section, Phi_0    */
    double   W;                /* disorder width (0 = no disorder)                       */
    uint64_t seed;             /* disorder stream                                        */
    const double* V;           /* optional npx x npy x npz potential, column-major       */
    int32_t  reserved[8];      /* must be zero                                           */
} negf_wire_model;
NEGF_API int negf_build_hamiltonian(negf_handle* h, int32_t slot, const negf_wire_model* model);
/* ---- per-energy interface (one energy point, Hamiltonian slot 0) ---------------------
 * The four calls below are the drop-in for the reference's subroutines, in the order
 * Energy_Sweep makes them.  All device results stay in the handle between calls.       */

/* Contact_Self_Energy (Source/Contact_Self_Energy.F90:1-106, contactType 0):
 * Sancho-Rubio decimation of both semi-infinite leads at `energy`.  Writes SigmaL,
 * SigmaR, GammaL, GammaR (M x M complex, any may be NULL) and dosc[2] = (DOSc1, DOSc2)
 * increments (:94-97).  Returns NEGF_ESR_NOCONV / NEGF_ENAN as errorFlag would be set. */
NEGF_API int negf_contact_self_energy(negf_handle* h, double energy,
                             double* SigmaL, double* SigmaR, double* GammaL, double* GammaR,
                             double* dosc);

/* Get_Retarded_Greens (Source/Recursive_Greens.F90:2-107) for the InvGRd that
 * Energy_Sweep.F90:31-38 assembles from Htotd, energy, eta and the self-energies of the
 * last negf_contact_self_energy call.  Results (the first and last block columns of G)
 * stay on the device.  Returns the INFO of the first singular inverse, if any.          */
NEGF_API int negf_get_retarded_greens(negf_handle* h);

/* Optional copy-out of GRLef = G(:,1) and GRRgt = G(:,N) (Ntot x M complex each,
 * Source/NEGF_Module.F90:70); either may be NULL.  Debug/parity use only.              */
NEGF_API int negf_copy_g_columns(negf_handle* h, double* GRLef, double* GRRgt);

/* Calculate_Gnp (Source/Calculate_Gnp.F90:1-136): Gn = f1 G1 GammaL G1^H + f2 GN GammaR GN^H,
 * Gp with (1-f), and the site densities RhoN/RhoP += Re diag * dE/(2 pi) (:117-124),
 * accumulated into the caller's npx x npy x npz arrays.                                 */
NEGF_API int negf_calculate_gnp(negf_handle* h, double f1, double f2, double dE,
                       double* RhoN, double* RhoP);

/* Calculate_Observables (Source/Calculate_Observables.F90:2-108, non-BdG branch):
 * writes T12, EDensity, HDensity, modes[2] = (Modec1, Modec2) for this energy, adds the
 * ContactCurrent increments to contact_current[2], and, if the handle has calc_spin and
 * the pointers are non-NULL, accumulates SigXExp/SigYExp/SigZExp (npx x npy x npz).      */
NEGF_API int negf_calculate_observables(negf_handle* h, double dE, double f1, double f2,
                               double* T12, double* EDensity, double* HDensity,
                               double* modes, double* contact_current,
                               double* SigX, double* SigY, double* SigZ);

/* Bond currents of Calculate_Observables (Source/Calculate_Observables.F90:110-169) for the
 * energy of the last negf_calculate_gnp call (its f1, f2, dE): adds the dE/(2 pi)-weighted
 * currents of every bond leaving site (x, y, z) towards +x, +y, +z into Jx, Jy, Jz
 * (npx x npy x npz, any may be NULL).  Each orbital-pair term is rounded to REAL(4) before
 * it is weighted and added, as the reference's dumVar (:7).  The x bonds use the site
 * blocks of HopX (:150-156).  NEGF_ESTATE unless the handle was created with
 * calc_currents = 1 and negf_calculate_gnp ran for this energy.                         */
NEGF_API int negf_calculate_currents(negf_handle* h, double* Jx, double* Jy, double* Jz);

/* Energy- and orbital-resolved current densities of Calculate_Observables (erCD/orCD,
 * Source/Calculate_Observables.F90:124-160, Source/Calculate_Gnp.F90:125-129) for the
 * energy of the last negf_calculate_gnp call; any pointer may be NULL, values are added.
 * ERJx/ERJy/ERJz/ERRhon: npx x npy x npz, the caller's column eCtr+1, unweighted
 * (ERRhon = sum over orbitals of Re Gn(i,i) - Re Gp(i,i)).  ORJx/ORJy/ORJz: npx x npy x
 * npz x norb^2 (pair ii*norb + jj), ORRhon: npx x npy x npz x norb, dE/(2 pi)-weighted.
 * NEGF_ESTATE unless the handle has calc_currents = 1 and negf_calculate_gnp ran.       */
NEGF_API int negf_calculate_resolved(negf_handle* h, double* ERJx, double* ERJy, double* ERJz, double* ERRhon,
                                     double* ORJx, double* ORJy, double* ORJz, double* ORRhon);
/* ---- batched interface -------------------------------------------------------------
 * Many energy points (and Hamiltonian slots, e.g. disorder seeds) in one device pass:
 * the GB300 replacement for the round-robin energy loop of Source/NEGF_Main.F90:21-27
 * plus the MPI sums of Source/MPI_Routines.F90:33-90.  n may exceed max_batch; requests
 * are processed in chunks of max_batch in order.                                       */
typedef struct negf_request {
    double  energy;
    double  f1, f2;          /* lead occupations at this energy (Energy_Sweep.F90:11-23) */
    double  dE;              /* quadrature weight (Energy_Sweep.F90:7-9)                 */
    int32_t slot;            /* Hamiltonian slot                                         */
    int32_t flags;           /* reserved, 0                                              */
} negf_request;

typedef struct negf_result {
    double  T12;             /* Calculate_Observables.F90:85-100                         */
    double  EDensity, HDensity;
    double  modes[2];
    double  dosc[2];
    int32_t status;          /* per-request status (NEGF_OK, INFO > 0, NEGF_E*)          */
    int32_t sr_iters;        /* Sancho-Rubio iterations taken                           */
} negf_result;

/* RhoN, RhoP, SigX/Y/Z (may be NULL) are npx x npy x npz x n_hamiltonians arrays
 * (slot slowest) that the requests' dE-weighted densities are ADDED to.  The call
 * returns < 0 only for call-level failures (arguments, CUDA); the outcome of each
 * request (INFO > 0, NEGF_ESR_NOCONV, NEGF_ENAN) is in res[i].status, and the batch
 * continues past failed requests as the reference's energy loop does.                  */
NEGF_API int negf_solve_batch(negf_handle* h, const negf_request* req, int32_t n, negf_result* res,
                     double* RhoN, double* RhoP, double* SigX, double* SigY, double* SigZ);

/* negf_solve_batch with every accumulated site array of the reference: RhoN, RhoP
 * (Calculate_Gnp), SigX/Y/Z (calc_spin) and Jx/Jy/Jz (calc_currents), each
 * npx x npy x npz x n_hamiltonians or NULL, summed over requests as
 * Source/MPI_Routines.F90:33-90 sums them over ranks.                                   */
typedef struct negf_batch_outputs {
    double* RhoN; double* RhoP;
    double* SigX; double* SigY; double* SigZ;
    double* Jx;   double* Jy;   double* Jz;
    /* energy-resolved arrays (erCD, Source/Calculate_Observables.F90:124-157,
     * Source/Calculate_Gnp.F90:125-127): npx x npy x npz x n, column n-1 for request n-1,
     * UNweighted as the reference's ERJx(:,:,:,eCtr+1): the bond sums of dumVar and
     * ERRhon = sum over orbitals of Re Gn(i,i) - Re Gp(i,i).  Need calc_currents.         */
    double* ERJx; double* ERJy; double* ERJz; double* ERRhon;
    /* orbital-resolved arrays (orCD, :127-160 and Calculate_Gnp.F90:128-129), summed over
     * requests with the dE/(2 pi) weight: ORJx/y/z are npx x npy x npz x norb^2 x
     * n_hamiltonians (pair index ii*norb + jj, ii on the bond's first site), ORRhon is
     * npx x npy x npz x norb x n_hamiltonians.  Need calc_currents.                        */
    double* ORJx; double* ORJy; double* ORJz; double* ORRhon;
    double* reserved[8];     /* must be NULL                                             */
} negf_batch_outputs;
NEGF_API int negf_solve_batch_ex(negf_handle* h, const negf_request* req, int32_t n, negf_result* res,
                                 const negf_batch_outputs* out);
/* ---- serving ----------------------------------------------------------------------
 * A request server in place of the MPI energy sweep, with every request's state (its
 * Hamiltonian, block store and results) kept on the device: wires of different
 * cross-sections arrive as requests (Hamiltonian + a list of energy points with their
 * occupations), are admitted while the HBM budget has room for their geometry's block
 * store (Npx*M^2*16 bytes per in-flight energy point) and a free Hamiltonian slot, and
 * their energy points are packed, with those of every other admitted request of the same
 * geometry, into the next device batch (continuous batching).  Each geometry is served by
 * its own worker thread and CUDA stream, so work of different geometries overlaps on the
 * device.  A request's results do not depend on what it was batched with.               */
typedef struct negf_server negf_server;

typedef struct negf_serve_params {
    int32_t device;
    int32_t precision;        /* NEGF_PREC_*                                                 */
    int32_t mixed_slices;     /* as in negf_params                                           */
    int32_t max_batch;        /* energy points per device batch, per geometry                */
    int32_t slots_per_geometry; /* Hamiltonians resident per geometry                       */
    int32_t calc_spin;
    double  eta, sr_tol;
    int32_t sr_max_iter;
    int32_t reserved0;
    int64_t hbm_budget_bytes; /* device memory the server may hold (0 = 80% of free)         */
    int32_t reserved[8];
} negf_serve_params;

typedef struct negf_wire_request {
    int32_t npx, npy, npz, norb;
    const double* Htotd;      /* M x M x npx complex, copied at submit (NULL with `model`)   */
    const double* HopX;       /* M x M complex, copied at submit (NULL with `model`)         */
    int32_t n_energies;
    int32_t reserved0;
    const double* energies;   /* n_energies each, copied at submit                           */
    const double* f1;
    const double* f2;
    const double* dE;
    const negf_wire_model* model; /* instead of Htotd/HopX: the wire is generated on the
                                 device by negf_build_hamiltonian (norb = 4); the model and
                                 its V array are copied at submit                          */
} negf_wire_request;

typedef struct negf_wire_status {
    int32_t done;             /* 1 when every energy point is solved                         */
    int32_t status;           /* first non-zero per-energy status                            */
    int32_t n_done;           /* energy points solved so far                                 */
    int32_t reserved0;
    double  t_submit, t_admit, t_done;   /* seconds on the server's monotonic clock         */
} negf_wire_status;

NEGF_API int negf_server_create(const negf_serve_params* p, negf_server** out);
NEGF_API int negf_server_submit(negf_server* s, const negf_wire_request* r, int64_t* id);
/* status only (results NULL) or, once done, copy out: per energy T12/EDensity/HDensity/
 * Modec1/Modec2/DOSc1/DOSc2 into res7[7*n_energies] and RhoN/RhoP (npx*npy*npz each,
 * dE-weighted sums) into rho[2*npx*npy*npz]; a finished request is released by the
 * call that copies its results out (release != 0).                                      */
NEGF_API int negf_server_poll(negf_server* s, int64_t id, negf_wire_status* st, double* res7, double* rho,
                              int32_t release);
/* block until request `id` is done or timeout_s elapses (NEGF_ETIMEDOUT)               */
NEGF_API int negf_server_wait(negf_server* s, int64_t id, double timeout_s);
NEGF_API double negf_server_clock(const negf_server* s);
/* Engine churn of the server (no reference counterpart): each geometry's engine is
 * created on its first admitted request and released when memory is needed elsewhere. */
typedef struct negf_server_stats {
    int64_t engines_created, engines_released, engines_live;
    double  create_s;         /* host seconds spent creating engines (device allocation)   */
    double  release_s;        /* host seconds spent releasing them (device frees)          */
    int64_t bytes_used, bytes_budget;
    int64_t reserved[4];
} negf_server_stats;
NEGF_API int negf_server_get_stats(negf_server* s, negf_server_stats* out);
NEGF_API int negf_server_destroy(negf_server* s);

/* ---- self-consistent bias point: Poisson ---------------------------------------------
 * The electrostatic step of the Poisson <-> NEGF loop (Solve_Equilibrium / SIP_V1,
 * Source/SIP_Solver.F90:1-201, called from Source/NEGF_Main.F90:10-12), on the current
 * CUDA device.  For each of n_grids site grids (npx x npy x npz, column-major, grids
 * consecutive) it solves for the electron potential energy U (eV)
 *     6 U_i - sum_{in-grid neighbours j} U_j = kappa rho_i + sum of the boundary values
 *                                              of i's neighbours outside the grid,
 * a 7-point Laplacian with uniform eps_r (kappa = q / (eps0 eps_r a)) and Dirichlet values
 * bc[0] on the plane x = -1 (left contact), bc[1] on x = npx (right contact) and bc[2] on
 * every y and z face (the gate).  rho = RhoN - RhoP per site.  U holds the initial guess
 * and receives the solution.  The reference iterates Stone's strongly implicit procedure;
 * this solves the same symmetric positive definite system by conjugate gradients, one CTA
 * per grid, until ||b - A U|| <= tol ||b||.  *iters (may be NULL) receives the largest
 * iteration count; NEGF_EREFINE if a grid did not reach tol within max_iter, NEGF_ENAN if
 * rho is not finite.                                                                    */
NEGF_API int negf_poisson_solve(int32_t npx, int32_t npy, int32_t npz, int32_t n_grids, const double* rho,
                                const double* bc, double kappa, double* U, double tol, int32_t max_iter,
                                int32_t* iters);
/* ---- stateless dense kernels -------------------------------------------------------
 * Drop-ins for the reference's dense calls on host arrays (column-major, interleaved
 * complex), run on the current CUDA device; `batch` matrices are consecutive in memory
 * (A at stride lda*k, B at ldb*n, C at ldc*n, G at n*n).                               */

/* zgemm('N','N', m, n, k, alpha, A, lda, B, ldb, beta, C, ldc) as called throughout
 * Source/Recursive_Greens.F90 and Source/Contact_Self_Energy.F90.  slices = 0 runs the
 * FP64 DFMA kernel; slices in 3..8 runs the tcgen05 tensor-core kernel on exact
 * 7-bit integer BF16 slices of row/column-scaled operands (truncation <= 2^(-7*slices)
 * of max|A_i.| max|B_.j| per term; 7-8 slices is FP64-class).  NEGF_ETIMEDOUT if a
 * bounded device wait expired.                                                          */
NEGF_API int negf_zgemm(int32_t slices, int32_t m, int32_t n, int32_t k, const double* alpha,
                        const double* A, int32_t lda, const double* B, int32_t ldb,
                        const double* beta, double* C, int32_t ldc, int32_t batch);

/* Invert_Matrix(invG, G, N, errorFlag) (Source/MKL_Routines_Cluster.F90:2-33): returns
 * the LAPACK INFO of the first singular matrix, 0 if all are invertible.               */
NEGF_API int negf_zinv(int32_t n, const double* G, double* invG, int32_t batch);

/* negf_zgemm_noalloc: no counterpart in the reference.  The tensor-core sliced GEMM of
 * negf_zgemm (C = alpha A B + beta C, one matrix, slices 3..8) on DEVICE arrays, for
 * callers that must not allocate device memory: code whose device memory is owned by
 * another allocator (a framework pool, a serving process with a fixed HBM budget) and
 * latency-critical loops that cannot absorb the device-wide synchronisation of
 * cudaMalloc/cudaFree.  It calls no allocating routine; its scratch is one static device
 * array of NEGF_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit, which limits m, n, k to NEGF_NOALLOC_MAX_DIM (larger sizes: NEGF_ESCRATCH).
 * A GPU holds the array from the first call on it (or from library load, when CUDA loads
 * modules eagerly); that first call looks up the array's device address.  All calls
 * share the scratch: calls that overlap on the GPU race, so the caller must order them.
 * Runs on `stream` (cudaStream_t, NULL = default stream), then reads the device error
 * flag and synchronises `stream`: it returns after the product is complete and cannot be
 * captured into a CUDA graph.  The first beta = 0 call of each shape with 2k <= 800 also
 * times the tensor-core kernel variants: it launches the product nine times and waits for
 * them before returning.                                                               */
#define NEGF_NOALLOC_MAX_DIM      512
#define NEGF_NOALLOC_MAX_SLICES   8
#define NEGF_NOALLOC_SCRATCH_BYTES (26u * 1024u * 1024u)
NEGF_API int negf_zgemm_noalloc(int32_t slices, int32_t m, int32_t n, int32_t k, const double* alpha,
                                const double* A, int32_t lda, const double* B, int32_t ldb,
                                const double* beta, double* C, int32_t ldc, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NEGF_GB300_H */
