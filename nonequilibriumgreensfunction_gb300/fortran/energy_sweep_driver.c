/*
 * energy_sweep_driver.c - a C caller that makes the calls Energy_Sweep makes
 * (Source/Energy_Sweep.F90:7-46) through the C ABI, the way the Fortran shim does, on
 * arrays in the reference's column-major layout read from raw files.
 *
 *   energy_sweep_driver <npx> <npy> <npz> <htotd.bin> <hopx.bin> <eta> <sr_tol>
 *                       <mu1> <mu2> <n_e> <e_min> <e_max> <out.bin>
 *
 * htotd.bin / hopx.bin: complex128 Htotd(M,M,npx) and HopX(M,M), column-major.
 * Energies: n_e uniform points in [e_min, e_max]; T = 0 steps f_c = [E <= mu_c]
 * (Energy_Sweep.F90:11-21); dE from the energy spacing (Energy_Sweep.F90:7-9).
 * out.bin: per energy (T12, EDensity, HDensity, Modec1, Modec2, DOSc1, DOSc2) followed by
 * the energy-integrated RhoN and RhoP (npx*npy*npz each), ContactCurrent[2] and the bond
 * currents Jx, Jy, Jz (npx*npy*npz each, Calculate_Observables.F90:110-169).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "negf.h"

static double* read_file(const char* path, size_t n_doubles) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  double* buf = (double*)malloc(n_doubles * sizeof(double));
  size_t got = buf ? fread(buf, sizeof(double), n_doubles, f) : 0;
  fclose(f);
  if (got != n_doubles) { free(buf); return NULL; }
  return buf;
}

int main(int argc, char** argv) {
  if (argc != 14) {
    fprintf(stderr, "usage: %s npx npy npz htotd.bin hopx.bin eta sr_tol mu1 mu2 n_e e_min e_max out.bin\n", argv[0]);
    return 2;
  }
  negf_params p;
  memset(&p, 0, sizeof(p));
  p.npx = atoi(argv[1]); p.npy = atoi(argv[2]); p.npz = atoi(argv[3]); p.norb = 4;
  p.n_hamiltonians = 1; p.max_batch = 1;
  p.eta = atof(argv[6]); p.sr_tol = atof(argv[7]); p.sr_max_iter = 20000;
  p.precision = NEGF_PREC_FP64;
  p.calc_currents = 1;
  const double mu1 = atof(argv[8]), mu2 = atof(argv[9]);
  const int n_e = atoi(argv[10]);
  const double e_min = atof(argv[11]), e_max = atof(argv[12]);
  const size_t M = (size_t)p.norb * p.npy * p.npz;
  const size_t nsites = (size_t)p.npx * p.npy * p.npz;
  double* htotd = read_file(argv[4], 2 * M * M * p.npx);
  double* hopx = read_file(argv[5], 2 * M * M);
  if (!htotd || !hopx) { fprintf(stderr, "cannot read inputs\n"); return 2; }

  negf_handle* h = NULL;
  int st = negf_create(&p, &h);
  if (st) { fprintf(stderr, "negf_create: %s\n", negf_strerror(st)); return 1; }
  st = negf_set_hamiltonian(h, 0, htotd, hopx);
  if (st) { fprintf(stderr, "negf_set_hamiltonian: %s\n", negf_strerror(st)); return 1; }

  const size_t n_out = 7 * (size_t)n_e + 5 * nsites + 2;
  double* out = (double*)calloc(n_out, sizeof(double));
  double* rhon = out + 7 * (size_t)n_e;
  double* rhop = rhon + nsites;
  double* cc = rhop + nsites;
  double* jx = cc + 2;
  double* jy = jx + nsites;
  double* jz = jy + nsites;
  const double de0 = n_e > 1 ? (e_max - e_min) / (n_e - 1) : 0.0;
  double dE = de0;
  int failures = 0;
  for (int k = 0; k < n_e; ++k) {
    const double energy = e_min + de0 * k;
    if (k != n_e - 1) dE = (e_min + de0 * (k + 1)) - energy;    /* Energy_Sweep.F90:7-9 */
    const double f1 = energy <= mu1 ? 1.0 : 0.0, f2 = energy <= mu2 ? 1.0 : 0.0;
    double dosc[2], t12, ed, hd, modes[2];
    st = negf_contact_self_energy(h, energy, NULL, NULL, NULL, NULL, dosc);
    if (st) { fprintf(stderr, "E=%g Contact_Self_Energy: %s\n", energy, negf_strerror(st)); ++failures; }
    st = negf_get_retarded_greens(h);
    if (st) { fprintf(stderr, "E=%g Get_Retarded_Greens: %s\n", energy, negf_strerror(st)); ++failures; }
    st = negf_calculate_gnp(h, f1, f2, dE, rhon, rhop);
    if (st) { fprintf(stderr, "E=%g Calculate_Gnp: %s\n", energy, negf_strerror(st)); ++failures; }
    st = negf_calculate_observables(h, dE, f1, f2, &t12, &ed, &hd, modes, cc, NULL, NULL, NULL);
    if (st) { fprintf(stderr, "E=%g Calculate_Observables: %s\n", energy, negf_strerror(st)); ++failures; }
    st = negf_calculate_currents(h, jx, jy, jz);
    if (st) { fprintf(stderr, "E=%g bond currents: %s\n", energy, negf_strerror(st)); ++failures; }
    double* o = out + 7 * (size_t)k;
    o[0] = t12; o[1] = ed; o[2] = hd; o[3] = modes[0]; o[4] = modes[1]; o[5] = dosc[0]; o[6] = dosc[1];
  }
  FILE* f = fopen(argv[13], "wb");
  if (!f) return 2;
  fwrite(out, sizeof(double), n_out, f);
  fclose(f);
  negf_destroy(h);
  free(out); free(htotd); free(hopx);
  return failures ? 1 : 0;
}
