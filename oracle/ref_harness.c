/*
 * ref_harness.c -- runs the reference's OWN step code as the oracle (test
 * infrastructure only).  The reference's src/qg.c is compiled in place
 * (never copied) with its main() renamed; this file then drives the
 * reference's own init_* / invert_pv / rhs / timestep functions the way
 * src/qg.c:103-200 does, minus the file output.
 *
 * usage: qgw_ref PARAMS Q_IN OUT_PREFIX NSTEPS [DT_FIXED [MODE [TOPO_IN]]]
 *   Q_IN      raw float64 (nl, ny+2, nx+2) initial q, or "-" for zeros
 *   DT_FIXED  > 0: dt = dt0 = dt1 = DT_max = DT_FIXED and t_out = 0, so
 *             adjust_timestep keeps dt unless the CFL limit is smaller;
 *             0: adaptive dt from check_timestep with the t_out snapping of
 *             the driver loop (src/qg.c:181-199)
 *   MODE      step (default) | rhs (write rhs(q) after NSTEPS steps)
 *   TOPO_IN   raw float64 (ny+2, nx+2) topography replacing init_vars'
 * Writes OUT_PREFIX.psi, .q (raw float64, reference layout, psi = the
 * inversion of the final q), .rhs (MODE rhs), .modes (cl2m, cm2l, iRd2) and
 * .time (text: t dt dt0 dt1 DT_max t_out steps).
 */
#define main qgw_reference_main
#include "qg.c"
#undef main

static int harness_read(const char* path, double* dst, size_t n) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  size_t got = fread(dst, sizeof(double), n, f);
  fclose(f);
  return got == n ? 0 : -1;
}

static int harness_write(const char* prefix, const char* ext, const double* src, size_t n) {
  char path[1024];
  snprintf(path, sizeof path, "%s.%s", prefix, ext);
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  fwrite(src, sizeof(double), n, f);
  fclose(f);
  return 0;
}

int main(int argc, char* argv[]) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s PARAMS Q_IN OUT_PREFIX NSTEPS [DT_FIXED [MODE [TOPO_IN]]]\n", argv[0]);
    return 2;
  }
  const char* mode = argc > 6 ? argv[6] : "step";
  const int nsteps = atoi(argv[4]);
  const double dt_fixed = argc > 5 ? atof(argv[5]) : 0.0;
  print = 0;
  init_mpi();
  /* the parameter table of src/qg.c:113-137 */
  params = list_append(params, &NX, "NX", "int");
  params = list_append(params, &NY, "NY", "int");
  params = list_append(params, &nl, "nl", "int");
  params = list_append(params, &n_hyper, "n_hyper", "int");
  params = list_append(params, &Lx, "Lx", "double");
  params = list_append(params, &dh, "dh", "array");
  params = list_append(params, &tau0, "tau0", "double");
  params = list_append(params, &forc_mode, "forc_mode", "double");
  params = list_append(params, &f0, "f0", "double");
  params = list_append(params, &beta, "beta", "double");
  params = list_append(params, &nu, "nu", "double");
  params = list_append(params, &nu_hyper, "nu_hyper", "double");
  params = list_append(params, &hEkb, "hEkb", "double");
  params = list_append(params, &N2, "N2", "array");
  params = list_append(params, &Ld, "Ld", "double");
  params = list_append(params, &h_topo, "h_topo", "double");
  params = list_append(params, &w_topo, "w_topo", "double");
  params = list_append(params, &bc_fac, "bc_fac", "double");
  params = list_append(params, &tend, "tend", "double");
  params = list_append(params, &dt_out, "dt_out", "double");
  params = list_append(params, &dt_forc, "dt_forc", "double");
  params = list_append(params, &dt_forc_period, "dt_forc_period", "double");
  params = list_append(params, &sigma_f, "sigma_f", "double");
  params = list_append(params, &k_f, "k_f", "double");
  params = list_append(params, &cfl, "cfl", "double");
  read_params(params, argv[1]);

  init_domain();
  init_elliptic();
  init_vars();
  init_timestep();
  init_stoch_forc();
  init_4d_forcing();

  const size_t n3 = (size_t)Nxp2 * Nyp2 * nl, n2 = (size_t)Nxp2 * Nyp2;
  if (strcmp(argv[2], "-") && harness_read(argv[2], q, n3)) {
    fprintf(stderr, "cannot read %s (%zu doubles expected)\n", argv[2], n3);
    return 1;
  }
  if (argc > 7 && harness_read(argv[7], topo, n2)) {
    fprintf(stderr, "cannot read %s\n", argv[7]);
    return 1;
  }
  invert_pv(q, psi);  /* first inversion, src/qg.c:167 */

  int steps = 0;
  if (dt_fixed > 0) {
    dt = dt0 = dt1 = DT_max = dt_fixed;
    t_out = 0;
    for (; steps < nsteps; ++steps) timestep(q);
  } else {
    while (t < tend && steps < nsteps) {  /* src/qg.c:181-199 */
      if (fabs(t - t_out) < TEPS * dt) t_out += dt_out;
      timestep(q);
      ++steps;
    }
  }
  if (!strcmp(mode, "rhs")) {
    rhs(q, f0_ab);
    harness_write(argv[3], "rhs", f0_ab, n3);
  }
  invert_pv(q, psi);
  harness_write(argv[3], "psi", psi, n3);
  harness_write(argv[3], "q", q, n3);
  double modes[3 * 64 * 64];
  size_t nm = 0;
  for (int s = 0; s < nl * nl; ++s) modes[nm++] = cl2m[s];
  for (int s = 0; s < nl * nl; ++s) modes[nm++] = cm2l[s];
  for (int s = 0; s < nl; ++s) modes[nm++] = iRd2[s];
  harness_write(argv[3], "modes", modes, nm);
  char path[1024];
  snprintf(path, sizeof path, "%s.time", argv[3]);
  FILE* f = fopen(path, "w");
  if (f) {
    fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %d\n", t, dt, dt0, dt1, DT_max, t_out, steps);
    fclose(f);
  }
  return 0;
}
