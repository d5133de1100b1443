// qg_gpu.cpp -- the qg executable on GB300: the reference's driver
// (src/qg.c:103-226) on top of libqgw_gpu.so.
//
//   qg_gpu [params.in] [--fp32c]
//
// Same inputs and outputs as the reference: parameters from params.in
// (default name, or the path given), output into the first free
// outdir_NNNN/ with a copy of params.in, optional restart from restart.nc
// (record 0 of q and, if present, topo), vars.nc written at t = 0, dt_out,
// 2 dt_out, ... with psi and q including the wall ring.  Between outputs
// the time loop stays on the GPU (qgw_step stops exactly where the
// reference's loop would write the next output).
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qgw_gpu.h"

namespace {

const double kTeps = 1e-9;  // src/timestep.h:16

bool file_exists(const char* p) {
  struct stat st;
  return stat(p, &st) == 0;
}

// create_outdir, src/extra.h:164-178
std::string create_outdir() {
  char name[80];
  for (int i = 1; i < 10000; ++i) {
    std::snprintf(name, sizeof name, "outdir_%04d/", i);
    if (mkdir(name, 0777) == 0) {
      std::printf("Writing output in %s\n", name);
      return name;
    }
  }
  return "";
}

// backup_config, src/extra.h:181-195
void backup_config(const char* src, const std::string& dir) {
  FILE* in = std::fopen(src, "rb");
  FILE* out = std::fopen((dir + "params.in").c_str(), "wb");
  if (in && out) {
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, in)) > 0) std::fwrite(buf, 1, n, out);
  }
  if (in) std::fclose(in);
  if (out) std::fclose(out);
}

}  // namespace

int main(int argc, char** argv) {
  const char* file_param = "params.in";
  int precision = QGW_FP64;
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--fp32c")) precision = QGW_FP32C;
    else file_param = argv[a];
  }
  qgw_params p;
  qgw_params_default(&p);
  int rc = qgw_params_read(&p, file_param);
  if (rc == QGW_ERR_FILE) {
    std::printf("file %s not found\n", file_param);
    return 1;
  }
  const std::string dir = create_outdir();
  if (dir.empty()) return 1;
  backup_config(file_param, dir);

  // interior points: NX - 1 in a closed basin (src/domain.h:71-74), NX when
  // periodic; files hold the full grid with walls, or the periodic interior
  // (ibc = 1, src/netcdf_io.h:41-47,295-301)
  const bool per = p.bc_fac == -1;
  const int nx = per ? p.NX : p.NX - 1, ny = per ? p.NY : p.NY - 1, nl = p.nl;
  const int ibc = per ? 1 : 0, nxo = nx + 2 - 2 * ibc, nyo = ny + 2 - 2 * ibc;
  const size_t n2 = (size_t)(nx + 2) * (ny + 2), n3 = n2 * nl;
  const size_t n2o = (size_t)nxo * nyo, n3o = n2o * nl;
  // file layout <-> reference layout, nk fields
  auto to_ref = [&](const std::vector<double>& f, std::vector<double>& full, int nk) {
    for (int k = 0; k < nk; ++k)
      for (int j = ibc; j < ny + 2 - ibc; ++j)
        for (int i = ibc; i < nx + 2 - ibc; ++i)
          full[(size_t)k * n2 + (size_t)j * (nx + 2) + i] = f[(size_t)k * n2o + (size_t)(j - ibc) * nxo + (i - ibc)];
  };
  auto to_file = [&](const std::vector<double>& full, std::vector<double>& f, int nk) {
    for (int k = 0; k < nk; ++k)
      for (int j = ibc; j < ny + 2 - ibc; ++j)
        for (int i = ibc; i < nx + 2 - ibc; ++i)
          f[(size_t)k * n2o + (size_t)(j - ibc) * nxo + (i - ibc)] = full[(size_t)k * n2 + (size_t)j * (nx + 2) + i];
  };
  std::vector<double> cl2m((size_t)nl * nl), cm2l((size_t)nl * nl), iRd2(nl);
  if ((rc = qgw_eigmode(&p, cl2m.data(), cm2l.data(), iRd2.data()))) {
    std::printf("vertical modes: %s\n", qgw_strerror(rc));
    return 1;
  }
  std::printf("Deformation radii: \n");
  for (int k = 0; k < nl; ++k)
    std::printf("iRd2: %g , def radius: %g\n", iRd2[k], iRd2[k] > 0 ? std::sqrt(1 / iRd2[k]) : 0.0);

  // restart (src/qg.c:160-164): q and topo from record 0 of restart.nc
  std::vector<double> q(n3, 0.0), psi(n3, 0.0), topo, fbuf(n3o);
  if (file_exists("restart.nc")) {
    if (qgw_nc_read("restart.nc", "q", 0, fbuf.data(), (long)n3o) > 0) {
      std::printf("Reading variable  q!\n");
      to_ref(fbuf, q, nl);
    }
    topo.assign(n2, 0.0);
    std::vector<double> tb(n2o);
    if (qgw_nc_read("restart.nc", "topo", 0, tb.data(), (long)n2o) > 0) {
      std::printf("Reading variable  topo!\n");
      to_ref(tb, topo, 1);
    } else {
      topo.clear();
    }
  }
  qgw_run* run = nullptr;
  rc = qgw_create(&p, cl2m.data(), cm2l.data(), iRd2.data(), topo.empty() ? nullptr : topo.data(), precision, &run);
  if (rc) {
    std::printf("qgw_create: %s\n", qgw_strerror(rc));
    return 1;
  }
  qgw_set_q(run, q.data());
  // 4-D forcing: the n_rec records of q_forcing_3d in input_vars.nc
  // (init_4d_forcing / calc_4d_forcing, src/forcing.h:226-288), all
  // resident on the device; a missing file leaves zero records, as the
  // reference's read_nc prints its error and returns
  if (p.dt_forc_period != 0) {
    std::printf("Init 4d forcing. \n");
    const int n_rec = (int)std::floor(p.dt_forc_period / p.dt_forc);
    std::vector<double> rec((size_t)n_rec * n3, 0.0), one(n3);
    for (int r = 0; r < n_rec; ++r) {
      if (qgw_nc_read("input_vars.nc", "q_forcing_3d", r, fbuf.data(), (long)n3o) <= 0) {
        std::printf("input_vars.nc: record %d of q_forcing_3d not read\n", r);
        continue;
      }
      std::fill(one.begin(), one.end(), 0.0);
      to_ref(fbuf, one, nl);
      std::copy(one.begin(), one.end(), rec.begin() + (size_t)r * n3);
    }
    if ((rc = qgw_set_forcing_records(run, rec.data(), n_rec))) {
      std::printf("qgw_set_forcing_records: %s\n", qgw_strerror(rc));
      return 1;
    }
  }
  qgw_time tm;
  qgw_get_time(run, &tm);
  std::printf("Maximum time step: DT_MAX = %g \nInitial time step: dt = %g \n", tm.DT_max, tm.dt);

  qgw_nc* nc = qgw_nc_create((dir + "vars.nc").c_str(), nl, nyo, nxo, p.Lx / p.NX);
  std::vector<double> psio(n3o), qo(n3o);
  if (!nc) {
    std::printf("cannot create %svars.nc\n", dir.c_str());
    return 1;
  }
  double t = tm.t, dt = tm.dt, t_out = 0.0;
  long it = 0;
  // main loop, src/qg.c:181-200
  while (t < p.tend) {
    std::printf("i = %ld, t = %e dt = %e \n", it, t, dt);
    if (std::fabs(t - t_out) < kTeps * dt) {
      t_out += p.dt_out;
      qgw_get(run, psi.data(), q.data());
      std::printf("Write output, t = %e \n", t);
      to_file(psi, psio, nl);
      to_file(q, qo, nl);
      qgw_nc_write(nc, t, psio.data(), qo.data());
    }
    qgw_step_info info;
    rc = qgw_step(run, 1 << 30, t_out, p.tend, &info);
    if (rc) {
      std::printf("qgw_step: %s\n", qgw_strerror(rc));
      break;
    }
    t = info.time.t;
    dt = info.time.dt;
    it += info.steps_taken;
    if (info.steps_taken == 0) break;
  }
  qgw_nc_close(nc);
  qgw_destroy(run);
  return rc ? 1 : 0;
}
