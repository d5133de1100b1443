// ncio.cpp -- netCDF-3 classic files for qgw output and restart, written
// from the published netCDF classic format specification (big-endian
// header of dimensions / attributes / variables, fixed-size variables
// first, then one record per unlimited-dimension step with every record
// variable's slice).  No netCDF library is needed.
//
// vars.nc layout of the reference (src/netcdf_io.h:38-163,171-277):
//   dims   t (unlimited), level (nl), y (NY_Out), x (NX_Out)
//   vars   t(t), y(y), x(x), level(level)   float coordinates
//          psi(t, level, y, x), q(t, level, y, x)   float, walls included
// restart.nc: record 0 of `q` (3-D) and `topo` (2-D) if present
// (src/netcdf_io.h:286-382); this reader uses the file's own dimension
// order, which avoids the reference's transposed x/y counts.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qgw_gpu.h"

namespace {

const uint32_t NC_DIMENSION = 0x0A, NC_VARIABLE = 0x0B, NC_ATTRIBUTE = 0x0C;
const uint32_t NC_FLOAT_T = 5, NC_DOUBLE_T = 6;

void put32(std::vector<uint8_t>& b, uint32_t v) {
  b.push_back((uint8_t)(v >> 24));
  b.push_back((uint8_t)(v >> 16));
  b.push_back((uint8_t)(v >> 8));
  b.push_back((uint8_t)v);
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
  put32(b, (uint32_t)(v >> 32));
  put32(b, (uint32_t)v);
}
void putname(std::vector<uint8_t>& b, const std::string& s) {
  put32(b, (uint32_t)s.size());
  for (char c : s) b.push_back((uint8_t)c);
  while (b.size() % 4) b.push_back(0);
}
void be_floats(const float* src, size_t n, std::vector<uint8_t>& out) {
  out.resize(n * 4);
  for (size_t i = 0; i < n; ++i) {
    uint32_t u;
    std::memcpy(&u, &src[i], 4);
    out[4 * i] = (uint8_t)(u >> 24);
    out[4 * i + 1] = (uint8_t)(u >> 16);
    out[4 * i + 2] = (uint8_t)(u >> 8);
    out[4 * i + 3] = (uint8_t)u;
  }
}

struct VarDef {
  std::string name;
  std::vector<int> dims;
  bool record;
  uint64_t vsize;
  uint64_t begin;
  size_t begin_pos;  // position of the begin field in the header
};

}  // namespace

struct qgw_nc {
  FILE* f = nullptr;
  int nl = 0, ny = 0, nx = 0;
  uint64_t recsize = 0, rec0 = 0;
  uint32_t numrecs = 0;
  uint64_t off_t_, off_psi, off_q;  // offsets inside one record
};

extern "C" {

// Create vars.nc for nl layers on a (ny_out, nx_out) grid (walls included)
// with coordinates x_i = i*Delta, y_j = j*Delta, level_k = k.
qgw_nc* qgw_nc_create(const char* path, int nl, int ny_out, int nx_out, double Delta) {
  if (!path || nl < 1 || ny_out < 1 || nx_out < 1) return nullptr;
  qgw_nc* h = new qgw_nc();
  h->nl = nl;
  h->ny = ny_out;
  h->nx = nx_out;
  std::vector<uint8_t> b;
  b.insert(b.end(), {'C', 'D', 'F', 2});  // 64-bit offsets: large grids exceed 2 GiB
  put32(b, 0);                          // numrecs
  // dimensions: t, level, y, x (src/netcdf_io.h:65-74)
  put32(b, NC_DIMENSION);
  put32(b, 4);
  putname(b, "t"); put32(b, 0);
  putname(b, "level"); put32(b, (uint32_t)nl);
  putname(b, "y"); put32(b, (uint32_t)ny_out);
  putname(b, "x"); put32(b, (uint32_t)nx_out);
  put32(b, 0); put32(b, 0);  // no global attributes
  // variables in the reference's definition order (src/netcdf_io.h:82-119)
  std::vector<VarDef> vars = {
      {"t", {0}, true, 4, 0, 0},
      {"y", {2}, false, (uint64_t)ny_out * 4, 0, 0},
      {"x", {3}, false, (uint64_t)nx_out * 4, 0, 0},
      {"level", {1}, false, (uint64_t)nl * 4, 0, 0},
      {"psi", {0, 1, 2, 3}, true, (uint64_t)nl * ny_out * nx_out * 4, 0, 0},
      {"q", {0, 1, 2, 3}, true, (uint64_t)nl * ny_out * nx_out * 4, 0, 0},
  };
  put32(b, NC_VARIABLE);
  put32(b, (uint32_t)vars.size());
  for (auto& v : vars) {
    putname(b, v.name);
    put32(b, (uint32_t)v.dims.size());
    for (int d : v.dims) put32(b, (uint32_t)d);
    put32(b, 0); put32(b, 0);  // no attributes
    put32(b, NC_FLOAT_T);
    const uint64_t vs = (v.vsize + 3) / 4 * 4;
    put32(b, vs > 0xffffffffULL ? 0xffffffffu : (uint32_t)vs);
    v.begin_pos = b.size();
    put64(b, 0);
  }
  // fixed-size variables, then the records
  uint64_t off = b.size();
  for (auto& v : vars)
    if (!v.record) { v.begin = off; off += (v.vsize + 3) / 4 * 4; }
  h->rec0 = off;
  uint64_t roff = 0;
  for (auto& v : vars)
    if (v.record) {
      v.begin = h->rec0 + roff;
      if (v.name == "t") h->off_t_ = roff;
      if (v.name == "psi") h->off_psi = roff;
      if (v.name == "q") h->off_q = roff;
      roff += v.vsize;  // record slices of float data are 4-byte multiples
    }
  h->recsize = roff;
  for (auto& v : vars)
    for (int k = 0; k < 8; ++k) b[v.begin_pos + k] = (uint8_t)(v.begin >> (56 - 8 * k));
  h->f = std::fopen(path, "wb+");
  if (!h->f) { delete h; return nullptr; }
  std::fwrite(b.data(), 1, b.size(), h->f);
  std::vector<float> yc(ny_out), xc(nx_out), zc(nl);
  for (int i = 0; i < ny_out; ++i) yc[i] = (float)(i * Delta);
  for (int i = 0; i < nx_out; ++i) xc[i] = (float)(i * Delta);
  for (int i = 0; i < nl; ++i) zc[i] = (float)i;
  std::vector<uint8_t> tmp;
  for (const auto* arr : {&yc, &xc, &zc}) {
    be_floats(arr->data(), arr->size(), tmp);
    std::fwrite(tmp.data(), 1, tmp.size(), h->f);
    while (tmp.size() % 4) { tmp.push_back(0); std::fputc(0, h->f); }
  }
  std::fflush(h->f);
  return h;
}

// Append one record: time t and the FP64 fields psi, q in the reference
// layout, cast to float (src/netcdf_io.h:181,248).
int qgw_nc_write(qgw_nc* h, double t, const double* psi, const double* q) {
  if (!h || !h->f || !psi || !q) return QGW_ERR_PARAM;
  const size_t n = (size_t)h->nl * h->ny * h->nx;
  std::vector<float> fl(n);
  std::vector<uint8_t> tmp;
  const uint64_t base = h->rec0 + (uint64_t)h->numrecs * h->recsize;
  float tf = (float)t;
  be_floats(&tf, 1, tmp);
  if (fseeko(h->f, (off_t)(base + h->off_t_), SEEK_SET)) return QGW_ERR_FILE;
  std::fwrite(tmp.data(), 1, 4, h->f);
  for (int v = 0; v < 2; ++v) {
    const double* src = v == 0 ? psi : q;
    for (size_t i = 0; i < n; ++i) fl[i] = (float)src[i];
    be_floats(fl.data(), n, tmp);
    if (fseeko(h->f, (off_t)(base + (v == 0 ? h->off_psi : h->off_q)), SEEK_SET)) return QGW_ERR_FILE;
    if (std::fwrite(tmp.data(), 1, tmp.size(), h->f) != tmp.size()) return QGW_ERR_FILE;
  }
  h->numrecs += 1;
  uint8_t nr[4] = {(uint8_t)(h->numrecs >> 24), (uint8_t)(h->numrecs >> 16), (uint8_t)(h->numrecs >> 8),
                   (uint8_t)h->numrecs};
  fseeko(h->f, 4, SEEK_SET);
  std::fwrite(nr, 1, 4, h->f);
  std::fflush(h->f);
  return QGW_OK;
}

void qgw_nc_close(qgw_nc* h) {
  if (!h) return;
  if (h->f) std::fclose(h->f);
  delete h;
}

// Read record `rec` of variable `name` (float or double, any rank whose
// trailing dimensions hold count values) into out as doubles.  Returns the
// number of values read, or a negative status (QGW_ERR_FILE when the file
// or the variable is missing, QGW_ERR_PARAM when the size differs).
long qgw_nc_read(const char* path, const char* name, int rec, double* out, long count) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return QGW_ERR_FILE;
  std::vector<uint8_t> buf;
  {
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    if (std::fread(buf.data(), 1, buf.size(), f) != buf.size()) { std::fclose(f); return QGW_ERR_FILE; }
  }
  std::fclose(f);
  size_t p = 0;
  auto need = [&](size_t n) { return p + n <= buf.size(); };
  auto get32 = [&]() -> uint32_t {
    uint32_t v = ((uint32_t)buf[p] << 24) | ((uint32_t)buf[p + 1] << 16) | ((uint32_t)buf[p + 2] << 8) | buf[p + 3];
    p += 4;
    return v;
  };
  auto getname = [&]() -> std::string {
    uint32_t n = get32();
    std::string s((const char*)&buf[p], n);
    p += (n + 3) / 4 * 4;
    return s;
  };
  if (!need(8) || buf[0] != 'C' || buf[1] != 'D' || buf[2] != 'F') return QGW_ERR_FILE;
  const int version = buf[3];
  p = 4;
  get32();  // numrecs
  std::vector<uint32_t> dimlen;
  int recdim = -1;
  uint32_t tag = get32(), nel = get32();
  if (tag == NC_DIMENSION)
    for (uint32_t i = 0; i < nel; ++i) {
      getname();
      uint32_t len = get32();
      if (len == 0) recdim = (int)i;
      dimlen.push_back(len);
    }
  auto skip_atts = [&]() {
    uint32_t t = get32(), n = get32();
    if (t != NC_ATTRIBUTE) return;
    for (uint32_t i = 0; i < n; ++i) {
      getname();
      uint32_t type = get32(), nv = get32();
      const uint32_t sz[] = {0, 1, 1, 2, 4, 4, 8};
      p += ((size_t)nv * (type < 7 ? sz[type] : 1) + 3) / 4 * 4;
    }
  };
  skip_atts();
  tag = get32();
  nel = get32();
  struct V { std::string name; std::vector<uint32_t> dims; uint32_t type; uint64_t vsize, begin; };
  std::vector<V> vars;
  if (tag == NC_VARIABLE)
    for (uint32_t i = 0; i < nel; ++i) {
      V v;
      v.name = getname();
      uint32_t nd = get32();
      for (uint32_t d = 0; d < nd; ++d) v.dims.push_back(get32());
      skip_atts();
      v.type = get32();
      v.vsize = get32();
      if (version == 1) v.begin = get32();
      else { uint64_t hi = get32(); v.begin = (hi << 32) | get32(); }
      vars.push_back(v);
    }
  uint64_t recsize = 0;
  for (auto& v : vars)
    if (!v.dims.empty() && (int)v.dims[0] == recdim) recsize += v.vsize;
  for (auto& v : vars) {
    if (v.name != name) continue;
    const bool isrec = !v.dims.empty() && (int)v.dims[0] == recdim;
    long n = 1;
    for (size_t d = isrec ? 1 : 0; d < v.dims.size(); ++d) n *= (long)dimlen[v.dims[d]];
    if (n != count) return QGW_ERR_PARAM;
    uint64_t off = v.begin + (isrec ? (uint64_t)rec * recsize : 0);
    const int esz = v.type == NC_DOUBLE_T ? 8 : 4;
    if (off + (uint64_t)n * esz > buf.size()) return QGW_ERR_FILE;
    const uint8_t* s = &buf[off];
    for (long i = 0; i < n; ++i) {
      if (esz == 4) {
        uint32_t u = ((uint32_t)s[4 * i] << 24) | ((uint32_t)s[4 * i + 1] << 16) | ((uint32_t)s[4 * i + 2] << 8) |
                     s[4 * i + 3];
        float fv;
        std::memcpy(&fv, &u, 4);
        out[i] = fv;
      } else {
        uint64_t u = 0;
        for (int k = 0; k < 8; ++k) u = (u << 8) | s[8 * i + k];
        double dv;
        std::memcpy(&dv, &u, 8);
        out[i] = dv;
      }
    }
    return n;
  }
  return QGW_ERR_FILE;
}

}  // extern "C"
