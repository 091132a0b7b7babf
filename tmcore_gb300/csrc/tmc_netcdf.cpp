// NetCDF classic files (CDF-1 "CDF\1" and 64-bit-offset CDF-2 "CDF\2"),
// written and read without the NetCDF library: the MPAS grid file the
// reference reads in mesh_mod.F90:79-167, and the history file of
// history_mod.F90:27-174 (one record per output time).
//
// Format (NetCDF classic, public specification): big-endian; header =
// magic, numrecs, dim_list, global att_list, var_list; each variable lists
// its dimension ids, attributes, type, vsize and begin offset; fixed-size
// variables are stored contiguously at their offsets, record variables are
// interleaved per record after them.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "tmcore_gpu.h"

namespace {

enum NcType { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
constexpr uint32_t kDim = 0x0A, kVar = 0x0B, kAtt = 0x0C;

int type_size(int t) {
  switch (t) {
    case NC_BYTE:
    case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT:
    case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
  }
  return 0;
}

// ---- big-endian byte buffer -------------------------------------------------
struct Out {
  std::vector<uint8_t> b;
  void u32(uint32_t v) {
    for (int i = 3; i >= 0; --i) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void u64(uint64_t v) {
    for (int i = 7; i >= 0; --i) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void name(const std::string& s) {
    u32((uint32_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    while (b.size() % 4) b.push_back(0);
  }
};

void put_be(uint8_t* dst, const void* src, int esize, size_t n) {
  const uint8_t* s = static_cast<const uint8_t*>(src);
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < esize; ++k) dst[i * esize + k] = s[i * esize + (esize - 1 - k)];
}

struct In {
  const uint8_t* p;
  size_t n, pos = 0;
  bool ok = true;
  uint32_t u32() {
    if (pos + 4 > n) {
      ok = false;
      return 0;
    }
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v = (v << 8) | p[pos++];
    return v;
  }
  uint64_t u64() {
    if (pos + 8 > n) {
      ok = false;
      return 0;
    }
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v = (v << 8) | p[pos++];
    return v;
  }
  std::string name() {
    const uint32_t len = u32();
    if (!ok || pos + len > n) {
      ok = false;
      return "";
    }
    std::string s(reinterpret_cast<const char*>(p + pos), len);
    pos += (len + 3) / 4 * 4;
    return s;
  }
  void skip_atts() {
    const uint32_t tag = u32(), count = u32();
    if (tag == 0) return;
    for (uint32_t i = 0; i < count && ok; ++i) {
      name();
      const int t = (int)u32();
      const uint32_t len = u32();
      pos += ((size_t)len * type_size(t) + 3) / 4 * 4;
    }
  }
};

// ---- the file model -------------------------------------------------------------
struct Var {
  std::string name;
  std::vector<int> dims;
  int type = NC_DOUBLE;
  uint64_t begin = 0, vsize = 0;
  bool record = false;
};

struct NcFile {
  std::vector<std::pair<std::string, uint64_t>> dims;  // length 0: the record dimension
  std::vector<Var> vars;
  std::vector<std::pair<std::string, std::string>> gatts;
  uint64_t numrecs = 0, recsize = 0;
  int version = 2;

  int dim(const std::string& n) const {
    for (size_t i = 0; i < dims.size(); ++i)
      if (dims[i].first == n) return (int)i;
    return -1;
  }
  const Var* var(const std::string& n) const {
    for (const Var& v : vars)
      if (v.name == n) return &v;
    return nullptr;
  }
  uint64_t count(const Var& v) const {  // elements per record (or in all)
    uint64_t c = 1;
    for (int d : v.dims)
      if (dims[d].second) c *= dims[d].second;
    return c;
  }
};

bool parse_header(const std::vector<uint8_t>& buf, NcFile& f, std::string& err) {
  In in{buf.data(), buf.size()};
  if (buf.size() < 8 || std::memcmp(buf.data(), "CDF", 3) != 0 || (buf[3] != 1 && buf[3] != 2)) {
    err = "not a NetCDF classic (CDF-1/CDF-2) file";
    return false;
  }
  f.version = buf[3];
  in.pos = 4;
  f.numrecs = in.u32();
  uint32_t tag = in.u32(), n = in.u32();
  if (tag == kDim)
    for (uint32_t i = 0; i < n && in.ok; ++i) {
      std::string nm = in.name();
      f.dims.push_back({nm, in.u32()});
    }
  else if (tag != 0 || n != 0) return (err = "bad dimension list", false);
  // global attributes: keep text ones
  tag = in.u32();
  n = in.u32();
  if (tag == kAtt)
    for (uint32_t i = 0; i < n && in.ok; ++i) {
      std::string nm = in.name();
      const int t = (int)in.u32();
      const uint32_t len = in.u32();
      if (t == NC_CHAR && in.pos + len <= buf.size())
        f.gatts.push_back({nm, std::string(reinterpret_cast<const char*>(buf.data() + in.pos), len)});
      in.pos += ((size_t)len * type_size(t) + 3) / 4 * 4;
    }
  tag = in.u32();
  n = in.u32();
  if (tag == kVar)
    for (uint32_t i = 0; i < n && in.ok; ++i) {
      Var v;
      v.name = in.name();
      const uint32_t nd = in.u32();
      for (uint32_t k = 0; k < nd; ++k) v.dims.push_back((int)in.u32());
      in.skip_atts();
      v.type = (int)in.u32();
      v.vsize = in.u32();
      v.begin = f.version == 2 ? in.u64() : in.u32();
      for (int d : v.dims)
        if (d < 0 || d >= (int)f.dims.size()) return (err = "bad dimension id", false);
      v.record = !v.dims.empty() && f.dims[v.dims[0]].second == 0;
      f.vars.push_back(v);
    }
  if (!in.ok) return (err = "truncated header", false);
  for (const Var& v : f.vars)
    if (v.record) f.recsize += (v.vsize + 3) / 4 * 4;
  return true;
}

std::vector<uint8_t> build_header(const NcFile& f) {
  Out o;
  o.b = {'C', 'D', 'F', 2};
  o.u32((uint32_t)f.numrecs);
  if (f.dims.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(kDim);
    o.u32((uint32_t)f.dims.size());
    for (auto& d : f.dims) {
      o.name(d.first);
      o.u32((uint32_t)d.second);
    }
  }
  if (f.gatts.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(kAtt);
    o.u32((uint32_t)f.gatts.size());
    for (auto& a : f.gatts) {
      o.name(a.first);
      o.u32(NC_CHAR);
      o.u32((uint32_t)a.second.size());
      o.b.insert(o.b.end(), a.second.begin(), a.second.end());
      while (o.b.size() % 4) o.b.push_back(0);
    }
  }
  o.u32(kVar);
  o.u32((uint32_t)f.vars.size());
  for (const Var& v : f.vars) {
    o.name(v.name);
    o.u32((uint32_t)v.dims.size());
    for (int d : v.dims) o.u32((uint32_t)d);
    o.u32(0);
    o.u32(0);
    o.u32((uint32_t)v.type);
    o.u32((uint32_t)std::min<uint64_t>(v.vsize, 0xFFFFFFFFu));
    o.u64(v.begin);
  }
  return o.b;
}

// Lay out the variables after a header of `hdr` bytes: fixed variables in
// order, then the record section.
void layout(NcFile& f, size_t hdr) {
  uint64_t off = (hdr + 3) / 4 * 4;
  f.recsize = 0;
  for (Var& v : f.vars) {
    v.record = !v.dims.empty() && f.dims[v.dims[0]].second == 0;
    v.vsize = f.count(v) * type_size(v.type);
    if (!v.record) {
      v.begin = off;
      off += (v.vsize + 3) / 4 * 4;
    }
  }
  for (Var& v : f.vars)
    if (v.record) {
      v.begin = off + f.recsize;
      f.recsize += (v.vsize + 3) / 4 * 4;
    }
}

bool read_file(const char* path, std::vector<uint8_t>& buf, std::string& err) {
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return (err = std::string("cannot open ") + path, false);
  std::fseek(fp, 0, SEEK_END);
  const long sz = std::ftell(fp);
  std::fseek(fp, 0, SEEK_SET);
  buf.resize(sz > 0 ? (size_t)sz : 0);
  const size_t got = buf.empty() ? 0 : std::fread(buf.data(), 1, buf.size(), fp);
  std::fclose(fp);
  if (got != buf.size()) return (err = "short read", false);
  return true;
}

// values of a fixed variable (or record 0 of a record variable) converted to T
template <class T>
bool get_var(const NcFile& f, const std::vector<uint8_t>& buf, const std::string& name, std::vector<T>& out,
             std::string& err) {
  const Var* v = f.var(name);
  if (!v) return (err = "missing variable " + name, false);
  const uint64_t n = f.count(*v);
  const int es = type_size(v->type);
  if (v->begin + n * es > buf.size()) return (err = "variable " + name + " beyond the end of the file", false);
  out.resize(n);
  const uint8_t* s = buf.data() + v->begin;
  for (uint64_t i = 0; i < n; ++i) {
    uint8_t tmp[8];
    for (int k = 0; k < es; ++k) tmp[k] = s[i * es + (es - 1 - k)];
    double d = 0.0;
    switch (v->type) {
      case NC_BYTE: d = (double)(int8_t)tmp[0]; break;
      case NC_CHAR: d = (double)tmp[0]; break;
      case NC_SHORT: {
        int16_t x;
        std::memcpy(&x, tmp, 2);
        d = x;
        break;
      }
      case NC_INT: {
        int32_t x;
        std::memcpy(&x, tmp, 4);
        d = x;
        break;
      }
      case NC_FLOAT: {
        float x;
        std::memcpy(&x, tmp, 4);
        d = x;
        break;
      }
      case NC_DOUBLE: std::memcpy(&d, tmp, 8); break;
    }
    out[i] = (T)d;
  }
  return true;
}

const char* kIntVars[] = {"nEdgesOnCell", "nEdgesOnEdge", "cellsOnCell", "edgesOnCell", "verticesOnCell",
                          "cellsOnEdge", "verticesOnEdge", "edgesOnEdge", "cellsOnVertex", "edgesOnVertex"};
const char* kRealVars[] = {"xCell", "yCell", "zCell", "latCell", "xEdge", "yEdge", "zEdge", "xVertex", "yVertex",
                           "zVertex", "latVertex", "dvEdge", "dcEdge", "areaCell", "areaTriangle",
                           "kiteAreasOnVertex", "weightsOnEdge", "lonCell", "lonVertex"};

}  // namespace

struct tmc_mesh_file {
  std::map<std::string, std::vector<int32_t>> ints;
  std::map<std::string, std::vector<double>> reals;
  std::string err;
};

struct tmc_history {
  NcFile f;
  std::string path;
  std::string err;
};

extern "C" {

int tmc_mesh_file_open(const char* path, tmc_mesh_file** out, tmc_mesh_desc* d) {
  if (!path || !out || !d) return TMC_E_ARG;
  auto mf = std::make_unique<tmc_mesh_file>();
  std::vector<uint8_t> buf;
  NcFile f;
  std::string err;
  auto fail = [&](const std::string& e) {
    mf->err = e;
    *out = mf.release();
    return TMC_E_ARG;
  };
  if (!read_file(path, buf, err) || !parse_header(buf, f, err)) return fail(err);
  std::memset(d, 0, sizeof(*d));
  const char* dn[6] = {"nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree"};
  int32_t* dv[6] = {&d->nCells, &d->nEdges, &d->nVertices, &d->maxEdges, &d->maxEdges2, &d->vertexDegree};
  for (int i = 0; i < 6; ++i) {
    const int k = f.dim(dn[i]);
    if (k < 0) return fail(std::string("missing dimension ") + dn[i]);
    *dv[i] = (int32_t)f.dims[k].second;
  }
  for (const char* nm : kIntVars) {
    if (!f.var(nm)) continue;
    if (!get_var(f, buf, nm, mf->ints[nm], err)) return fail(err);
  }
  for (const char* nm : kRealVars) {
    if (!f.var(nm)) continue;
    if (!get_var(f, buf, nm, mf->reals[nm], err)) return fail(err);
  }
  auto I = [&](const char* nm) -> const int32_t* {
    auto it = mf->ints.find(nm);
    return it == mf->ints.end() ? nullptr : it->second.data();
  };
  auto R = [&](const char* nm) -> const double* {
    auto it = mf->reals.find(nm);
    return it == mf->reals.end() ? nullptr : it->second.data();
  };
  d->nEdgesOnCell = I("nEdgesOnCell");
  d->nEdgesOnEdge = I("nEdgesOnEdge");
  d->cellsOnCell = I("cellsOnCell");
  d->edgesOnCell = I("edgesOnCell");
  d->verticesOnCell = I("verticesOnCell");
  d->cellsOnEdge = I("cellsOnEdge");
  d->verticesOnEdge = I("verticesOnEdge");
  d->edgesOnEdge = I("edgesOnEdge");
  d->cellsOnVertex = I("cellsOnVertex");
  d->edgesOnVertex = I("edgesOnVertex");
  d->xCell = R("xCell");
  d->yCell = R("yCell");
  d->zCell = R("zCell");
  d->latCell = R("latCell");
  d->xEdge = R("xEdge");
  d->yEdge = R("yEdge");
  d->zEdge = R("zEdge");
  d->xVertex = R("xVertex");
  d->yVertex = R("yVertex");
  d->zVertex = R("zVertex");
  d->latVertex = R("latVertex");
  d->dvEdge = R("dvEdge");
  d->dcEdge = R("dcEdge");
  d->areaCell = R("areaCell");
  d->areaTriangle = R("areaTriangle");
  d->kiteAreasOnVertex = R("kiteAreasOnVertex");
  d->weightsOnEdge = R("weightsOnEdge");
  d->lonCell = R("lonCell");
  d->lonVertex = R("lonVertex");
  *out = mf.release();
  return TMC_OK;
}

const char* tmc_mesh_file_error(const tmc_mesh_file* f) { return f ? f->err.c_str() : "null file"; }

int tmc_mesh_file_close(tmc_mesh_file* f) {
  delete f;
  return TMC_OK;
}

// Fixed-size MPAS grid file: the dimensions and the arrays of d that are not NULL.
int tmc_mesh_file_write(const char* path, const tmc_mesh_desc* d) {
  if (!path || !d || d->nCells <= 0) return TMC_E_ARG;
  NcFile f;
  const char* dn[6] = {"nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree"};
  const int32_t dv[6] = {d->nCells, d->nEdges, d->nVertices, d->maxEdges, d->maxEdges2, d->vertexDegree};
  for (int i = 0; i < 6; ++i) f.dims.push_back({dn[i], (uint64_t)dv[i]});
  f.gatts.push_back({"on_a_sphere", "YES"});
  f.gatts.push_back({"source", "tmcore_gb300 tmc_mesh_file_write"});
  enum { C = 0, E = 1, V = 2, ME = 3, ME2 = 4, VD = 5 };
  struct Item {
    const char* name;
    const void* data;
    int type;
    std::vector<int> dims;
  };
  const Item items[] = {
      {"nEdgesOnCell", d->nEdgesOnCell, NC_INT, {C}},
      {"nEdgesOnEdge", d->nEdgesOnEdge, NC_INT, {E}},
      {"cellsOnCell", d->cellsOnCell, NC_INT, {C, ME}},
      {"edgesOnCell", d->edgesOnCell, NC_INT, {C, ME}},
      {"verticesOnCell", d->verticesOnCell, NC_INT, {C, ME}},
      {"cellsOnEdge", d->cellsOnEdge, NC_INT, {E, 6}},
      {"verticesOnEdge", d->verticesOnEdge, NC_INT, {E, 6}},
      {"edgesOnEdge", d->edgesOnEdge, NC_INT, {E, ME2}},
      {"cellsOnVertex", d->cellsOnVertex, NC_INT, {V, VD}},
      {"edgesOnVertex", d->edgesOnVertex, NC_INT, {V, VD}},
      {"xCell", d->xCell, NC_DOUBLE, {C}},
      {"yCell", d->yCell, NC_DOUBLE, {C}},
      {"zCell", d->zCell, NC_DOUBLE, {C}},
      {"latCell", d->latCell, NC_DOUBLE, {C}},
      {"lonCell", d->lonCell, NC_DOUBLE, {C}},
      {"xEdge", d->xEdge, NC_DOUBLE, {E}},
      {"yEdge", d->yEdge, NC_DOUBLE, {E}},
      {"zEdge", d->zEdge, NC_DOUBLE, {E}},
      {"xVertex", d->xVertex, NC_DOUBLE, {V}},
      {"yVertex", d->yVertex, NC_DOUBLE, {V}},
      {"zVertex", d->zVertex, NC_DOUBLE, {V}},
      {"latVertex", d->latVertex, NC_DOUBLE, {V}},
      {"lonVertex", d->lonVertex, NC_DOUBLE, {V}},
      {"dvEdge", d->dvEdge, NC_DOUBLE, {E}},
      {"dcEdge", d->dcEdge, NC_DOUBLE, {E}},
      {"areaCell", d->areaCell, NC_DOUBLE, {C}},
      {"areaTriangle", d->areaTriangle, NC_DOUBLE, {V}},
      {"kiteAreasOnVertex", d->kiteAreasOnVertex, NC_DOUBLE, {V, VD}},
      {"weightsOnEdge", d->weightsOnEdge, NC_DOUBLE, {E, ME2}},
  };
  f.dims.push_back({"TWO", 2});  // index 6
  std::vector<const void*> data;
  for (const Item& it : items) {
    if (!it.data) continue;
    Var v;
    v.name = it.name;
    v.dims = it.dims;
    v.type = it.type;
    f.vars.push_back(v);
    data.push_back(it.data);
  }
  std::vector<uint8_t> hdr = build_header(f);
  layout(f, hdr.size());
  hdr = build_header(f);  // same size: offsets are fixed-width
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return TMC_E_ARG;
  bool ok = std::fwrite(hdr.data(), 1, hdr.size(), fp) == hdr.size();
  for (size_t i = 0; i < f.vars.size() && ok; ++i) {
    const Var& v = f.vars[i];
    std::vector<uint8_t> out((v.vsize + 3) / 4 * 4, 0);
    put_be(out.data(), data[i], type_size(v.type), f.count(v));
    std::fseek(fp, (long)v.begin, SEEK_SET);
    ok = std::fwrite(out.data(), 1, out.size(), fp) == out.size();
  }
  std::fclose(fp);
  return ok ? TMC_OK : TMC_E_ARG;
}

// ---- history (history_mod.F90:27-174) ---------------------------------------------
int tmc_history_create(const char* path, const tmc_mesh_desc* d, tmc_history** out) {
  if (!path || !d || !out) return TMC_E_ARG;
  *out = nullptr;
  auto hw = std::make_unique<tmc_history>();
  hw->path = path;
  NcFile& f = hw->f;
  f.dims = {{"nCells", (uint64_t)d->nCells}, {"nEdges", (uint64_t)d->nEdges}, {"nVertices", (uint64_t)d->nVertices},
            {"Time", 0}};
  f.gatts.push_back({"source", "tmcore_gb300 history (history_mod.F90 fields)"});
  struct Item {
    const char* name;
    const double* data;
    int dim;
  };
  const Item fixed[] = {{"lonCell", d->lonCell, 0},     {"latCell", d->latCell, 0},     {"xCell", d->xCell, 0},
                        {"yCell", d->yCell, 0},         {"zCell", d->zCell, 0},         {"xEdge", d->xEdge, 1},
                        {"yEdge", d->yEdge, 1},         {"zEdge", d->zEdge, 1},         {"lonVertex", d->lonVertex, 2},
                        {"latVertex", d->latVertex, 2}, {"xVertex", d->xVertex, 2},     {"yVertex", d->yVertex, 2},
                        {"zVertex", d->zVertex, 2},     {"areaCell", d->areaCell, 0},   {"areaTriangle", d->areaTriangle, 2}};
  std::vector<const double*> fdata;
  for (const Item& it : fixed) {
    if (!it.data) continue;
    Var v;
    v.name = it.name;
    v.dims = {it.dim};
    f.vars.push_back(v);
    fdata.push_back(it.data);
  }
  // record variables: time, then the fields of history_write_state
  const std::pair<const char*, std::vector<int>> rec[] = {
      {"time", {3}},     {"u", {3, 1}},   {"zonalWind", {3, 0}}, {"merdionalWind", {3, 0}}, {"h", {3, 0}},
      {"pv", {3, 2}},    {"vor", {3, 2}}, {"div", {3, 0}},       {"tm", {3}},               {"te", {3}}};
  for (auto& r : rec) {
    Var v;
    v.name = r.first;
    v.dims = r.second;
    f.vars.push_back(v);
  }
  std::vector<uint8_t> hdr = build_header(f);
  layout(f, hdr.size());
  hdr = build_header(f);
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return TMC_E_ARG;
  bool ok = std::fwrite(hdr.data(), 1, hdr.size(), fp) == hdr.size();
  size_t k = 0;
  for (const Var& v : f.vars) {
    if (v.record || !ok) continue;
    std::vector<uint8_t> outb((v.vsize + 3) / 4 * 4, 0);
    put_be(outb.data(), fdata[k++], 8, f.count(v));
    std::fseek(fp, (long)v.begin, SEEK_SET);
    ok = std::fwrite(outb.data(), 1, outb.size(), fp) == outb.size();
  }
  std::fclose(fp);
  if (!ok) return TMC_E_ARG;
  *out = hw.release();
  return TMC_OK;
}

// One record: the history fields of state(old) of the handle's selected
// member and its total mass and energy, at `seconds`.
int tmc_history_write(tmc_history* hw, tmc_handle* h, double seconds) {
  if (!hw || !h) return TMC_E_ARG;
  NcFile& f = hw->f;
  const int nc = (int)f.dims[0].second, ne = (int)f.dims[1].second, nv = (int)f.dims[2].second;
  std::vector<double> u(ne), zon(nc), mer(nc), hc(nc), div(nc), pv(nv), vor(nv), diag(5);
  int rc = tmc_history_fields(h, u.data(), zon.data(), mer.data(), hc.data(), div.data(), pv.data(), vor.data());
  if (rc) return rc;
  if ((rc = tmc_get_diag(h, diag.data()))) return rc;
  const double t = seconds, tm = diag[0], te = diag[1];
  std::map<std::string, const double*> src = {{"time", &t},  {"u", u.data()},   {"zonalWind", zon.data()},
                                              {"merdionalWind", mer.data()}, {"h", hc.data()}, {"pv", pv.data()},
                                              {"vor", vor.data()}, {"div", div.data()}, {"tm", &tm}, {"te", &te}};
  FILE* fp = std::fopen(hw->path.c_str(), "r+b");
  if (!fp) return TMC_E_ARG;
  bool ok = true;
  for (const Var& v : f.vars) {
    if (!v.record || !ok) continue;
    std::vector<uint8_t> outb((v.vsize + 3) / 4 * 4, 0);
    put_be(outb.data(), src[v.name], 8, f.count(v));
    std::fseek(fp, (long)(v.begin + f.numrecs * f.recsize), SEEK_SET);
    ok = std::fwrite(outb.data(), 1, outb.size(), fp) == outb.size();
  }
  f.numrecs += 1;
  uint8_t nr[4];
  const uint32_t n32 = (uint32_t)f.numrecs;
  for (int i = 0; i < 4; ++i) nr[i] = (uint8_t)(n32 >> (8 * (3 - i)));
  std::fseek(fp, 4, SEEK_SET);
  ok = ok && std::fwrite(nr, 1, 4, fp) == 4;
  std::fclose(fp);
  return ok ? TMC_OK : TMC_E_ARG;
}

int tmc_history_close(tmc_history* hw) {
  delete hw;
  return TMC_OK;
}

}  // extern "C"
