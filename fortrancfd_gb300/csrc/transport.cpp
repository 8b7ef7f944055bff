// Transport fit loader: TRANLIB's linking file and the library's text form.
//
// The linking file is what the reference reads at start-up (set_trans,
// SRC/trans.f90:20-43, through MCLEN/MCINIT). Its records, in the order
// MCINIT reads them (tranlib.f:214-258):
//   1. VERS (16 chars), PREC (16 chars), KERR (logical)
//   2. LENIMC, LENRMC, NO, KK, NLITE (integers)
//   3. PATMOS, then per species WT, EPS, SIG, DIP, POL, ZROT (reals) and
//      NLIN (integer), then COFLAM(NO,KK), COFETA(NO,KK), COFD(NO,KK,KK),
//      KTDIF(NLITE) (integers) and COFTD(NO,KK,NLITE), Fortran array order.
// Each record is framed by 4-byte length markers (gfortran's sequential
// unformatted form). The text form holds the same numbers, printed with 17
// significant digits so that they read back bit for bit.
#include "transport.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

void set_err(char* err, int errlen, const std::string& s) {
  if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", s.c_str());
}

bool read_records(const char* path, std::vector<std::string>& recs) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::string all((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  size_t off = 0;
  while (off + 4 <= all.size()) {
    uint32_t n0, n1;
    std::memcpy(&n0, all.data() + off, 4);
    if (off + 8 + (size_t)n0 > all.size()) return false;
    std::memcpy(&n1, all.data() + off + 4 + n0, 4);
    if (n0 != n1) return false;
    recs.push_back(all.substr(off + 4, n0));
    off += 8 + (size_t)n0;
  }
  return off == all.size();
}

struct Cursor {
  const std::string& s;
  size_t p = 0;
  bool ok = true;
  double d() {
    double v = 0.0;
    if (p + 8 > s.size()) { ok = false; return v; }
    std::memcpy(&v, s.data() + p, 8);
    p += 8;
    return v;
  }
  int i() {
    int32_t v = 0;
    if (p + 4 > s.size()) { ok = false; return 0; }
    std::memcpy(&v, s.data() + p, 4);
    p += 4;
    return (int)v;
  }
};

}  // namespace

extern "C" int edyn_tran_read_bin(const char* path, edyn_tran* t, char* err, int errlen) {
  std::vector<std::string> recs;
  if (!read_records(path, recs) || recs.size() < 3) {
    set_err(err, errlen, std::string(path) + ": not a TRANLIB linking file");
    return 1;
  }
  std::memset(t, 0, sizeof(*t));
  if (recs[0].size() < 32 || recs[0].compare(16, 6, "DOUBLE") != 0) {
    set_err(err, errlen, std::string(path) + ": not a double-precision linking file");
    return 1;
  }
  Cursor h{recs[1]};
  h.i();
  h.i();
  t->no = h.i();
  t->kk = h.i();
  t->nlite = h.i();
  if (!h.ok || t->no != EDYN_TRAN_NO || t->kk < 1 || t->kk > EDYN_MAX_SPECIES || t->nlite < 0 ||
      t->nlite > EDYN_TRAN_MAXLITE) {
    set_err(err, errlen, std::string(path) + ": unsupported sizes (fit order 4, up to 64 species)");
    return 1;
  }
  const int kk = t->kk, no = t->no;
  Cursor c{recs[2]};
  t->patmos = c.d();
  for (int k = 0; k < kk; ++k) {
    t->wt[k] = c.d();
    t->eps[k] = c.d();
    t->sig[k] = c.d();
    t->dip[k] = c.d();
    t->pol[k] = c.d();
    t->zrot[k] = c.d();
    t->nlin[k] = c.i();
  }
  for (int k = 0; k < kk; ++k)
    for (int n = 0; n < no; ++n) t->coflam[k][n] = c.d();
  for (int k = 0; k < kk; ++k)
    for (int n = 0; n < no; ++n) t->cofeta[k][n] = c.d();
  for (int k = 0; k < kk; ++k)
    for (int j = 0; j < kk; ++j)
      for (int n = 0; n < no; ++n) t->cofd[k][j][n] = c.d();
  for (int l = 0; l < t->nlite; ++l) t->ktdif[l] = c.i() - 1;
  for (int l = 0; l < t->nlite; ++l)
    for (int k = 0; k < kk; ++k)
      for (int n = 0; n < no; ++n) t->coftd[l][k][n] = c.d();
  if (!c.ok || c.p != recs[2].size()) {
    set_err(err, errlen, std::string(path) + ": record 3 has the wrong length");
    return 1;
  }
  return 0;
}

extern "C" int edyn_tran_write(const edyn_tran* t, const edyn_mech* m, const char* path) {
  FILE* f = std::fopen(path, "w");
  if (!f) return 1;
  const int kk = t->kk, no = t->no;
  std::fprintf(f, "EDYNTRAN 1\n");
  std::fprintf(f, "KK %d NO %d NLITE %d PATMOS %.17g\n", kk, no, t->nlite, t->patmos);
  std::fprintf(f, "SPECIES\n");
  for (int k = 0; k < kk; ++k)
    std::fprintf(f, "%s %.17g %.17g %.17g %.17g %.17g %.17g %d\n", m ? m->spec_name[k] : "-", t->wt[k], t->eps[k],
                 t->sig[k], t->dip[k], t->pol[k], t->zrot[k], t->nlin[k]);
  std::fprintf(f, "COFETA\n");
  for (int k = 0; k < kk; ++k) {
    std::fprintf(f, "%d", k);
    for (int n = 0; n < no; ++n) std::fprintf(f, " %.17g", t->cofeta[k][n]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "COFLAM\n");
  for (int k = 0; k < kk; ++k) {
    std::fprintf(f, "%d", k);
    for (int n = 0; n < no; ++n) std::fprintf(f, " %.17g", t->coflam[k][n]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "COFD\n");
  for (int k = 0; k < kk; ++k)
    for (int j = 0; j < kk; ++j) {
      std::fprintf(f, "%d %d", k, j);
      for (int n = 0; n < no; ++n) std::fprintf(f, " %.17g", t->cofd[k][j][n]);
      std::fprintf(f, "\n");
    }
  std::fprintf(f, "KTDIF");
  for (int l = 0; l < t->nlite; ++l) std::fprintf(f, " %d", t->ktdif[l]);
  std::fprintf(f, "\nCOFTD\n");
  for (int l = 0; l < t->nlite; ++l)
    for (int k = 0; k < kk; ++k) {
      std::fprintf(f, "%d %d", l, k);
      for (int n = 0; n < no; ++n) std::fprintf(f, " %.17g", t->coftd[l][k][n]);
      std::fprintf(f, "\n");
    }
  std::fprintf(f, "END\n");
  return std::fclose(f) == 0 ? 0 : 1;
}

extern "C" int edyn_tran_read(const char* path, edyn_tran* t, char* err, int errlen) {
  std::ifstream f(path);
  if (!f) {
    set_err(err, errlen, std::string("cannot open ") + path);
    return 1;
  }
  std::memset(t, 0, sizeof(*t));
  std::string word;
  auto expect = [&](const char* w) {
    f >> word;
    return (bool)f && word == w;
  };
  auto bad = [&](const std::string& what) {
    set_err(err, errlen, std::string(path) + ": " + what);
    return 1;
  };
  int ver = 0;
  if (!expect("EDYNTRAN") || !(f >> ver) || ver != 1) return bad("not an EDYNTRAN 1 file");
  if (!expect("KK") || !(f >> t->kk) || !expect("NO") || !(f >> t->no) || !expect("NLITE") || !(f >> t->nlite) ||
      !expect("PATMOS") || !(f >> t->patmos))
    return bad("bad header");
  if (t->no != EDYN_TRAN_NO || t->kk < 1 || t->kk > EDYN_MAX_SPECIES || t->nlite < 0 ||
      t->nlite > EDYN_TRAN_MAXLITE)
    return bad("unsupported sizes");
  const int kk = t->kk, no = t->no;
  if (!expect("SPECIES")) return bad("SPECIES expected");
  for (int k = 0; k < kk; ++k) {
    std::string name;
    if (!(f >> name >> t->wt[k] >> t->eps[k] >> t->sig[k] >> t->dip[k] >> t->pol[k] >> t->zrot[k] >> t->nlin[k]))
      return bad("bad species line");
  }
  if (!expect("COFETA")) return bad("COFETA expected");
  for (int k = 0; k < kk; ++k) {
    int kr;
    if (!(f >> kr) || kr != k) return bad("bad COFETA line");
    for (int n = 0; n < no; ++n) f >> t->cofeta[k][n];
  }
  if (!expect("COFLAM")) return bad("COFLAM expected");
  for (int k = 0; k < kk; ++k) {
    int kr;
    if (!(f >> kr) || kr != k) return bad("bad COFLAM line");
    for (int n = 0; n < no; ++n) f >> t->coflam[k][n];
  }
  if (!expect("COFD")) return bad("COFD expected");
  for (int k = 0; k < kk; ++k)
    for (int j = 0; j < kk; ++j) {
      int kr, jr;
      if (!(f >> kr >> jr) || kr != k || jr != j) return bad("bad COFD line");
      for (int n = 0; n < no; ++n) f >> t->cofd[k][j][n];
    }
  if (!expect("KTDIF")) return bad("KTDIF expected");
  for (int l = 0; l < t->nlite; ++l) f >> t->ktdif[l];
  if (!expect("COFTD")) return bad("COFTD expected");
  for (int l = 0; l < t->nlite; ++l)
    for (int k = 0; k < kk; ++k) {
      int lr, kr;
      if (!(f >> lr >> kr) || lr != l || kr != k) return bad("bad COFTD line");
      for (int n = 0; n < no; ++n) f >> t->coftd[l][k][n];
    }
  if (!expect("END")) return bad("END expected");
  return 0;
}

extern "C" int edyn_tran_load_dir(const char* dir, edyn_tran* t, char* err, int errlen) {
  std::string d(dir ? dir : ".");
  std::string bin = d + "/tran.bin", txt = d + "/tran.edyn";
  if (std::ifstream(bin)) return edyn_tran_read_bin(bin.c_str(), t, err, errlen);
  if (std::ifstream(txt)) return edyn_tran_read(txt.c_str(), t, err, errlen);
  set_err(err, errlen, d + " holds neither tran.bin nor tran.edyn");
  return 1;
}
