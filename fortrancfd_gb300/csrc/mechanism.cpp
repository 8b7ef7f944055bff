// CHEMKIN-II text mechanism front end (host C++).
//
// Replaces the reference's CKINTERP step (GRI/ckinterp.f), which turns
// chem.inp + therm.dat into the chem.bin linking file that set_thermo loads
// (SRC/thermo.f90:25-67). The parser reads the same text and fills an
// edyn_mech struct; it reproduces the numeric conventions of that interpreter
// so that every derived table matches the reference bit for bit:
//   * atomic weights come from single-precision literals widened to double
//     (DATA table at GRI/ckinterp.f:968-972), and molecular weights are summed
//     over the element fields of the thermo card in card order
//     (GRI/ckinterp.f:1079-1099);
//   * activation energies are converted to Kelvin with EFAC = 4.184/RU_JOUL
//     where 4.184 is again a single-precision literal
//     (GRI/ckinterp.f:2420-2443);
//   * the thermo card's first seven coefficients are the upper range, the
//     next seven the lower range (GRI/ckinterp.f:1120-1124);
//   * a species repeated on one side of a reaction is folded into one slot
//     with a summed coefficient (GRI/ckinterp.f:1484-1500).
// A compact text form of the same tables ("mech.edyn") can be written and
// read back, so a run needs no CHEMKIN sources at all.
#include "mechanism.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

const double RU_JOUL = 8.314510;

std::string upper(std::string s) {
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

std::vector<std::string> split_ws(const std::string& s) {
  std::istringstream is(s);
  std::vector<std::string> out;
  std::string t;
  while (is >> t) out.push_back(t);
  return out;
}

bool parse_double(std::string s, double* v) {
  s = trim(s);
  if (s.empty()) return false;
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'E';
  char* end = nullptr;
  *v = std::strtod(s.c_str(), &end);
  return end && *end == '\0';
}

// Atomic weights of the interpreter's element table, as the single-precision
// literals it declares.
bool default_atomic_weight(const std::string& e, double* w) {
  static const std::map<std::string, float> tab = {
      {"H", 1.00797f},  {"HE", 4.00260f}, {"C", 12.01115f}, {"N", 14.00670f},
      {"O", 15.99940f}, {"F", 18.99840f}, {"NE", 20.18300f}, {"AR", 39.94800f},
      {"S", 32.06400f}, {"CL", 35.45300f}, {"KR", 83.80000f}, {"XE", 131.30000f},
      {"E", 5.45e-4f}};
  auto it = tab.find(upper(e));
  if (it == tab.end()) return false;
  *w = (double)it->second;
  return true;
}

struct Ctx {
  edyn_mech* m;
  std::string err;
  int find_species(const std::string& name) const {
    std::string u = upper(name);
    for (int k = 0; k < m->nspec; ++k)
      if (upper(m->spec_name[k]) == u) return k;
    return -1;
  }
  int find_element(const std::string& name) const {
    std::string u = upper(trim(name));
    for (int e = 0; e < m->nelem; ++e)
      if (upper(m->elem_name[e]) == u) return e;
    return -1;
  }
};

std::string strip_comment(const std::string& line) {
  size_t p = line.find('!');
  return p == std::string::npos ? line : line.substr(0, p);
}

// Parses thermo cards (NASA-7, 80-column fixed format). Only species of the
// mechanism that have not yet received data are filled; the first card wins.
bool read_thermo(Ctx& c, const std::vector<std::string>& lines, size_t start, std::vector<bool>& have) {
  edyn_mech* m = c.m;
  double tlo = 300.0, tmid = 1000.0, thi = 5000.0;
  size_t i = start;
  // Optional default temperature line directly after the THERMO keyword.
  while (i < lines.size() && trim(strip_comment(lines[i])).empty()) ++i;
  if (i < lines.size()) {
    auto tk = split_ws(strip_comment(lines[i]));
    double v[3];
    if (tk.size() >= 3 && parse_double(tk[0], &v[0]) && parse_double(tk[1], &v[1]) &&
        parse_double(tk[2], &v[2])) {
      tlo = v[0]; tmid = v[1]; thi = v[2];
      ++i;
    }
  }
  for (; i < lines.size(); ++i) {
    const std::string& l1 = lines[i];
    std::string u = upper(trim(l1));
    if (u.rfind("END", 0) == 0 || u.rfind("REAC", 0) == 0) break;
    if (l1.size() < 80 || l1[79] != '1') continue;
    std::string name = split_ws(l1.substr(0, 18)).empty() ? "" : split_ws(l1.substr(0, 18))[0];
    int k = c.find_species(name);
    if (i + 3 >= lines.size()) break;
    if (k < 0 || have[k]) { i += 3; continue; }
    const std::string &l2 = lines[i + 1], &l3 = lines[i + 2], &l4 = lines[i + 3];
    if (l2.size() < 75 || l3.size() < 75 || l4.size() < 60) {
      c.err = "short thermo card for " + name;
      return false;
    }
    // Element fields: columns 25-44 (four of five characters) and 74-78.
    double wt = 0.0;
    for (int f = 0; f < 5; ++f) {
      size_t col = (f < 4) ? (size_t)(24 + 5 * f) : (size_t)73;
      if (l1.size() < col + 5) continue;
      std::string el = l1.substr(col, 2), cnt = l1.substr(col + 2, 3);
      int ne = 0;
      if (!trim(cnt).empty()) {
        double v;
        if (!parse_double(cnt, &v)) { c.err = "bad element count for " + name; return false; }
        ne = (int)v;
      }
      if (trim(el).empty() || ne == 0) continue;
      int e = c.find_element(el);
      if (e < 0) { c.err = "undeclared element " + el + " in " + name; return false; }
      m->elem_count[k][e] = ne;
      wt = wt + m->elem_weight[e] * (double)(float)ne;
    }
    m->W[k] = wt;
    double v;
    m->T_lo[k] = tlo; m->T_mid[k] = tmid; m->T_hi[k] = thi;
    if (!trim(l1.substr(45, 10)).empty() && parse_double(l1.substr(45, 10), &v)) m->T_lo[k] = v;
    if (!trim(l1.substr(65, 8)).empty() && parse_double(l1.substr(65, 8), &v)) m->T_mid[k] = v;
    if (!trim(l1.substr(55, 10)).empty() && parse_double(l1.substr(55, 10), &v)) m->T_hi[k] = v;
    double a[15];
    const std::string* src[3] = {&l2, &l3, &l4};
    int n = 0;
    for (int r = 0; r < 3; ++r) {
      int nf = (r < 2) ? 5 : 4;
      for (int f = 0; f < nf; ++f) {
        if (!parse_double(src[r]->substr(15 * f, 15), &a[n])) {
          c.err = "bad thermo coefficient for " + name;
          return false;
        }
        ++n;
      }
    }
    for (int j = 0; j < 7; ++j) {
      m->a[k][1][j] = a[j];      // upper range
      m->a[k][0][j] = a[7 + j];  // lower range
    }
    have[k] = true;
    i += 3;
  }
  return true;
}

// Splits "KEY/values/ KEY/values/ DUP" auxiliary lines into (key, value) items.
std::vector<std::pair<std::string, std::string>> aux_items(const std::string& line) {
  std::vector<std::pair<std::string, std::string>> out;
  size_t i = 0, n = line.size();
  while (i < n) {
    while (i < n && std::isspace((unsigned char)line[i])) ++i;
    if (i >= n) break;
    size_t k0 = i;
    while (i < n && line[i] != '/' && !std::isspace((unsigned char)line[i])) ++i;
    std::string key = line.substr(k0, i - k0);
    size_t j = i;
    while (j < n && std::isspace((unsigned char)line[j])) ++j;
    std::string val;
    bool has = false;
    if (j < n && line[j] == '/') {
      size_t e = line.find('/', j + 1);
      if (e == std::string::npos) e = n;
      val = line.substr(j + 1, e - j - 1);
      has = true;
      i = (e < n) ? e + 1 : n;
    }
    if (!key.empty()) out.push_back({key, has ? val : std::string()});
  }
  return out;
}

bool parse_side(Ctx& c, std::string s, int ireac, bool reactants, int* tb_flag) {
  edyn_mech* m = c.m;
  // Split on '+' that separates species (a '+' at position 0 cannot).
  std::vector<std::string> toks;
  std::string cur;
  for (size_t i = 0; i < s.size(); ++i) {
    if (s[i] == '+' && i > 0 && !cur.empty()) {
      toks.push_back(cur);
      cur.clear();
    } else {
      cur += s[i];
    }
  }
  if (!cur.empty()) toks.push_back(cur);
  int base = reactants ? 0 : 3;
  for (auto& t : toks) {
    if (upper(t) == "M") { *tb_flag = 1; continue; }
    int coef = 1;
    std::string name = t;
    int k = c.find_species(name);
    if (k < 0) {
      size_t d = 0;
      while (d < t.size() && std::isdigit((unsigned char)t[d])) ++d;
      if (d > 0 && d < t.size()) {
        coef = std::atoi(t.substr(0, d).c_str());
        name = t.substr(d);
        k = c.find_species(name);
      }
    }
    if (k < 0) { c.err = "unknown species '" + t + "' in reaction " + m->equation[ireac]; return false; }
    int slot = -1;
    for (int q = base; q < base + 3; ++q)
      if (m->nunk[ireac][q] == k) slot = q;
    if (slot < 0) {
      for (int q = base; q < base + 3; ++q)
        if (m->nunk[ireac][q] < 0) { slot = q; break; }
      if (slot < 0) { c.err = std::string("more than three species on one side: ") + m->equation[ireac]; return false; }
      m->nunk[ireac][slot] = k;
      m->nu[ireac][slot] = 0;
    }
    m->nu[ireac][slot] += reactants ? -coef : coef;
  }
  return true;
}

// Removes a "(+M)" / "(+SPECIES)" marker; returns 0 none, -1 mixture, k+1 species.
int strip_falloff(Ctx& c, std::string& s) {
  size_t p = s.find("(+");
  while (p != std::string::npos) {
    size_t e = s.find(')', p);
    if (e == std::string::npos) return 0;
    std::string inner = s.substr(p + 2, e - p - 2);
    int code = 0;
    if (upper(inner) == "M") code = -1;
    else {
      int k = c.find_species(inner);
      if (k >= 0) code = k + 1;
    }
    if (code != 0) {
      s = s.substr(0, p) + s.substr(e + 1);
      return code;
    }
    p = s.find("(+", p + 2);
  }
  return 0;
}

bool parse_reaction_line(Ctx& c, const std::string& line, double efac) {
  edyn_mech* m = c.m;
  auto tk = split_ws(line);
  if (tk.size() < 4) { c.err = "reaction line needs an equation and three numbers: " + line; return false; }
  double A, b, E;
  size_t nt = tk.size();
  if (!parse_double(tk[nt - 3], &A) || !parse_double(tk[nt - 2], &b) || !parse_double(tk[nt - 1], &E)) {
    c.err = "bad Arrhenius numbers: " + line;
    return false;
  }
  std::string eq;
  for (size_t i = 0; i + 3 < nt; ++i) eq += tk[i];
  if (m->nreac >= EDYN_MAX_REACTIONS) { c.err = "too many reactions"; return false; }
  int i = m->nreac++;
  std::snprintf(m->equation[i], sizeof(m->equation[i]), "%s", eq.c_str());
  for (int q = 0; q < 6; ++q) { m->nunk[i][q] = -1; m->nu[i][q] = 0; }
  std::string lhs, rhs;
  size_t p;
  if ((p = eq.find("<=>")) != std::string::npos) { lhs = eq.substr(0, p); rhs = eq.substr(p + 3); m->rev[i] = 1; }
  else if ((p = eq.find("=>")) != std::string::npos) { lhs = eq.substr(0, p); rhs = eq.substr(p + 2); m->rev[i] = 0; }
  else if ((p = eq.find('=')) != std::string::npos) { lhs = eq.substr(0, p); rhs = eq.substr(p + 1); m->rev[i] = 1; }
  else { c.err = "no '=' in reaction " + eq; return false; }
  int fl = strip_falloff(c, lhs), fr = strip_falloff(c, rhs);
  m->tb[i] = EDYN_TB_NONE;
  m->kfal[i] = -1;
  m->ifop[i] = EDYN_FO_NONE;
  if (fl != 0 || fr != 0) {
    if (fl != fr) { c.err = "mismatched fall-off collider in " + eq; return false; }
    m->tb[i] = EDYN_TB_FALLOFF;
    m->ifop[i] = EDYN_FO_LINDEMANN;
    m->kfal[i] = fl > 0 ? fl - 1 : -1;
  }
  int tbl = 0, tbr = 0;
  if (!parse_side(c, lhs, i, true, &tbl)) return false;
  if (!parse_side(c, rhs, i, false, &tbr)) return false;
  if (tbl || tbr) {
    if (m->tb[i] == EDYN_TB_FALLOFF) { c.err = "both +M and (+M) in " + eq; return false; }
    m->tb[i] = EDYN_TB_M;
  }
  m->A[i] = A;
  m->beta[i] = b;
  m->E_R[i] = E * efac;
  m->dup[i] = 0;
  m->neff[i] = 0;
  return true;
}

bool parse_aux_line(Ctx& c, const std::string& line, double efac) {
  edyn_mech* m = c.m;
  if (m->nreac == 0) { c.err = "auxiliary data before the first reaction: " + line; return false; }
  int i = m->nreac - 1;
  for (auto& kv : aux_items(line)) {
    std::string key = upper(kv.first);
    std::vector<std::string> vals = split_ws(kv.second);
    std::vector<double> v;
    for (auto& s : vals) {
      double d;
      if (!parse_double(s, &d)) { c.err = "bad number '" + s + "' in: " + line; return false; }
      v.push_back(d);
    }
    if (key == "DUP" || key == "DUPLICATE") { m->dup[i] = 1; continue; }
    if (key == "LOW") {
      if (v.size() != 3 || m->tb[i] != EDYN_TB_FALLOFF) { c.err = "bad LOW for " + std::string(m->equation[i]); return false; }
      m->low[i][0] = v[0]; m->low[i][1] = v[1]; m->low[i][2] = v[2] * efac;
      continue;
    }
    if (key == "TROE") {
      if ((v.size() != 3 && v.size() != 4) || m->tb[i] != EDYN_TB_FALLOFF) { c.err = "bad TROE for " + std::string(m->equation[i]); return false; }
      for (size_t q = 0; q < 4; ++q) m->troe[i][q] = q < v.size() ? v[q] : 0.0;
      m->ifop[i] = v.size() == 3 ? EDYN_FO_TROE3 : EDYN_FO_TROE4;
      continue;
    }
    if (key == "SRI" || key == "REV" || key == "LT" || key == "RLT" || key == "PLOG" || key == "FORD" ||
        key == "RORD" || key == "HIGH" || key == "TDEP" || key == "EXCI" || key == "JAN" || key == "FIT1" ||
        key == "HV" || key == "UNITS" || key == "MOME" || key == "XSMI") {
      c.err = "auxiliary keyword " + key + " is not supported";
      return false;
    }
    int k = c.find_species(kv.first);
    if (k < 0) { c.err = "unknown keyword or species '" + kv.first + "'"; return false; }
    if (v.size() != 1) { c.err = "efficiency needs one value: " + line; return false; }
    if (m->tb[i] == EDYN_TB_NONE) { c.err = "efficiency on a reaction without third body: " + std::string(m->equation[i]); return false; }
    if (m->neff[i] >= EDYN_MAX_EFF) { c.err = "too many efficiencies"; return false; }
    m->eff_sp[i][m->neff[i]] = k;
    m->eff_val[i][m->neff[i]] = v[0];
    m->neff[i]++;
  }
  return true;
}

bool read_lines(const std::string& path, std::vector<std::string>& out) {
  std::ifstream f(path);
  if (!f) return false;
  std::string l;
  while (std::getline(f, l)) {
    if (!l.empty() && l.back() == '\r') l.pop_back();
    out.push_back(l);
  }
  return true;
}

}  // namespace

extern "C" int edyn_mech_parse_chemkin(const char* chem_inp, const char* therm_dat, edyn_mech* m, char* err,
                                       int errlen) {
  std::memset(m, 0, sizeof(*m));
  Ctx c{m, ""};
  std::vector<std::string> L;
  auto fail = [&](const std::string& msg) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", msg.c_str());
    return 1;
  };
  if (!read_lines(chem_inp, L)) return fail(std::string("cannot open ") + chem_inp);
  enum { NONE, ELEM, SPEC, REAC } sec = NONE;
  double efac = (double)4.184f / RU_JOUL;
  std::vector<bool> have(EDYN_MAX_SPECIES, false);
  size_t thermo_at = (size_t)-1;
  bool thermo_all = false;
  for (size_t li = 0; li < L.size(); ++li) {
    std::string line = strip_comment(L[li]);
    std::string t = trim(line);
    if (t.empty()) continue;
    auto tk = split_ws(t);
    std::string u0 = upper(tk[0]);
    if (sec != REAC) {
      if (u0.rfind("ELEM", 0) == 0) { sec = ELEM; tk.erase(tk.begin()); }
      else if (u0.rfind("SPEC", 0) == 0) { sec = SPEC; tk.erase(tk.begin()); }
      else if (u0.rfind("THER", 0) == 0) {
        thermo_at = li + 1;
        thermo_all = tk.size() > 1 && upper(tk[1]) == "ALL";
        // skip to END of thermo section
        while (li + 1 < L.size() && upper(trim(strip_comment(L[li + 1]))).rfind("END", 0) != 0) ++li;
        ++li;
        sec = NONE;
        continue;
      } else if (u0.rfind("REAC", 0) == 0) {
        sec = REAC;
        for (size_t q = 1; q < tk.size(); ++q) {
          std::string un = upper(tk[q]);
          if (un.rfind("KCAL", 0) == 0) efac = 4184.0 / RU_JOUL;
          else if (un.rfind("CAL", 0) == 0) efac = (double)4.184f / RU_JOUL;
          else if (un.rfind("KJOU", 0) == 0) efac = 4000.0 / RU_JOUL;  // as the reference interpreter has it
          else if (un.rfind("JOUL", 0) == 0) efac = 1.0 / RU_JOUL;
          else if (un.rfind("KELV", 0) == 0) efac = 1.0;
          else if (un.rfind("MOLE", 0) == 0) {}
          else return fail("unsupported REACTIONS unit keyword " + tk[q]);
        }
        continue;
      }
      if (!tk.empty() && upper(tk[0]) == "END") { sec = NONE; tk.clear(); }
      for (auto& s : tk) {
        if (upper(s) == "END") { sec = NONE; break; }
        if (sec == ELEM) {
          if (m->nelem >= EDYN_MAX_ELEMENTS) return fail("too many elements");
          std::string name = s, wtxt;
          size_t sl = s.find('/');
          if (sl != std::string::npos) {
            name = s.substr(0, sl);
            size_t e2 = s.find('/', sl + 1);
            wtxt = s.substr(sl + 1, e2 == std::string::npos ? std::string::npos : e2 - sl - 1);
          }
          int e = m->nelem++;
          std::snprintf(m->elem_name[e], sizeof(m->elem_name[e]), "%s", upper(name).c_str());
          double w;
          if (!wtxt.empty()) {
            if (!parse_double(wtxt, &w)) return fail("bad element weight " + s);
          } else if (!default_atomic_weight(name, &w)) {
            return fail("no atomic weight for element " + name);
          }
          m->elem_weight[e] = w;
        } else if (sec == SPEC) {
          if (m->nspec >= EDYN_MAX_SPECIES) return fail("too many species");
          if (c.find_species(s) >= 0) continue;
          std::snprintf(m->spec_name[m->nspec++], EDYN_NAME_LEN, "%s", s.c_str());
        }
      }
      continue;
    }
    // REACTIONS section
    if (u0 == "END") { sec = NONE; continue; }
    if (t.find('=') != std::string::npos) {
      if (!parse_reaction_line(c, t, efac)) return fail(c.err);
    } else {
      if (!parse_aux_line(c, t, efac)) return fail(c.err);
    }
  }
  (void)thermo_all;
  if (thermo_at != (size_t)-1) {
    if (!read_thermo(c, L, thermo_at, have)) return fail(c.err);
  }
  bool missing = false;
  for (int k = 0; k < m->nspec; ++k) missing |= !have[k];
  if (missing && therm_dat && therm_dat[0]) {
    std::vector<std::string> T;
    if (!read_lines(therm_dat, T)) return fail(std::string("cannot open ") + therm_dat);
    size_t s0 = 0;
    while (s0 < T.size() && upper(trim(strip_comment(T[s0]))).rfind("THER", 0) != 0) ++s0;
    if (s0 < T.size()) ++s0; else s0 = 0;
    if (!read_thermo(c, T, s0, have)) return fail(c.err);
  }
  for (int k = 0; k < m->nspec; ++k)
    if (!have[k]) return fail(std::string("no thermo data for species ") + m->spec_name[k]);
  for (int i = 0; i < m->nreac; ++i) {
    if (m->tb[i] == EDYN_TB_FALLOFF && m->low[i][0] == 0.0) return fail(std::string("fall-off reaction without LOW: ") + m->equation[i]);
    // element balance
    for (int e = 0; e < m->nelem; ++e) {
      long bal = 0;
      for (int q = 0; q < 6; ++q)
        if (m->nunk[i][q] >= 0) bal += (long)m->nu[i][q] * m->elem_count[m->nunk[i][q]][e];
      if (bal != 0) return fail(std::string("element imbalance in ") + m->equation[i]);
    }
  }
  return 0;
}

extern "C" int edyn_mech_write(const edyn_mech* m, const char* path) {
  FILE* f = std::fopen(path, "w");
  if (!f) return 1;
  std::fprintf(f, "EDYNMECH 1\nELEMENTS %d\n", m->nelem);
  for (int e = 0; e < m->nelem; ++e) std::fprintf(f, "%s %.17g\n", m->elem_name[e], m->elem_weight[e]);
  std::fprintf(f, "SPECIES %d\n", m->nspec);
  for (int k = 0; k < m->nspec; ++k) {
    std::fprintf(f, "%s %.17g %.17g %.17g %.17g", m->spec_name[k], m->W[k], m->T_lo[k], m->T_mid[k], m->T_hi[k]);
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 7; ++j) std::fprintf(f, " %.17g", m->a[k][r][j]);
    for (int e = 0; e < m->nelem; ++e) std::fprintf(f, " %d", m->elem_count[k][e]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "REACTIONS %d\n", m->nreac);
  for (int i = 0; i < m->nreac; ++i) {
    std::fprintf(f, "%s %d", m->equation[i], m->rev[i]);
    for (int q = 0; q < 6; ++q) std::fprintf(f, " %d %d", m->nunk[i][q], m->nu[i][q]);
    std::fprintf(f, " %.17g %.17g %.17g %d %d %d", m->A[i], m->beta[i], m->E_R[i], m->tb[i], m->kfal[i], m->ifop[i]);
    for (int q = 0; q < 3; ++q) std::fprintf(f, " %.17g", m->low[i][q]);
    for (int q = 0; q < 4; ++q) std::fprintf(f, " %.17g", m->troe[i][q]);
    std::fprintf(f, " %d %d", m->dup[i], m->neff[i]);
    for (int q = 0; q < m->neff[i]; ++q) std::fprintf(f, " %d %.17g", m->eff_sp[i][q], m->eff_val[i][q]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "END\n");
  return std::fclose(f) != 0;
}

extern "C" int edyn_mech_read(const char* path, edyn_mech* m, char* err, int errlen) {
  std::memset(m, 0, sizeof(*m));
  std::ifstream f(path);
  auto fail = [&](const std::string& msg) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s: %s", path, msg.c_str());
    return 1;
  };
  if (!f) return fail("cannot open");
  std::string tag;
  int ver = 0;
  f >> tag >> ver;
  if (tag != "EDYNMECH" || ver != 1) return fail("not an EDYNMECH 1 file");
  f >> tag >> m->nelem;
  if (tag != "ELEMENTS" || m->nelem < 0 || m->nelem > EDYN_MAX_ELEMENTS) return fail("bad ELEMENTS");
  for (int e = 0; e < m->nelem; ++e) {
    std::string n;
    f >> n >> m->elem_weight[e];
    std::snprintf(m->elem_name[e], sizeof(m->elem_name[e]), "%s", n.c_str());
  }
  f >> tag >> m->nspec;
  if (tag != "SPECIES" || m->nspec <= 0 || m->nspec > EDYN_MAX_SPECIES) return fail("bad SPECIES");
  for (int k = 0; k < m->nspec; ++k) {
    std::string n;
    f >> n >> m->W[k] >> m->T_lo[k] >> m->T_mid[k] >> m->T_hi[k];
    std::snprintf(m->spec_name[k], EDYN_NAME_LEN, "%s", n.c_str());
    for (int r = 0; r < 2; ++r)
      for (int j = 0; j < 7; ++j) f >> m->a[k][r][j];
    for (int e = 0; e < m->nelem; ++e) f >> m->elem_count[k][e];
  }
  f >> tag >> m->nreac;
  if (tag != "REACTIONS" || m->nreac < 0 || m->nreac > EDYN_MAX_REACTIONS) return fail("bad REACTIONS");
  for (int i = 0; i < m->nreac; ++i) {
    std::string eq;
    f >> eq >> m->rev[i];
    std::snprintf(m->equation[i], sizeof(m->equation[i]), "%s", eq.c_str());
    for (int q = 0; q < 6; ++q) f >> m->nunk[i][q] >> m->nu[i][q];
    f >> m->A[i] >> m->beta[i] >> m->E_R[i] >> m->tb[i] >> m->kfal[i] >> m->ifop[i];
    for (int q = 0; q < 3; ++q) f >> m->low[i][q];
    for (int q = 0; q < 4; ++q) f >> m->troe[i][q];
    f >> m->dup[i] >> m->neff[i];
    if (m->neff[i] < 0 || m->neff[i] > EDYN_MAX_EFF) return fail("bad efficiency count");
    for (int q = 0; q < m->neff[i]; ++q) f >> m->eff_sp[i][q] >> m->eff_val[i][q];
    for (int q = 0; q < 6; ++q)
      if (m->nunk[i][q] < -1 || m->nunk[i][q] >= m->nspec) return fail("species index out of range");
  }
  f >> tag;
  if (!f || tag != "END") return fail("truncated file");
  return 0;
}

extern "C" int edyn_mech_load_dir(const char* dir, edyn_mech* m, char* err, int errlen) {
  std::string d(dir ? dir : ".");
  std::string chem = d + "/chem.inp", therm = d + "/therm.dat", edyn = d + "/mech.edyn";
  if (std::ifstream(chem)) return edyn_mech_parse_chemkin(chem.c_str(), therm.c_str(), m, err, errlen);
  if (std::ifstream(edyn)) return edyn_mech_read(edyn.c_str(), m, err, errlen);
  if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s holds neither chem.inp nor mech.edyn", d.c_str());
  return 1;
}
