// Reader for the "<Elements>.<xc>.in" potential format.
//
// Fortran list-directed semantics (the reference reads each record with
// read(1,*), src/util.F90:550-1106): every read begins on a new line,
// consumes lines until it has its items, and discards the remainder of its
// last line. Items are separated by blanks or commas.
#include "potential.hpp"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>

#include "magace.h"

namespace magace {
namespace {

class Records {
 public:
  explicit Records(std::ifstream& f) : f_(f) {}

  // Next `n` items; false at end of file.
  bool take(size_t n, std::vector<std::string>& items) {
    items.clear();
    std::string line;
    while (items.size() < n) {
      if (!std::getline(f_, line)) return false;
      tokenize(line, items);
    }
    items.resize(n);
    return true;
  }
  bool skip_line() {
    std::string line;
    return static_cast<bool>(std::getline(f_, line));
  }

 private:
  static void tokenize(const std::string& s, std::vector<std::string>& out) {
    std::string cur;
    bool quoted = false;
    char q = 0;
    for (size_t i = 0; i <= s.size(); ++i) {
      char c = i < s.size() ? s[i] : ' ';
      if (quoted) {
        if (c == q) {
          quoted = false;
          out.push_back(cur);
          cur.clear();
        } else {
          cur += c;
        }
        continue;
      }
      if (c == '\'' || c == '"') {
        quoted = true;
        q = c;
        continue;
      }
      if (c == '/' && cur.empty()) return;  // list terminator
      if (std::isspace(static_cast<unsigned char>(c)) || c == ',') {
        if (!cur.empty()) out.push_back(cur);
        cur.clear();
      } else {
        cur += c;
      }
    }
  }
  std::ifstream& f_;
};

bool as_int(const std::string& s, int& v) {
  char* e = nullptr;
  long x = std::strtol(s.c_str(), &e, 10);
  if (e == s.c_str() || *e) return false;
  v = static_cast<int>(x);
  return true;
}

bool as_real(std::string s, double& v) {
  for (char& c : s)
    if (c == 'd' || c == 'D') c = 'e';  // Fortran double exponent
  char* e = nullptr;
  v = std::strtod(s.c_str(), &e);
  return !(e == s.c_str() || *e);
}

}  // namespace

int read_potential(const std::string& path, const std::string& element, const std::string& xc,
                   double smearing, Potential& pot, std::string& msg) {
  pot = Potential();
  pot.element = element;
  pot.xc = xc;
  std::ifstream f(path);
  if (!f) {
    msg = "potential file not found: " + path;
    return MAGACE_ERR_FILE;
  }
  Records rec(f);
  std::vector<std::string> it;
  auto fail = [&](const std::string& what) {
    msg = "malformed potential file " + path + ": " + what;
    return MAGACE_ERR_FORMAT;
  };

  if (!rec.skip_line()) return fail("empty file");
  if (!rec.take(7, it)) return fail("missing creation line");
  if (!rec.take(2, it)) return fail("missing element line");
  if (it[1] != element) {
    msg = "inconsistent element information in " + path;
    return MAGACE_ERR_FORMAT;
  }
  if (!rec.take(2, it)) return fail("missing XC line");
  if (it[1] != xc) {
    msg = "inconsistent XC functional in " + path;
    return MAGACE_ERR_FORMAT;
  }
  if (!rec.take(2, it) || !as_real(it[1], pot.smearing)) return fail("bad gauss-smearing line");
  if (std::fabs(pot.smearing - smearing) > 1e-6) {
    msg = "inconsistent gauss-smearing in " + path;
    return MAGACE_ERR_FORMAT;
  }
  if (!rec.take(3, it) || !as_real(it[1], pot.lambda[0]) || !as_real(it[2], pot.lambda[1]))
    return fail("bad lambda line");
  if (!rec.take(10, it)) return fail("bad cutoff line");
  double* cv[6] = {&pot.cut[0], &pot.cut[1], &pot.dcut[0], &pot.dcut[1], &pot.ecut, &pot.decut};
  for (int q = 0; q < 6; ++q)
    if (!as_real(it[4 + q], *cv[q])) return fail("bad cutoff value");
  BasisDims& d = pot.dims;
  int* rows[5][4] = {{&d.nradbase_a, &d.nradbase_m, &d.nradial2_m, &d.l2max_m},
                     {&d.nradial3_a, &d.nradial3_m, &d.l3max_a, &d.l3max_m},
                     {&d.nradial4_a, &d.nradial4_m, &d.l4max_a, &d.l4max_m},
                     {&d.nradial5_a, &d.nradial5_m, &d.l5max_a, &d.l5max_m},
                     {&d.nradial6_a, &d.nradial6_m, &d.l6max_a, &d.l6max_m}};
  for (auto& row : rows) {
    if (!rec.take(6, it)) return fail("bad basis dimension line");
    for (int q = 0; q < 4; ++q)
      if (!as_int(it[2 + q], *row[q])) return fail("bad basis dimension");
  }
  if (!rec.take(2, it) || !as_int(it[1], d.ndensity)) return fail("bad ndensity line");
  if (!rec.take(5, it) || !as_int(it[1], d.npot) || !as_int(it[2], d.nfemb) ||
      !as_int(it[3], d.radtype_a) || !as_int(it[4], d.radtype_m))
    return fail("bad npot-nfemb-radtype line");
  if (d.ndensity < 1 || d.ndensity > 2) {
    msg = "ndensity must be 1 or 2";
    return MAGACE_ERR_UNSUPPORTED;
  }
  if (d.nradbase_a < 1 || d.nradbase_m < 1 || d.nradial2_m < 0 || d.l2max_m < 0 ||
      d.nradial3_a < 0 || d.nradial3_m < 0 || d.l3max_a < 0 || d.l3max_m < 0 ||
      d.nradial4_a < 0 || d.nradial4_m < 0 || d.l4max_a < 0 || d.l4max_m < 0)
    return fail("negative or zero basis dimension");

  // default radial contraction: identity on the first nradial functions
  // (src/util.F90:282-302)
  const int la = d.l3max_a + 1, lm = d.l2max_m + 1;
  pot.crad_a.assign(static_cast<size_t>(la) * d.nradial3_a * d.nradbase_a, 0.0);
  pot.crad_m.assign(static_cast<size_t>(lm) * d.nradial2_m * d.nradbase_m, 0.0);
  auto ca = [&](int n, int nr, int l) -> double& {
    return pot.crad_a[(static_cast<size_t>(l) * d.nradial3_a + (nr - 1)) * d.nradbase_a + (n - 1)];
  };
  auto cm = [&](int n, int nr, int l) -> double& {
    return pot.crad_m[(static_cast<size_t>(l) * d.nradial2_m + (nr - 1)) * d.nradbase_m + (n - 1)];
  };
  for (int l = 0; l < la; ++l)
    for (int nr = 1; nr <= d.nradial3_a; ++nr) ca(nr, nr, l) = 1.0;
  for (int l = 0; l < lm; ++l)
    for (int nr = 1; nr <= d.nradial2_m; ++nr) cm(nr, nr, l) = 1.0;

  // typed records (src/util.F90:669-1106)
  const size_t width[7] = {0, 1, 4, 9, 15, 21, 27};
  while (rec.take(3, it)) {
    const std::string type = it[0];
    int order = 0, dens = 0;
    if (!as_int(it[1], order) || !as_int(it[2], dens)) return fail("bad record header '" + type + "'");
    ++pot.records_read;
    if (type == "clu") {
      if (order < 1 || order > 6) return fail("cluster order out of range");
      const size_t nitem = order + width[order] + 2;
      if (!rec.take(nitem, it)) break;
      for (int q = 0; q < order; ++q)
        if (it[q] != element) {
          msg = "cluster record with an element other than " + element;
          return MAGACE_ERR_FORMAT;
        }
      ClusterKey key(width[order]);
      for (size_t q = 0; q < width[order]; ++q)
        if (!as_int(it[order + q], key[q])) return fail("bad cluster index");
      double val;
      if (!as_real(it[order + width[order]], val)) return fail("bad cluster value");
      if (dens >= 1 && dens <= d.ndensity) {
        auto& slot = pot.clusters[order][key];
        slot[dens - 1] = val;
      }
    } else if (type == "par") {
      if (order < 1 || order > 2) return fail("par order must be 1 or 2");
      if (!rec.take(3, it)) break;
      double val;
      if (!as_real(it[1], val)) return fail("bad par value");
      if (it[0] == element && dens >= 1 && dens <= d.ndensity) pot.par[order - 1][dens - 1] = val;
    } else if (type == "core") {
      if (order < 1 || order > 2) return fail("core order must be 1 or 2");
      if (!rec.take(4, it)) break;
      double val;
      if (!as_real(it[2], val)) return fail("bad core value");
      if (it[0] != element || it[1] != element) return fail("core record for another element pair");
      (order == 1 ? pot.core_pre : pot.core_lambda) = val;
    } else if (type == "rad_atomic" || type == "rad_magnetic") {
      if (!rec.take(7, it)) break;
      int n, nr, l;
      double val;
      if (!as_int(it[2], n) || !as_int(it[3], nr) || !as_int(it[4], l) || !as_real(it[5], val))
        return fail("bad radial record");
      if (it[0] != element || it[1] != element) return fail("radial record for another element pair");
      if (type == "rad_atomic") {
        if (n >= 1 && n <= d.nradbase_a && nr >= 1 && nr <= d.nradial3_a && l >= 0 && l <= d.l3max_a)
          ca(n, nr, l) = val;
      } else {
        if (n >= 1 && n <= d.nradbase_m && nr >= 1 && nr <= d.nradial2_m && l >= 0 && l <= d.l2max_m)
          cm(n, nr, l) = val;
      }
    }
    // any other record type is ignored, as in the reference
  }
  return MAGACE_OK;
}

}  // namespace magace
