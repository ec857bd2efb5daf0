// Potential file model: the mag-ace "<Elements>.<xc>.in" parameter format.
//
// The format is the reference's (read by rwpara, src/util.F90:459-1108): a
// fixed header (creation stamp, element list, XC functional, Gaussian
// smearing, lambda, cutoffs, basis dimensions, ndensity, npot/nfemb/radtype)
// followed by typed records, each a header line "<type> <order> <density>"
// and one data line: 'clu' (expansion coefficient of one cluster), 'par'
// (embedding parameters), 'core' (hard-core repulsion), 'rad_atomic' and
// 'rad_magnetic' (radial contraction coefficients).
#pragma once

#include <array>
#include <map>
#include <string>
#include <vector>

namespace magace {

struct BasisDims {
  int nradbase_a = 0, nradbase_m = 0, nradial2_m = 0, l2max_m = 0;
  int nradial3_a = 0, nradial3_m = 0, l3max_a = 0, l3max_m = 0;
  int nradial4_a = 0, nradial4_m = 0, l4max_a = 0, l4max_m = 0;
  int nradial5_a = 0, nradial5_m = 0, l5max_a = 0, l5max_m = 0;
  int nradial6_a = 0, nradial6_m = 0, l6max_a = 0, l6max_m = 0;
  int ndensity = 0, npot = 0, nfemb = 0, radtype_a = 0, radtype_m = 0;
};

// A cluster record key: the integer index tuple of one 'clu' data line
// (rank 1: n0'; rank 2: n0',n1',n1,l0'; rank 3: 9 ints; rank 4: 15 ints;
// rank 5: 21 ints; rank 6: 27 ints).
typedef std::vector<int> ClusterKey;

struct Potential {
  std::string element;
  std::string xc;
  double smearing = 0;
  double lambda[2] = {0, 0};  // atomic, magnetic radial scaling
  double cut[2] = {0, 0};     // atomic cutoff (A), magnetic cutoff (mu_B)
  double dcut[2] = {0, 0};    // taper widths
  double ecut = 0, decut = 0; // inner (core-energy) cutoff
  BasisDims dims;

  // radial contraction crad[l][nr][n] (defaults: identity), see setup
  std::vector<double> crad_a, crad_m;
  double core_pre = 3.0, core_lambda = 3.0;  // defaults of src/util.F90:314
  double par[2][2] = {{1.0, 1.0}, {1.0, 1.0}};  // par[order-1][density-1]

  // cluster coefficients as read: rank -> key -> per-density value
  std::map<ClusterKey, std::array<double, 2>> clusters[7];
  int records_read = 0;
};

// Parses `path`. Checks the element and XC against the caller's and the
// smearing to 1e-6 (src/util.F90:580-597). Returns 0 or a MAGACE_ERR_* code
// and fills `msg`.
int read_potential(const std::string& path, const std::string& element, const std::string& xc,
                   double smearing, Potential& pot, std::string& msg);

}  // namespace magace
