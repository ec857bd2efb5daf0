// CPU FP64 oracle for the mag-ace potential-evaluation path.
//
// TEST INFRASTRUCTURE ONLY: this code is the parity checker. Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it. The
// product path (mag-ace_gb300/) never links or calls it.
//
// It restates the reference Fortran (mttrin93/mag-ace, src/*.F90) operation for
// operation: module-global state (src/modules.F90) becomes the OracleState
// struct, and every array keeps its Fortran bounds through FArr. Only a single
// chemical element is supported, as in the reference C-ABI (src/ace.F90:46-49).
// Ranks 5 and 6 (5- and 6-body clusters) are not restated; a potential file
// that enables them is rejected at init.
#pragma once

#include <complex>
#include <string>

#include "farr.h"

typedef std::complex<double> cplx;

enum OracleStatus {
  ORACLE_OK = 0,
  ORACLE_ERR_FILE = 1,        // potential file missing or unreadable
  ORACLE_ERR_FORMAT = 2,      // malformed or inconsistent potential file
  ORACLE_ERR_UNSUPPORTED = 3, // nele != 1, ranks 5/6, unknown radtype/nfemb
  ORACLE_ERR_SMALL_R = 4,     // bond length below one LUT bin (src/radial.F90:71-75)
  ORACLE_ERR_MOMENT = 5,      // negative or over-cutoff moment magnitude (src/radial.F90:129-133)
  ORACLE_ERR_NOT_INIT = 6,
  ORACLE_ERR_ARGS = 7,
};

struct OracleState {
  bool initialized = false;
  std::string element;
  std::string xc;
  // acelibini arguments (src/ace.F90:41-44)
  double cutoff = 0, cutoff_magnetic = 0, smearing = 0;

  // per-pair radial settings, single element (src/util.F90:608-611)
  double lambda[2] = {0, 0}, cut[2] = {0, 0}, dcut[2] = {0, 0};
  double ecut = 0, decut = 0;

  // header dims (src/util.F90:646-652, 198-231)
  int nradbase_atomic = 0, nradbase_magnetic = 0, nradial2_magnetic = 0, l2max_magnetic = 0;
  int nradial3_atomic = 0, nradial3_magnetic = 0, l3max_atomic = 0, l3max_magnetic = 0;
  int nradial4_atomic = 0, nradial4_magnetic = 0, l4max_atomic = 0, l4max_magnetic = 0;
  int nradial5_atomic = 0, nradial5_magnetic = 0, l5max_atomic = 0, l5max_magnetic = 0;
  int nradial6_atomic = 0, nradial6_magnetic = 0, l6max_atomic = 0, l6max_magnetic = 0;
  int ndensity = 0, npot = 0, nfemb = 0, radtype_atomic = 0, radtype_magnetic = 0;
  int nradbase = 0, nradial = 0, lmax = 0;

  // spherical-harmonic packing (src/util.F90:1676-1776)
  int lmaxsq_atomic = 0, lmaxhalf_atomic = 0, lmaxsq_magnetic = 0, lmaxhalf_magnetic = 0;
  FArr<int> shindex_atomic, shindex_magnetic, shback_atomic, shback_magnetic;

  // Clebsch-Gordan tables (src/util.F90:4149-4252)
  FArr<double> fac, cgcoeff;

  // basis enumeration (src/util.F90:1803-2814)
  int nvar1 = 0, nvar2 = 0, nvar3 = 0, nvar4 = 0;
  int nvar2l = 0, nvar3l_atomic = 0, nvar3l_magnetic = 0, nvar4l_atomic = 0, nvar4l_magnetic = 0;
  FArr<int> b1occ, b1index;
  FArr<int> b2lindex, b2occ, b2index, b2map, madd2, b2lm;
  FArr<int> b3lindex_atomic, b3lindex_magnetic, b3occ, b3index, b3map_atomic, b3map_magnetic;
  FArr<int> madd3_atomic, madd3_magnetic, b3lm_atomic, b3lm_magnetic;
  FArr<int> b4lindex_atomic, b4occ, b4index, b4nint, b4map_atomic, b4map_magnetic;
  FArr<int> b4lindex_magnetic, madd4_atomic, madd4_magnetic, b4lm_atomic, b4lm_magnetic;

  // 5- and 6-body clusters (src/util.F90:2817-3760): the index rows of the
  // 'clu' records (b5index 21 ints, b6index 27 ints), and per cluster the
  // m-terms of its atomic and of its magnetic part with their generalized
  // couplings (cg04/cg05, src/util.F90:4389-4546). The reference shares
  // these lists between the clusters of one angular part (b5map, b5lm,
  // madd5); each cluster holds its own copy here. A cluster whose atomic or
  // magnetic half the enumeration padded with zeros has empty lists.
  struct MTerm {
    int m[6];
    double cf;
  };
  int nvar5 = 0, nvar6 = 0;
  FArr<int> b5index, b6index;
  std::vector<std::vector<MTerm>> b5mt_atomic, b5mt_magnetic, b6mt_atomic, b6mt_magnetic;

  // generalized couplings (src/util.F90:4256-4388)
  FArr<double> cg01_magnetic, cg02_atomic, cg02_magnetic, cg03_atomic, cg03_magnetic;

  // expansion coefficients and radial parameters (src/util.F90:281-350, 667-1106)
  FArr<double> crad_atomic, crad_magnetic, corepara, p1;
  FArr<double> c0, c2, c3, c4, c5, c6;

  // lookup tables (src/radial.F90:164-426)
  int nlut = 0;
  double rscalelookup_atomic = 0, invrscalelookup_atomic = 0;
  double rscalelookup_magnetic = 0, invrscalelookup_magnetic = 0;
  FArr<double> lutfrs_atomic, lutgrs_atomic, luthcrs_atomic;
  FArr<double> lutfrs_magnetic, lutgrs_magnetic;

  // spherical-harmonic recurrence constants (src/spherical.F90:5-51)
  FArr<double> alm_atomic, blm_atomic, alm_magnetic, blm_magnetic, cl, dl;
};

// Setup: reads "<path>" (the reference reads "<El>.<xc>.in" from the working
// directory, src/util.F90:525) and builds every table.
int oracle_setup(OracleState& s, const char* path, const char* element, double rcut,
                 double rcut_magnetic, double smear, int xcnumber, std::string& err);
