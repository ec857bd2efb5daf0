// A LAMMPS-free stand-in for the caller of the drop-in ABI: it does what the
// reference's pair style does around acelib_ (lammps/pair_spin_ace.cpp:340-646)
// for one periodic orthorhombic box, so that the library can be exercised by
// a C++ program exactly as an MD code would use it.
//
//   * local atoms plus ghost images within rcut + skin of the box (the atoms a
//     LAMMPS rank holds), spins stored as sp[i] = (m_hat, |m|);
//   * a full neighbour list with skin: every local i lists every atom or
//     ghost j closer than rcut + skin (bonds beyond rcut contribute zero,
//     src/radial.F90:77-83);
//   * the flat 1-based arrays of acelibini_/acelib_ (pair_spin_ace.cpp:446-543),
//     with acelibini_ reading ./<El>.<xc>.in;
//   * the reductions of pair_spin_ace.cpp:571-646 with newton_pair on:
//     f_i -= f_ij, f_j += f_ij, fm_j -= t_ij, fm_i -= t0_i, the virial
//     v += (x_i - x_j) f_ij per bond, E = sum_i E_i; then the ghosts' forces
//     and fields are added to their owners (LAMMPS reverse communication).
//
// Input (stdin, whitespace separated): natom, the three box lengths (A),
// rcut, skin, rcut_magnetic, smear, then per atom x y z mx my mz (moment in
// mu_B). Output (stdout): "energy E", "virial v0..v5" (xx yy zz xy xz yz),
// then per atom "f fx fy fz fmx fmy fmz". Exit code 0, or 1 on any error
// the library reports.
#include <cmath>
#include <cstdio>
#include <vector>

extern "C" {
void acelibini_(int* nele, double* rcut, double* rcut_magnetic, double* smear, int* xcnumber, int* elenumbers);
void acelib_(int* natom, int* nall, int* nei, int* nlist, int* occ, int* occlist, int* nstart, int* nstop,
             double* eout, double* dlist, double* elist, double* flist, double* dlist_momi, double* elist_momi,
             double* dlist_mom, double* elist_mom, double* tlist, double* tlist0);
int ace_last_error(void);
const char* ace_last_error_message(void);
}

int main() {
  int nlocal = 0;
  double box[3], rcut, skin, rcut_mag, smear;
  if (std::scanf("%d %lf %lf %lf %lf %lf %lf %lf", &nlocal, &box[0], &box[1], &box[2], &rcut, &skin, &rcut_mag,
                 &smear) != 8 || nlocal <= 0)
    return 1;
  // x[nall][3], sp[nall][4] = (direction, magnitude), owner[nall]
  std::vector<double> x, sp;
  std::vector<int> owner;
  for (int i = 0; i < nlocal; ++i) {
    double p[3], m[3];
    if (std::scanf("%lf %lf %lf %lf %lf %lf", &p[0], &p[1], &p[2], &m[0], &m[1], &m[2]) != 6) return 1;
    const double mag = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    for (int c = 0; c < 3; ++c) x.push_back(p[c]);
    for (int c = 0; c < 3; ++c) sp.push_back(mag > 0.0 ? m[c] / mag : (c == 2 ? 1.0 : 0.0));
    sp.push_back(mag);
    owner.push_back(i);
  }
  // ghost images within rcut + skin of the box
  const double rl = rcut + skin;
  int reach[3];
  for (int c = 0; c < 3; ++c) reach[c] = static_cast<int>(std::ceil(rl / box[c]));
  for (int a = -reach[0]; a <= reach[0]; ++a)
    for (int b = -reach[1]; b <= reach[1]; ++b)
      for (int d = -reach[2]; d <= reach[2]; ++d) {
        if (a == 0 && b == 0 && d == 0) continue;
        const double s[3] = {a * box[0], b * box[1], d * box[2]};
        for (int i = 0; i < nlocal; ++i) {
          double p[3];
          bool near = true;
          for (int c = 0; c < 3; ++c) {
            p[c] = x[3 * i + c] + s[c];
            if (p[c] < -rl || p[c] > box[c] + rl) near = false;
          }
          if (!near) continue;
          for (int c = 0; c < 3; ++c) x.push_back(p[c]);
          for (int c = 0; c < 4; ++c) sp.push_back(sp[4 * i + c]);
          owner.push_back(i);
        }
      }
  const int nall = static_cast<int>(owner.size());
  // full neighbour list with skin, per local atom
  std::vector<std::vector<int>> neigh(nlocal);
  for (int i = 0; i < nlocal; ++i)
    for (int j = 0; j < nall; ++j) {
      if (j == i) continue;
      double r2 = 0.0;
      for (int c = 0; c < 3; ++c) r2 += (x[3 * i + c] - x[3 * j + c]) * (x[3 * i + c] - x[3 * j + c]);
      if (r2 < rl * rl) neigh[i].push_back(j);
    }
  // the potential, as the pair style's init_one does it: one element, Fe = 26 + 1
  int nele = 1, xc = 1, el[1] = {27};
  acelibini_(&nele, &rcut, &rcut_mag, &smear, &xc, el);
  if (ace_last_error() != 0) {
    std::fprintf(stderr, "acelibini_: %s\n", ace_last_error_message());
    return 1;
  }
  // the flat arrays (0-based while filled, then shifted to Fortran's 1-based)
  int nei = 0;
  for (int i = 0; i < nlocal; ++i) nei += static_cast<int>(neigh[i].size());
  std::vector<int> nlist(nei), occ(nlocal), occlist(nei), nstart(nlocal), nstop(nlocal);
  std::vector<double> dlist(nei), elist(3 * nei), dlist_mom(nei), elist_mom(3 * nei);
  std::vector<double> dlist_momi(nlocal), elist_momi(3 * nlocal);
  std::vector<double> eout(nlocal), flist(3 * nei), tlist(3 * nei), tlist0(3 * nlocal);
  int k = 0;
  for (int i = 0; i < nlocal; ++i) {
    occ[i] = 0;
    nstart[i] = k;
    dlist_momi[i] = sp[4 * i + 3];
    for (int c = 0; c < 3; ++c) elist_momi[3 * i + c] = sp[4 * i + c];
    for (int j : neigh[i]) {
      nlist[k] = j;
      occlist[k] = 0;
      double del[3], r2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        del[c] = x[3 * i + c] - x[3 * j + c];
        r2 += del[c] * del[c];
      }
      const double r = std::sqrt(r2);
      dlist[k] = r;
      for (int c = 0; c < 3; ++c) elist[3 * k + c] = del[c] / r;
      dlist_mom[k] = sp[4 * j + 3];
      for (int c = 0; c < 3; ++c) elist_mom[3 * k + c] = sp[4 * j + c];
      ++k;
    }
    nstop[i] = k - 1;
  }
  for (int b = 0; b < nei; ++b) {
    ++nlist[b];
    ++occlist[b];
  }
  for (int i = 0; i < nlocal; ++i) {
    ++nstart[i];
    ++nstop[i];
    ++occ[i];
  }
  int natom = nlocal, nall_arg = nall;
  acelib_(&natom, &nall_arg, &nei, nlist.data(), occ.data(), occlist.data(), nstart.data(), nstop.data(),
          eout.data(), dlist.data(), elist.data(), flist.data(), dlist_momi.data(), elist_momi.data(),
          dlist_mom.data(), elist_mom.data(), tlist.data(), tlist0.data());
  if (ace_last_error() != 0) {
    std::fprintf(stderr, "acelib_: %s\n", ace_last_error_message());
    return 1;
  }
  // reductions with newton_pair on, then ghosts to their owners
  std::vector<double> f(3 * nall, 0.0), fm(3 * nall, 0.0);
  double virial[6] = {0, 0, 0, 0, 0, 0}, energy = 0.0;
  k = 0;
  for (int i = 0; i < nlocal; ++i) {
    for (int c = 0; c < 3; ++c) fm[3 * i + c] -= tlist0[3 * i + c];
    for (int j : neigh[i]) {
      double del[3];
      for (int c = 0; c < 3; ++c) del[c] = x[3 * i + c] - x[3 * j + c];
      const double* fij = &flist[3 * k];
      const double* tij = &tlist[3 * k];
      for (int c = 0; c < 3; ++c) {
        f[3 * i + c] -= fij[c];
        f[3 * j + c] += fij[c];
        fm[3 * j + c] -= tij[c];
      }
      virial[0] += del[0] * fij[0];
      virial[1] += del[1] * fij[1];
      virial[2] += del[2] * fij[2];
      virial[3] += del[0] * fij[1];
      virial[4] += del[0] * fij[2];
      virial[5] += del[1] * fij[2];
      ++k;
    }
    energy += eout[i];
  }
  for (int g = nlocal; g < nall; ++g)
    for (int c = 0; c < 3; ++c) {
      f[3 * owner[g] + c] += f[3 * g + c];
      fm[3 * owner[g] + c] += fm[3 * g + c];
    }
  std::printf("energy %.17g\n", energy);
  std::printf("virial %.17g %.17g %.17g %.17g %.17g %.17g\n", virial[0], virial[1], virial[2], virial[3], virial[4],
              virial[5]);
  for (int i = 0; i < nlocal; ++i)
    std::printf("f %.17g %.17g %.17g %.17g %.17g %.17g\n", f[3 * i], f[3 * i + 1], f[3 * i + 2], fm[3 * i],
                fm[3 * i + 1], fm[3 * i + 2]);
  return 0;
}
