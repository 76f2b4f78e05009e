// fb_fdata.cpp -- host reader of FIREBALL Fdata (libfbgpu).
//
// Parses the text files read by read_info (c.SYSTEM/M_species.f90:1057-1251),
// read_Fdata_2c (e.FDATA/M_Fdata_2c.f90:149-272) and read_Fdata_3c
// (e.FDATA/M_Fdata_3c.f90:143-264) with Fortran list-directed semantics:
// every READ starts on a new record, may continue over records until its
// item list is satisfied, and discards the rest of its last record.  A munu
// unit that is re-opened on the file it already has open keeps its position
// (the reference re-opens it once per cell), so a 3c munu file holds one
// (mu, nu, mvalue) triple of records per theta cell.
//
// The tables are then repacked for the GPU: 2c values point-major (all MEs of
// a grid point contiguous), 3c values node-major with the five theta terms
// and all MEs of a grid node contiguous, and the gradient switch of
// getMEs_Fdata_3c (M_Fdata_3c.f90:383-385) precomputed per node.  This file
// is compiled with -ffp-contract=off so that switch is decided exactly as in
// the reference.
#include "fb_fdata.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "../../include/fbgpu.h"

namespace fb {

namespace {

struct Text {
  std::vector<std::string> rec;
  size_t pos = 0;
  bool load(const std::string &path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    rec.clear();
    while (std::getline(f, line)) {
      if (!line.empty() && line.back() == '\r') line.pop_back();
      rec.push_back(line);
    }
    pos = 0;
    return true;
  }
  // one list-directed READ of n items
  bool read(size_t n, std::vector<std::string> &out) {
    out.clear();
    while (out.size() < n) {
      if (pos >= rec.size()) return false;
      const std::string &r = rec[pos++];
      size_t i = 0;
      while (i < r.size() && out.size() < n) {
        while (i < r.size() && (r[i] == ' ' || r[i] == '\t' || r[i] == ',')) i++;
        if (i >= r.size()) break;
        size_t j = i;
        while (j < r.size() && r[j] != ' ' && r[j] != '\t' && r[j] != ',') j++;
        out.push_back(r.substr(i, j - i));
        i = j;
      }
    }
    return true;
  }
  bool skip() {
    if (pos >= rec.size()) return false;
    pos++;
    return true;
  }
  bool line(std::string &s) {
    if (pos >= rec.size()) return false;
    s = rec[pos++];
    return true;
  }
};

double to_d(const std::string &t) {
  std::string s = t;
  for (char &ch : s)
    if (ch == 'D' || ch == 'd') ch = 'E';
  return std::strtod(s.c_str(), nullptr);
}

bool read_ints(Text &t, size_t n, int *v) {
  std::vector<std::string> tok;
  if (!t.read(n, tok)) return false;
  for (size_t k = 0; k < n; k++) v[k] = std::atoi(tok[k].c_str());
  return true;
}
bool read_dbls(Text &t, size_t n, double *v) {
  std::vector<std::string> tok;
  if (!t.read(n, tok)) return false;
  for (size_t k = 0; k < n; k++) v[k] = to_d(tok[k]);
  return true;
}

std::string zz(int a) {
  char b[8];
  std::snprintf(b, sizeof b, "%02d", a);
  return b;
}

struct Cell2 {
  int nME = 0, nx = 0;
  double xmax = 0;
  std::vector<int> mu, nu, mv;
  std::vector<double> F;  // F[ix + nx*e]
};
struct Cell3 {
  int nME = 0, nx = 0, ny = 0;
  double xmax = 0, ymax = 0;
  std::vector<int> mu, nu, mv;
  std::vector<double> F;  // F[ix + nx*(iy + ny*e)]
};

// a munu unit: re-opening the file already open keeps the position
struct Unit {
  std::string name;
  Text t;
  bool open(const std::string &path) {
    if (path == name) return true;
    name = path;
    return t.load(path);
  }
};

bool map_equal(const Cell2 &c, const MEMap &m) {
  if (c.nME != m.n) return false;
  for (int e = 0; e < m.n; e++)
    if (c.mu[e] - 1 != m.mu[e] || c.nu[e] - 1 != m.nu[e]) return false;
  return true;
}
bool map_equal3(const Cell3 &c, const MEMap &m) {
  if (c.nME != m.n) return false;
  for (int e = 0; e < m.n; e++)
    if (c.mu[e] - 1 != m.mu[e] || c.nu[e] - 1 != m.nu[e] || c.mv[e] != m.mv[e]) return false;
  return true;
}

}  // namespace

int fdata_read(const std::string &dir, int nspecies, const int *nZ, FdataHost &out, std::string &err) {
  if (nspecies < 1 || nspecies > MAXSP) {
    err = "nspecies out of range";
    return FB_ERR_ARG;
  }
  out = FdataHost();
  out.nspecies = nspecies;
  for (int k = 0; k < nspecies; k++) out.sp[k].nZ = nZ[k];

  // ---- read_info ----------------------------------------------------------
  {
    Text t;
    std::string path = dir + "/info.dat", s;
    if (!t.load(path)) {
      err = "cannot open " + path;
      return FB_ERR_IO;
    }
    int nsf = 0;
    t.line(s);  // signature
    if (!read_ints(t, 1, &nsf)) goto bad_info;
    for (int b = 0; b < nsf; b++) {
      int z = 0;
      t.skip();
      t.skip();
      t.line(s);  // symbol
      if (!read_ints(t, 1, &z)) goto bad_info;
      int isp = -1;
      for (int k = 0; k < nspecies; k++)
        if (out.sp[k].nZ == z) {
          isp = k;
          break;
        }
      if (isp < 0) {
        for (int l = 0; l < 12; l++) t.skip();
        continue;
      }
      SpeciesHost &sp = out.sp[isp];
      double xmass, q[8], rc[8], rcpp, ae;
      int lpp[8];
      if (!read_dbls(t, 1, &xmass) || !read_ints(t, 1, &sp.nssh) || sp.nssh < 1 || sp.nssh > 8) goto bad_info;
      if (!read_ints(t, sp.nssh, sp.lssh) || !read_dbls(t, sp.nssh, q) || !read_dbls(t, sp.nssh, rc)) goto bad_info;
      if (!read_ints(t, 1, &sp.nssh_pp) || sp.nssh_pp < 0 || sp.nssh_pp > 8) goto bad_info;
      if (sp.nssh_pp > 0 && !read_ints(t, sp.nssh_pp, lpp)) goto bad_info;
      if (!read_dbls(t, 1, &rcpp)) goto bad_info;
      sp.rc_pp = rcpp;  // M_species.f90:1147, used as read (M_neighbors_PP.f90:469)
      for (int k = 0; k < sp.nssh_pp; k++) sp.lpp[k] = lpp[k];
      t.skip();
      t.skip();
      if (!read_dbls(t, 1, &ae)) goto bad_info;
      t.skip();
      sp.q0 = 0.0;
      for (int k = 0; k < sp.nssh; k++) sp.q0 += q[k], sp.qn[k] = q[k];
      sp.rcA = -99.0;
      sp.rcmin = 99.0;
      sp.norb = 0;
      for (int k = 0; k < sp.nssh; k++) {
        double r = rc[k] * P_abohr;  // M_species.f90:1164-1167
        if (r > sp.rcA) sp.rcA = r;
        sp.rcmin = std::fmin(sp.rcmin, r);  // M_assemble_2c_DOGS.f90:746-754
        sp.norb += 2 * sp.lssh[k] + 1;
      }
    }
    for (int k = 0; k < nspecies; k++) {
      SpeciesHost &sp = out.sp[k];
      if (sp.nssh == 0) {
        err = "species nZ=" + std::to_string(sp.nZ) + " not in info.dat";
        return FB_ERR_IO;
      }
      if (sp.nssh == 1 && sp.lssh[0] == 0) sp.pattern = PAT_S;
      else if (sp.nssh == 2 && sp.lssh[0] == 0 && sp.lssh[1] == 1) sp.pattern = PAT_SP;
      else if (sp.nssh == 3 && sp.lssh[0] == 0 && sp.lssh[1] == 1 && sp.lssh[2] == 2) sp.pattern = PAT_SPD;
      else {
        err = "basis of species nZ=" + std::to_string(sp.nZ) + " is not s, sp or spd";
        return FB_ERR_UNSUPPORTED;
      }
      if (sp.pattern == PAT_SPD) out.have_d = 1;
      sp.norb_pp = 0;
      for (int k = 0; k < sp.nssh_pp; k++) sp.norb_pp += 2 * sp.lpp[k] + 1;
    }
    goto info_done;
  bad_info:
    err = "parse error in " + path;
    return FB_ERR_IO;
  }
info_done:

  // ---- read_Fdata_2c --------------------------------------------------------
  bool dogs_ok = true;  // every DOGS sub-cell and z-dipole table found
  bool pp_ok = true;    // every vnl table found
  bool vxc_ok = true;   // every McWEDA table found
  for (int is = 0; is < nspecies; is++) {
    for (int js = 0; js < nspecies; js++) {
      std::string pz = zz(out.sp[is].nZ) + "." + zz(out.sp[js].nZ);
      Text t;
      std::string path = dir + "/2c." + pz + ".dat";
      int ncell = 0;
      if (!t.load(path)) {
        err = "cannot open " + path;
        return FB_ERR_IO;
      }
      if (!read_ints(t, 1, &ncell) || ncell < 1) {
        err = "bad " + path;
        return FB_ERR_IO;
      }
      std::vector<Cell2> cells(ncell);
      int index[26][10];
      for (auto &r : index)
        for (int &v : r) v = -1;
      Text td;
      path = dir + "/2c." + pz + ".dir";
      if (!td.load(path)) {
        err = "cannot open " + path;
        return FB_ERR_IO;
      }
      Unit u14;
      for (int ic = 0; ic < ncell; ic++) {
        std::vector<std::string> tok;
        if (!td.read(7, tok)) {
          err = "short " + path;
          return FB_ERR_IO;
        }
        int iindex = std::atoi(tok[0].c_str()), itype = std::atoi(tok[1].c_str()), isub = std::atoi(tok[2].c_str());
        Cell2 &c = cells[ic];
        c.nME = std::atoi(tok[4].c_str());
        c.nx = std::atoi(tok[5].c_str());
        c.xmax = to_d(tok[6]);
        if (itype < 1 || itype > 25 || isub < 0 || isub > 9 || c.nME < 1 || c.nx < 7) {
          err = "bad entry in " + path;
          return FB_ERR_IO;
        }
        index[itype][isub] = iindex;
        c.F.resize((size_t)c.nx * c.nME);
        Text tf;
        std::string fpath = dir + "/" + tok[3];
        if (!tf.load(fpath)) {
          err = "cannot open " + fpath;
          return FB_ERR_IO;
        }
        std::vector<double> row(c.nME);
        for (int ix = 0; ix < c.nx; ix++) {
          if (!read_dbls(tf, c.nME, row.data())) {
            err = "short data " + fpath;
            return FB_ERR_IO;
          }
          for (int e = 0; e < c.nME; e++) c.F[ix + (size_t)c.nx * e] = row[e];
        }
        std::string mpath = dir + "/" + zz(itype) + "_munu_2c." + pz + ".dat";
        c.mu.resize(c.nME);
        c.nu.resize(c.nME);
        c.mv.resize(c.nME);
        if (!u14.open(mpath) || !read_ints(u14.t, c.nME, c.mu.data()) || !read_ints(u14.t, c.nME, c.nu.data()) ||
            !read_ints(u14.t, c.nME, c.mv.data())) {
          err = "bad munu " + mpath;
          return FB_ERR_IO;
        }
      }
      // stage cell (itype, isub) into d: 0 staged, 1 absent, else an error
      int PA = out.sp[is].pattern, PB = out.sp[js].pattern;
      auto stage_map = [&](int it, int isub, const MEMap &m, Cell2cDev &d) -> int {
        int k = index[it][isub];
        d.off = -1;
        if (k < 1 || k > ncell) return 1;
        const Cell2 &c = cells[k - 1];
        if (!map_equal(c, m)) {
          err = "2c table " + pz + " interaction " + std::to_string(it) + " sub " + std::to_string(isub) +
                " has a non-canonical ME map";
          return FB_ERR_UNSUPPORTED;
        }
        d.nx = c.nx;
        d.nME = c.nME;
        d.xmax = c.xmax;
        d.dx = c.xmax / (c.nx - 1);  // M_Fdata_2c.f90:222
        double dx3 = d.dx * d.dx * d.dx;
        d.inv_dx6 = 1.0 / (dx3 * dx3);
        d.off = (long long)out.table2c.size();
        for (int ix = 0; ix < c.nx; ix++)
          for (int e = 0; e < c.nME; e++) out.table2c.push_back(c.F[ix + (size_t)c.nx * e]);
        return 0;
      };
      auto stage = [&](int it, int isub, Cell2cDev &d) -> int {
        return stage_map(it, isub, make_munu(PA, it == 5 ? PA : PB), d);
      };
      // the five Harris interactions (isub = 0)
      for (int it = 1; it <= 5; it++) {
        int r = stage(it, 0, out.dev.c2[is][js][it - 1]);
        if (r == 1) {
          err = "2c table " + pz + " lacks interaction " + std::to_string(it);
          return FB_ERR_TABLE;
        }
        if (r) return r;
      }
      // non-local pseudopotential table (itype 6): basis of is, projectors of js
      {
        int PPB = out.sp[js].pattern_pp();
        Cell2cDev &d = out.dev.c2vnl[is][js];
        d.off = -1;
        int k = index[6][0];
        if (PPB < 0 || k < 1 || k > ncell) {
          pp_ok = false;
        } else {
          const Cell2 &c = cells[k - 1];
          if (!map_equal(c, make_munu(PA, PPB))) {
            err = "2c table " + pz + " vnl has a non-canonical ME map";
            return FB_ERR_UNSUPPORTED;
          }
          d.nx = c.nx;
          d.nME = c.nME;
          d.xmax = c.xmax;
          d.dx = c.xmax / (c.nx - 1);
          double dx3 = d.dx * d.dx * d.dx;
          d.inv_dx6 = 1.0 / (dx3 * dx3);
          d.off = (long long)out.table2c.size();
          for (int ix = 0; ix < c.nx; ix++)
            for (int e = 0; e < c.nME; e++) out.table2c.push_back(c.F[ix + (size_t)c.nx * e]);
        }
      }
      // DOGS: charged-shell sub-cells of vna ontop L (shells of the first
      // species), ontop R and atom (shells of the second), and dipole_z
      int nsub[3] = {out.sp[is].nssh, out.sp[js].nssh, out.sp[js].nssh};
      for (int q = 0; q < 3; q++)
        for (int isorp = 1; isorp <= MAXSUB; isorp++) {
          Cell2cDev &d = out.dev.c2s[is][js][q][isorp - 1];
          d.off = -1;
          if (isorp > nsub[q]) continue;
          int r = stage(3 + q, isorp, d);
          if (r == 1) dogs_ok = false;
          else if (r) return r;
        }
      if (nsub[0] > MAXSUB || nsub[1] > MAXSUB) dogs_ok = false;
      {
        int r = stage(10, 0, out.dev.c2dip[is][js]);
        if (r == 1) dogs_ok = false;
        else if (r) return r;
      }
      // McWEDA: vxc_ontop and the density sub-cells
      {
        int r = stage(7, 0, out.dev.c2vxc[is][js]);
        if (r == 1) vxc_ok = false;
        else if (r) return r;
        const int its[6] = {15, 16, 17, 19, 20, 21};
        const MEMap maps[6] = {make_munu(PA, PB), make_munu(PA, PB), make_munu(PA, PA),
                               make_munu_s(PA, PB), make_munu_s(PA, PB), make_munu_s(PA, PA)};
        int nsh[6] = {out.sp[is].nssh, out.sp[js].nssh, out.sp[js].nssh,
                      out.sp[is].nssh, out.sp[js].nssh, out.sp[js].nssh};
        for (int q = 0; q < 6; q++)
          for (int isorp = 1; isorp <= MAXSUB; isorp++) {
            Cell2cDev &d = out.dev.c2rho[is][js][q][isorp - 1];
            d.off = -1;
            if (isorp > nsh[q]) continue;
            r = stage_map(its[q], isorp, maps[q], d);
            if (r == 1) vxc_ok = false;
            else if (r) return r;
          }
        if (nsh[0] > MAXSUB || nsh[1] > MAXSUB) vxc_ok = false;
      }
    }
    // clPP.ZZ.dat is opened unconditionally (M_Fdata_2c.f90:252-258)
    Text t;
    std::string path = dir + "/clPP." + zz(out.sp[is].nZ) + ".dat";
    if (!t.load(path)) {
      err = "cannot open " + path;
      return FB_ERR_IO;
    }
    for (int k = 0; k < out.sp[is].nssh_pp; k++) {
      double cl;
      if (!read_dbls(t, 1, &cl)) {
        err = "short " + path;
        return FB_ERR_IO;
      }
      out.sp[is].cl_pp[k] = cl;
    }
  }

  // ---- read_Fdata_3c --------------------------------------------------------
  for (int is = 0; is < nspecies; is++)
    for (int js = 0; js < nspecies; js++)
      for (int ks = 0; ks < nspecies; ks++) {
        std::string pz = zz(out.sp[is].nZ) + "." + zz(out.sp[js].nZ) + "." + zz(out.sp[ks].nZ);
        Text t;
        std::string path = dir + "/3c." + pz + ".dat";
        int ncell = 0;
        if (!t.load(path)) {
          err = "cannot open " + path;
          return FB_ERR_IO;
        }
        if (!read_ints(t, 1, &ncell) || ncell < 1) {
          err = "bad " + path;
          return FB_ERR_IO;
        }
        std::vector<Cell3> cells(ncell);
        int index[5][7][6];
        for (auto &a : index)
          for (auto &b : a)
            for (int &v : b) v = -1;
        Text td;
        path = dir + "/3c." + pz + ".dir";
        if (!td.load(path)) {
          err = "cannot open " + path;
          return FB_ERR_IO;
        }
        Unit u13;
        for (int ic = 0; ic < ncell; ic++) {
          std::vector<std::string> tok;
          if (!td.read(10, tok)) {
            err = "short " + path;
            return FB_ERR_IO;
          }
          int iindex = std::atoi(tok[0].c_str()), itype = std::atoi(tok[1].c_str());
          int isub = std::atoi(tok[2].c_str()), ith = std::atoi(tok[3].c_str());
          Cell3 &c = cells[ic];
          c.nME = std::atoi(tok[5].c_str());
          c.nx = std::atoi(tok[6].c_str());
          c.xmax = to_d(tok[7]);
          c.ny = std::atoi(tok[8].c_str());
          c.ymax = to_d(tok[9]);
          if (itype < 1 || itype > 4 || isub < 0 || isub > 6 || ith < 1 || ith > 5 || c.nME < 1 || c.nx < 4 ||
              c.ny < 4) {
            err = "bad entry in " + path;
            return FB_ERR_IO;
          }
          index[itype][isub][ith] = iindex;
          c.F.resize((size_t)c.nx * c.ny * c.nME);
          Text tf;
          std::string fpath = dir + "/" + tok[4];
          if (!tf.load(fpath)) {
            err = "cannot open " + fpath;
            return FB_ERR_IO;
          }
          std::vector<double> row(c.nME);
          for (int iy = 0; iy < c.ny; iy++)
            for (int ix = 0; ix < c.nx; ix++) {
              if (!read_dbls(tf, c.nME, row.data())) {
                err = "short data " + fpath;
                return FB_ERR_IO;
              }
              for (int e = 0; e < c.nME; e++) c.F[ix + (size_t)c.nx * (iy + (size_t)c.ny * e)] = row[e];
            }
          std::string mpath = dir + "/" + zz(itype) + "_munu_3c." + pz + ".dat";
          c.mu.resize(c.nME);
          c.nu.resize(c.nME);
          c.mv.resize(c.nME);
          if (!u13.open(mpath) || !read_ints(u13.t, c.nME, c.mu.data()) || !read_ints(u13.t, c.nME, c.nu.data()) ||
              !read_ints(u13.t, c.nME, c.mv.data())) {
            err = "bad munu " + mpath;
            return FB_ERR_IO;
          }
        }
        // stage bcna (interaction 3) sub-cell isub, theta 1..5: 0 staged,
        // 1 absent, else an error
        int PA = out.sp[is].pattern, PB = out.sp[js].pattern;
        auto stage3m = [&](int itype, int isub, const MEMap &m, Cell3cDev &d) -> int {
          d.off = -1;
          const Cell3 *th[NTHETA];
          for (int it = 1; it <= NTHETA; it++) {
            int k = index[itype][isub][it];
            if (k < 1 || k > ncell) return 1;
            th[it - 1] = &cells[k - 1];
            if (!map_equal3(*th[it - 1], m)) {
              err = "3c table " + pz + " sub " + std::to_string(isub) + " has a non-canonical ME map";
              return FB_ERR_UNSUPPORTED;
            }
            if (th[it - 1]->nx != th[0]->nx || th[it - 1]->ny != th[0]->ny) {
              err = "3c table " + pz + ": theta cells on different grids";
              return FB_ERR_UNSUPPORTED;
            }
          }
          const Cell3 &c1 = *th[0];
          d.nx = c1.nx;
          d.ny = c1.ny;
          d.nME = c1.nME;
          d.xmax = c1.xmax;
          d.ymax = c1.ymax;
          d.dx = c1.xmax / (c1.nx - 1.0);  // M_Fdata_3c.f90:367-368
          d.dy = c1.ymax / (c1.ny - 1.0);
          {
            double ix = 1.0 / d.dx, iy = 1.0 / d.dy;
            d.idxd = ix;
            d.idyd = iy;
            d.idx_h = (float)ix;
            d.idx_l = (float)(ix - (double)d.idx_h);
            d.idy_h = (float)iy;
            d.idy_l = (float)(iy - (double)d.idy_h);
          }
          d.off = (long long)out.table3c.size();
          d.node_off = (long long)out.lin.size();
          for (int iy = 0; iy < c1.ny; iy++)
            for (int ix = 0; ix < c1.nx; ix++) {
              for (int it = 0; it < NTHETA; it++)
                for (int e = 0; e < c1.nME; e++)
                  out.table3c.push_back(th[it]->F[ix + (size_t)c1.nx * (iy + (size_t)c1.ny * e)]);
              // gradient switch from theta 1, ME 1 (M_Fdata_3c.f90:383-385)
              double gx = 0.0, gy = 0.0;
              unsigned char lin = 0;
              if (ix + 1 < c1.nx && iy + 1 < c1.ny) {
                double f00 = c1.F[ix + (size_t)c1.nx * iy];
                gx = (c1.F[(ix + 1) + (size_t)c1.nx * iy] - f00) / d.dx;
                gy = (c1.F[ix + (size_t)c1.nx * (iy + 1)] - f00) / d.dy;
                double gg = gx * gx + gy * gy;
                lin = gg < 1.0e-6 ? 1 : 0;
              }
              out.lin.push_back(lin);
              out.gxy.push_back(gx);
              out.gxy.push_back(gy);
            }
          return 0;
        };
        auto stage3 = [&](int isub, Cell3cDev &d) -> int { return stage3m(3, isub, make_munu_3c(PA, PB), d); };
        int r = stage3(0, out.dev.c3[is][js][ks]);
        if (r == 1) {
          err = "3c table " + pz + " lacks bcna";
          return FB_ERR_TABLE;
        }
        if (r) return r;
        // DOGS: the neutral atom's charged shells isorp = 1..nssh
        int nk = out.sp[ks].nssh;
        if (nk > MAXSUB) dogs_ok = false;
        for (int isorp = 1; isorp <= MAXSUB; isorp++) {
          Cell3cDev &dd = out.dev.c3s[is][js][ks][isorp - 1];
          dd.off = -1;
          if (isorp > nk) continue;
          r = stage3(isorp, dd);
          if (r == 1) dogs_ok = false;
          else if (r) return r;
        }
        // McWEDA three-center densities den3 (itype 1) and denS3 (itype 2)
        for (int q = 0; q < 2; q++)
          for (int isorp = 1; isorp <= MAXSUB; isorp++) {
            Cell3cDev &dd = out.dev.c3rho[is][js][ks][q][isorp - 1];
            dd.off = -1;
            if (isorp > nk) continue;
            r = stage3m(q + 1, isorp, q == 0 ? make_munu_3c(PA, PB) : make_munu_s(PA, PB), dd);
            if (r == 1) vxc_ok = false;
            else if (r) return r;
          }
        if (nk > MAXSUB) vxc_ok = false;
        // Qneutral-weighted sums of the sub-cells
        for (int q = 0; q < 2; q++) {
          Cell3cDev &dq = out.dev.c3rhoq[is][js][ks][q];
          dq.off = -1;
          if (nk < 1 || nk > MAXSUB) continue;
          const Cell3cDev &c0 = out.dev.c3rho[is][js][ks][q][0];
          bool ok = c0.off >= 0;
          for (int k = 1; k < nk && ok; k++) {
            const Cell3cDev &ck = out.dev.c3rho[is][js][ks][q][k];
            ok = ck.off >= 0 && ck.nx == c0.nx && ck.ny == c0.ny && ck.nME == c0.nME && ck.dx == c0.dx && ck.dy == c0.dy;
          }
          long long nn = (long long)c0.nx * c0.ny;
          if (!ok) continue;
          dq = c0;
          dq.off = (long long)out.table3c.size();
          dq.node_off = (long long)out.lin.size();
          long long nv = nn * NTHETA * c0.nME;
          for (long long k = 0; k < nv; k++) {
            double acc = 0.0;
            for (int i = 0; i < nk; i++)
              acc += out.sp[ks].qn[i] * out.table3c[out.dev.c3rho[is][js][ks][q][i].off + k];
            out.table3c.push_back(acc);
          }
          for (long long n = 0; n < nn; n++) {
            // the common gradient switch, or 2 where the sub-cells disagree
            // (a triplet on such a node takes the sub-cells one by one)
            unsigned char l0 = out.lin[c0.node_off + n];
            for (int k = 1; k < nk; k++)
              if (out.lin[out.dev.c3rho[is][js][ks][q][k].node_off + n] != l0) l0 = 2;
            out.lin.push_back(l0);
            for (int d = 0; d < 2; d++) {
              double acc = 0.0;
              for (int i = 0; i < nk; i++)
                acc += out.sp[ks].qn[i] * out.gxy[2 * (out.dev.c3rho[is][js][ks][q][i].node_off + n) + d];
              out.gxy.push_back(acc);
            }
          }
        }
      }

  // one-center McWEDA xc (read_Fdata_1c, e.FDATA/M_Fdata_1c_McWEDA_Harris.f90:
  // 99-136): vxc_1c.ZZ.dat, nssh records of E then nssh records of V
  for (int k = 0; k < nspecies && vxc_ok; k++) {
    Text t;
    int n = out.sp[k].nssh;
    if (n > MAXSUB || !t.load(dir + "/vxc_1c." + zz(out.sp[k].nZ) + ".dat")) {
      vxc_ok = false;
      break;
    }
    double row[8];
    for (int a = 0; a < n && vxc_ok; a++) vxc_ok = read_dbls(t, n, row);  // E
    for (int a = 0; a < n && vxc_ok; a++) {
      vxc_ok = read_dbls(t, n, row);
      for (int b = 0; b < n; b++) out.dev.vxc1c[k][a * MAXSUB + b] = row[b];
    }
    if (!vxc_ok) {
      err = "parse error in vxc_1c." + zz(out.sp[k].nZ) + ".dat";
      return FB_ERR_IO;
    }
  }

  // double-float copy of the 3c values: hi = nearest float, lo = nearest
  // float of the remainder (exact in double)
  out.table3c_df.resize(2 * out.table3c.size());
  for (size_t k = 0; k < out.table3c.size(); k++) {
    double v = out.table3c[k];
    float h = (float)v;
    out.table3c_df[2 * k] = h;
    out.table3c_df[2 * k + 1] = (float)(v - (double)h);
  }
  out.dev.nspecies = nspecies;
  out.dev.have_d = out.have_d;
  for (int k = 0; k < nspecies; k++) {
    out.dev.sp[k].pattern = out.sp[k].pattern;
    out.dev.sp[k].norb = out.sp[k].norb;
    out.dev.sp[k].rcA = out.sp[k].rcA;
    out.dev.sp[k].nssh = out.sp[k].nssh;
    out.dev.sp[k].rcmin = out.sp[k].rcmin;
    // cl (b.FUNCTIONS/cl.f90:50-90): the shell's cl for each of its 2l+1 projectors
    const SpeciesHost &sh = out.sp[k];
    out.dev.sp[k].pp_pattern = sh.pattern_pp();
    out.dev.sp[k].norb_pp = sh.norb_pp;
    out.dev.sp[k].rc_pp = sh.rc_pp;
    out.dev.sp[k].q0 = sh.q0;
    for (int q = 0; q < MAXSUB; q++) out.dev.sp[k].qn[q] = q < sh.nssh ? sh.qn[q] : 0.0;
    int o = 0;
    for (int q = 0; q < sh.nssh_pp && o < 9; q++)
      for (int m = 0; m < 2 * sh.lpp[q] + 1 && o < 9; m++) out.dev.sp[k].cl[o++] = sh.cl_pp[q];
    if (sh.pattern_pp() < 0) pp_ok = false;
  }
  out.dev.have_pp = pp_ok ? 1 : 0;
  out.dev.have_dogs = dogs_ok ? 1 : 0;
  out.dev.have_vxc = vxc_ok ? 1 : 0;
  out.dev.vxc_qsum_all = 1;
  for (int is = 0; is < nspecies; is++)
    for (int js = 0; js < nspecies; js++)
      for (int ks = 0; ks < nspecies; ks++)
        for (int q = 0; q < 2; q++) {
          const Cell3cDev &cq = out.dev.c3rhoq[is][js][ks][q];
          if (cq.off < 0) {
            out.dev.vxc_qsum_all = 0;
            continue;
          }
          for (long long n = 0; n < (long long)cq.nx * cq.ny; n++)
            if (out.lin[cq.node_off + n] == 2) out.dev.vxc_qsum_all = 0;
        }
  return FB_OK;
}

}  // namespace fb
