// fb_fdata.h -- host reader of the FIREBALL Fdata text format (libfbgpu).
#pragma once
#include <string>
#include <vector>
#include "fb_internal.h"

namespace fb {

struct SpeciesHost {
  int nZ = 0, nssh = 0, norb = 0, pattern = -1, nssh_pp = 0;
  int lssh[8] = {0};
  double rcA = 0.0;
  double rcmin = 99.0;
  int lpp[8] = {0};
  double rc_pp = 0.0;
  double q0 = 0.0;  // sum of the shells' Qneutral
  double qn[8] = {0};  // Qneutral per shell
  double cl_pp[8] = {0};
  int norb_pp = 0;
  // projector shells as a basis pattern: s, sp or spd, else -1
  int pattern_pp() const {
    if (nssh_pp == 1 && lpp[0] == 0) return PAT_S;
    if (nssh_pp == 2 && lpp[0] == 0 && lpp[1] == 1) return PAT_SP;
    if (nssh_pp == 3 && lpp[0] == 0 && lpp[1] == 1 && lpp[2] == 2) return PAT_SPD;
    return -1;
  }
};

struct FdataHost {
  int nspecies = 0, have_d = 0;
  SpeciesHost sp[MAXSP];
  std::vector<double> table2c, table3c, gxy;
  std::vector<float> table3c_df;  // hi, lo float pairs of table3c
  std::vector<unsigned char> lin;
  FdataDev dev{};
};

// read_info + read_Fdata_2c + read_Fdata_3c; returns an FB_ERR_* status
int fdata_read(const std::string &dir, int nspecies, const int *nZ, FdataHost &out, std::string &err);

}  // namespace fb
