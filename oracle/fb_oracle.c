/*
 * fb_oracle.c -- CPU oracle: plain-C restatement of the FIREBALL Harris
 * matrix-element assembly (reference: thunder-dft/thunder-master, Fortran).
 *
 * TEST INFRASTRUCTURE ONLY (see fb_oracle.h).  Parity status: UNPINNED --
 * the reference has no tests or golden data and cannot be compiled here.
 *
 * Every routine below names the reference file:line range it restates.  The
 * floating-point expressions keep the reference's operation order; the file
 * is compiled with -ffp-contract=off so no fused multiply-adds are formed.
 * Fortran 1-based indices are kept where they appear in arithmetic (grid
 * points, orbital numbers) and converted to 0-based only for storage.
 */
#include "fb_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* status codes, identical to include/fbgpu.h */
enum {
  OK = 0, E_ARG = 1, E_IO = 2, E_TABLE = 3, E_XNEG = 4, E_XLARGE = 5,
  E_CLOSE = 6, E_SELF = 7, E_BACK = 8, E_UNSUP = 13
};

/* include/constants.h:2,4 */
#define P_abohr 0.529177
#define P_eq2 14.39975

/* include/interactions_2c.h:2-3, interactions_3c.h:2-4 */
#define P_MAXTYPE2 25
#define P_MAXSUB2 9
#define P_MAXTYPE3 4
#define P_MAXSUB3 6
#define P_MAXTHETA 5
#define P_overlap 1
#define P_kinetic 2
#define P_vna_ontopL 3
#define P_vna_ontopR 4
#define P_vna_atom 5
#define P_vnl 6
#define P_dipole_z 10
#define P_bcna 3
#define P_mbox 4 /* c.SYSTEM/M_configuraciones.f90:359 */

#define MAXSP 8
#define MAXSH 8
#define MAXORB 16

static __thread char g_err[512];
static int g_threads = 1;
/* test switch (or_set_exact_derivatives): 0 keeps the reference's forms */
static int g_exact = 0;

static void seterr(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}
const char *or_last_error(void) { return g_err; }
void or_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
void or_set_exact_derivatives(int on) { g_exact = on ? 1 : 0; }

/* ------------------------------------------------------------------------ */
/* data types: T_Fdata_cell_2c/bundle (e.FDATA/M_Fdata_2c.f90:83-109),       */
/* T_Fdata_cell_3c/bundle (e.FDATA/M_Fdata_3c.f90:77-103), T_species         */
/* (c.SYSTEM/M_species.f90:116-164)                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nME, nx;
  double dx, xmax;
  int *mu, *nu, *mvalue;
  double *F; /* F[(ix-1) + nx*(iME-1)] */
} cell2c;

typedef struct {
  int ncell;
  int index[P_MAXTYPE2 + 1][P_MAXSUB2 + 1];
  cell2c *cells;
} bundle2c;

typedef struct {
  int nME, nx, ny;
  double xmax, ymax;
  int *mu, *nu, *mvalue;
  double *F; /* F[(ix-1) + nx*((iy-1) + ny*(iME-1))] */
} cell3c;

typedef struct {
  int ncell;
  int index[P_MAXTYPE3 + 1][P_MAXSUB3 + 1][P_MAXTHETA + 1];
  cell3c *cells;
} bundle3c;

typedef struct {
  int nZ, nssh, nssh_PP, norb_max;
  int lssh[MAXSH];
  double rcutoffA[MAXSH];
  double rcutoffA_max;
  /* pseudopotential projectors: shells, orbitals, cutoff (as read), cl */
  int lssh_PP[MAXSH], norb_PP_max;
  double rcutoff_PP, cl_PP[MAXSH];
  double Q0; /* sum of the shells' Qneutral */
  double qn[MAXSH]; /* Qneutral per shell */
  /* one-center McWEDA xc (e.FDATA/M_Fdata_1c_McWEDA_Harris.f90:58-61):
   * E(issh, jssh), V(issh, jssh) at [issh * MAXSH + jssh], 0-based */
  int have_vxc1c;
  double vxc1c_E[MAXSH * MAXSH], vxc1c_V[MAXSH * MAXSH];
} species_t;

struct or_fdata {
  int nspecies, have_dorbitals, have_dorbitals_PP;
  species_t sp[MAXSP + 1]; /* 1-based */
  bundle2c b2[MAXSP + 1][MAXSP + 1];
  bundle3c b3[MAXSP + 1][MAXSP + 1][MAXSP + 1];
};

struct or_sys {
  or_fdata *fd;
  int natoms, icluster, mbeta_max;
  double *ratom; /* 3N */
  int *imass;
  double lattice[3][3];
  double (*xl)[3];
  /* neighbors */
  int *neighn, *pair_off, *neigh_j, *neigh_b, *neigh_back, *neigh_self;
  long long *blk_off;
  long long nblock;
  int npairs;
  int *ncommon, *trip_off, *ci_j, *ci_b, *cj_j, *cj_b, *cneigh;
  int ntrip;
  /* DOGS shell charges dQ[i * nssh_max + isorp - 1] */
  double *dQ;
  int nssh_max;
  /* pseudopotential neighbor maps (c.SYSTEM/M_neighbors_PP.f90), CSR by
   * atom, 0-based: PP (basis i, projector j), PPx (projector i, basis j),
   * PPp (pairs sharing a projector), and the PP common-neighbor triplets */
  int have_pp;
  int *pp_off, *pp_j, *pp_b, *pp_self, *pp_map;
  int *ppx_off, *ppx_j, *ppx_b, *ppx_self, *ppx_map, *ppx_point;
  int *ppp_off, *ppp_j, *ppp_b, *ppp_self;
  long long *svnl_off, *vnl_off, nsvnl, nvnl;
  int *ppc_off, *ppc_i, *ppc_ib, *ppc_j, *ppc_jb, *ppc_m, *ppc_m31, *ppc_m32;
};

/* ------------------------------------------------------------------------ */
/* list-directed text input                                                  */
/* ------------------------------------------------------------------------ */
typedef struct {
  char *buf;
  size_t len, pos; /* pos = start of the next record */
} txt;

static int txt_open(txt *t, const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) {
    seterr("cannot open %s", path);
    return E_IO;
  }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  t->buf = (char *)malloc((size_t)n + 1);
  t->len = fread(t->buf, 1, (size_t)n, f);
  t->buf[t->len] = 0;
  t->pos = 0;
  fclose(f);
  return OK;
}
static void txt_close(txt *t) {
  free(t->buf);
  t->buf = NULL;
}

/* One list-directed READ of ntok tokens: starts at the next record, may span
 * records, and leaves the file at the record after the last one touched.
 * Tokens are separated by blanks or commas.  Returns number of tokens read. */
static int txt_read(txt *t, int ntok, char tok[][64]) {
  int got = 0;
  size_t p = t->pos;
  if (p >= t->len) return 0;
  while (got < ntok && p < t->len) {
    /* scan this record */
    while (p < t->len && t->buf[p] != '\n') {
      while (p < t->len && (t->buf[p] == ' ' || t->buf[p] == '\t' ||
                            t->buf[p] == ',' || t->buf[p] == '\r'))
        p++;
      if (p >= t->len || t->buf[p] == '\n') break;
      size_t q = p;
      while (q < t->len && !isspace((unsigned char)t->buf[q]) && t->buf[q] != ',')
        q++;
      if (got < ntok) {
        size_t L = q - p < 63 ? q - p : 63;
        memcpy(tok[got], t->buf + p, L);
        tok[got][L] = 0;
        got++;
      }
      p = q;
      if (got == ntok) break;
    }
    /* advance to the next record */
    while (p < t->len && t->buf[p] != '\n') p++;
    if (p < t->len) p++;
  }
  t->pos = p;
  return got;
}

/* skip one record (READ with empty list) */
static int txt_skip(txt *t) {
  if (t->pos >= t->len) return 0;
  while (t->pos < t->len && t->buf[t->pos] != '\n') t->pos++;
  if (t->pos < t->len) t->pos++;
  return 1;
}

/* raw record (formatted A read) */
static int txt_line(txt *t, char *out, int n) {
  if (t->pos >= t->len) return 0;
  size_t q = t->pos;
  int k = 0;
  while (q < t->len && t->buf[q] != '\n') {
    if (k < n - 1) out[k++] = t->buf[q];
    q++;
  }
  out[k] = 0;
  t->pos = q < t->len ? q + 1 : q;
  return 1;
}

static double tok_d(const char *s) {
  char b[64];
  int i;
  for (i = 0; s[i] && i < 63; i++) b[i] = (s[i] == 'D' || s[i] == 'd') ? 'E' : s[i];
  b[i] = 0;
  return strtod(b, NULL);
}

static int read_ints(txt *t, int n, int *out) {
  char tok[64][64];
  if (n > 64 || txt_read(t, n, tok) != n) return E_IO;
  for (int i = 0; i < n; i++) out[i] = atoi(tok[i]);
  return OK;
}
static int read_dbls(txt *t, int n, double *out) {
  static __thread char tok[128][64];
  if (n > 128 || txt_read(t, n, tok) != n) return E_IO;
  for (int i = 0; i < n; i++) out[i] = tok_d(tok[i]);
  return OK;
}

/* ------------------------------------------------------------------------ */
/* read_info (c.SYSTEM/M_species.f90:1057-1251) -- species block structure   */
/* ------------------------------------------------------------------------ */
static int read_info(or_fdata *fd, const char *dir, const int *nZreq) {
  char path[1024], line[256];
  txt t;
  snprintf(path, sizeof path, "%s/info.dat", dir);
  if (txt_open(&t, path)) return E_IO;
  int nsf;
  txt_line(&t, line, sizeof line); /* signature (2x, a70) */
  if (read_ints(&t, 1, &nsf)) goto bad;
  for (int k = 1; k <= fd->nspecies; k++) fd->sp[k].nZ = nZreq[k - 1], fd->sp[k].nssh = 0;
  for (int iskip = 0; iskip < nsf; iskip++) {
    int nZ, isp = 0;
    txt_skip(&t);
    txt_skip(&t);
    txt_line(&t, line, sizeof line); /* symbol (2x, a2) */
    if (read_ints(&t, 1, &nZ)) goto bad;
    for (int k = 1; k <= fd->nspecies; k++)
      if (fd->sp[k].nZ == nZ) { isp = k; break; }
    if (!isp) {
      for (int l = 0; l < 12; l++) txt_skip(&t);
      continue;
    }
    species_t *s = &fd->sp[isp];
    double xmass, qn[MAXSH], rc[MAXSH], rcpp, atomicE;
    int nssh, lpp[MAXSH];
    if (read_dbls(&t, 1, &xmass) || read_ints(&t, 1, &nssh) || nssh < 1 || nssh > MAXSH) goto bad;
    s->nssh = nssh;
    if (read_ints(&t, nssh, s->lssh) || read_dbls(&t, nssh, qn) || read_dbls(&t, nssh, rc)) goto bad;
    if (read_ints(&t, 1, &s->nssh_PP) || s->nssh_PP < 0 || s->nssh_PP > MAXSH) goto bad;
    if (s->nssh_PP > 0 && read_ints(&t, s->nssh_PP, lpp)) goto bad;
    if (read_dbls(&t, 1, &rcpp)) goto bad;
    s->rcutoff_PP = rcpp; /* :1147, used as read (M_neighbors_PP.f90:469) */
    s->Q0 = 0.0;
    for (int i = 0; i < nssh; i++) s->Q0 = s->Q0 + qn[i], s->qn[i] = qn[i];
    s->norb_PP_max = 0;   /* :1188-1194 */
    for (int i = 0; i < s->nssh_PP; i++) {
      if (lpp[i] < 0 || lpp[i] > 2) { seterr("unsupported PP l=%d", lpp[i]); txt_close(&t); return E_UNSUP; }
      s->lssh_PP[i] = lpp[i];
      s->norb_PP_max += 2 * lpp[i] + 1;
    }
    txt_skip(&t); /* wffile names */
    txt_skip(&t); /* na files */
    if (read_dbls(&t, 1, &atomicE)) goto bad;
    txt_skip(&t);
    /* :1164-1193 cutoffs in Angstrom, norb_max = sum(2l+1) */
    s->norb_max = 0;
    s->rcutoffA_max = -99.0;
    for (int i = 0; i < nssh; i++) {
      s->rcutoffA[i] = rc[i] * P_abohr;
      s->norb_max += 2 * s->lssh[i] + 1;
      if (s->lssh[i] < 0 || s->lssh[i] > 2) { seterr("unsupported l=%d", s->lssh[i]); txt_close(&t); return E_UNSUP; }
    }
  }
  txt_close(&t);
  fd->have_dorbitals = 0; /* :1212-1221 */
  fd->have_dorbitals_PP = 0;
  for (int k = 1; k <= fd->nspecies; k++) {
    if (fd->sp[k].nssh == 0) { seterr("species nZ=%d not in info.dat", fd->sp[k].nZ); return E_IO; }
    for (int i = 0; i < fd->sp[k].nssh_PP; i++)
      if (fd->sp[k].lssh_PP[i] == 2) fd->have_dorbitals_PP = 1;
    for (int i = 0; i < fd->sp[k].nssh; i++) {
      if (fd->sp[k].lssh[i] == 2) fd->have_dorbitals = 1;
      if (fd->sp[k].rcutoffA[i] > fd->sp[k].rcutoffA_max) fd->sp[k].rcutoffA_max = fd->sp[k].rcutoffA[i];
    }
    if (fd->sp[k].norb_max > MAXORB) { seterr("norb %d > %d", fd->sp[k].norb_max, MAXORB); return E_UNSUP; }
  }
  return OK;
bad:
  seterr("parse error in %s", path);
  txt_close(&t);
  return E_IO;
}

/* munu file state: a unit re-opened on the same file keeps its position */
typedef struct {
  char name[1024];
  txt t;
  int open;
} unit_t;

static int unit_open(unit_t *u, const char *path) {
  if (u->open && strcmp(u->name, path) == 0) return OK;
  if (u->open) txt_close(&u->t);
  u->open = 0;
  if (txt_open(&u->t, path)) return E_IO;
  snprintf(u->name, sizeof u->name, "%s", path);
  u->open = 1;
  return OK;
}
static void unit_close(unit_t *u) {
  if (u->open) txt_close(&u->t);
  u->open = 0;
}

/* read_Fdata_2c (e.FDATA/M_Fdata_2c.f90:149-272) */
static int read_fdata_2c(or_fdata *fd, const char *dir) {
  char path[1024], tok[8][64];
  for (int is = 1; is <= fd->nspecies; is++) {
    for (int js = 1; js <= fd->nspecies; js++) {
      bundle2c *b = &fd->b2[is][js];
      txt t;
      snprintf(path, sizeof path, "%s/2c.%02d.%02d.dat", dir, fd->sp[is].nZ, fd->sp[js].nZ);
      if (txt_open(&t, path)) return E_IO;
      if (read_ints(&t, 1, &b->ncell) || b->ncell < 1) { txt_close(&t); seterr("bad %s", path); return E_IO; }
      txt_close(&t);
      b->cells = (cell2c *)calloc((size_t)b->ncell, sizeof(cell2c));
      for (int a = 0; a <= P_MAXTYPE2; a++)
        for (int c = 0; c <= P_MAXSUB2; c++) b->index[a][c] = -1;
      snprintf(path, sizeof path, "%s/2c.%02d.%02d.dir", dir, fd->sp[is].nZ, fd->sp[js].nZ);
      txt tdir;
      if (txt_open(&tdir, path)) return E_IO;
      unit_t u14 = {0};
      for (int icell = 1; icell <= b->ncell; icell++) {
        cell2c *c = &b->cells[icell - 1];
        if (txt_read(&tdir, 7, tok) != 7) { seterr("short %s", path); txt_close(&tdir); return E_IO; }
        int iindex = atoi(tok[0]), itype = atoi(tok[1]), isub = atoi(tok[2]);
        c->nME = atoi(tok[4]);
        c->nx = atoi(tok[5]);
        c->xmax = tok_d(tok[6]);
        if (itype < 1 || itype > P_MAXTYPE2 || isub < 0 || isub > P_MAXSUB2 || c->nME < 1 || c->nx < 7) {
          seterr("bad dir entry in %s", path); txt_close(&tdir); return E_IO;
        }
        c->F = (double *)malloc(sizeof(double) * (size_t)c->nx * c->nME);
        c->mu = (int *)malloc(sizeof(int) * c->nME);
        c->nu = (int *)malloc(sizeof(int) * c->nME);
        c->mvalue = (int *)malloc(sizeof(int) * c->nME);
        b->index[itype][isub] = iindex;                 /* :221 */
        c->dx = c->xmax / (c->nx - 1);                  /* :222 */
        char dpath[1200];
        snprintf(dpath, sizeof dpath, "%s/%s", dir, tok[3]);
        txt td;
        if (txt_open(&td, dpath)) { txt_close(&tdir); return E_IO; }
        double row[128];
        if (c->nME > 128) { seterr("nME too large"); return E_UNSUP; }
        for (int ix = 1; ix <= c->nx; ix++) {         /* :230-232 */
          if (read_dbls(&td, c->nME, row)) { seterr("short data %s", dpath); txt_close(&td); txt_close(&tdir); return E_IO; }
          for (int m = 0; m < c->nME; m++) c->F[(ix - 1) + (size_t)c->nx * m] = row[m];
        }
        txt_close(&td);
        snprintf(dpath, sizeof dpath, "%s/%02d_munu_2c.%02d.%02d.dat", dir, itype, fd->sp[is].nZ, fd->sp[js].nZ);
        if (unit_open(&u14, dpath) || read_ints(&u14.t, c->nME, c->mu) ||
            read_ints(&u14.t, c->nME, c->nu) || read_ints(&u14.t, c->nME, c->mvalue)) {
          seterr("bad munu %s", dpath); unit_close(&u14); txt_close(&tdir); return E_IO;
        }
      }
      txt_close(&tdir);
      unit_close(&u14);
    }
    /* :252-258 Kleinman-Bylander coefficients, read unconditionally */
    txt t;
    snprintf(path, sizeof path, "%s/clPP.%02d.dat", dir, fd->sp[is].nZ);
    if (txt_open(&t, path)) return E_IO;
    for (int k = 0; k < fd->sp[is].nssh_PP; k++) {
      double cl;
      if (read_dbls(&t, 1, &cl)) { txt_close(&t); seterr("short %s", path); return E_IO; }
      fd->sp[is].cl_PP[k] = cl;
    }
    txt_close(&t);
  }
  return OK;
}

/* read_Fdata_3c (e.FDATA/M_Fdata_3c.f90:143-264) */
static int read_fdata_3c(or_fdata *fd, const char *dir) {
  char path[1024], tok[12][64];
  for (int is = 1; is <= fd->nspecies; is++)
    for (int js = 1; js <= fd->nspecies; js++)
      for (int ks = 1; ks <= fd->nspecies; ks++) {
        bundle3c *b = &fd->b3[is][js][ks];
        txt t;
        snprintf(path, sizeof path, "%s/3c.%02d.%02d.%02d.dat", dir, fd->sp[is].nZ, fd->sp[js].nZ, fd->sp[ks].nZ);
        if (txt_open(&t, path)) return E_IO;
        if (read_ints(&t, 1, &b->ncell) || b->ncell < 1) { txt_close(&t); seterr("bad %s", path); return E_IO; }
        txt_close(&t);
        b->cells = (cell3c *)calloc((size_t)b->ncell, sizeof(cell3c));
        for (int a = 0; a <= P_MAXTYPE3; a++)
          for (int c = 0; c <= P_MAXSUB3; c++)
            for (int d = 0; d <= P_MAXTHETA; d++) b->index[a][c][d] = -1;
        snprintf(path, sizeof path, "%s/3c.%02d.%02d.%02d.dir", dir, fd->sp[is].nZ, fd->sp[js].nZ, fd->sp[ks].nZ);
        txt tdir;
        if (txt_open(&tdir, path)) return E_IO;
        unit_t u13 = {0};
        for (int icell = 1; icell <= b->ncell; icell++) {
          cell3c *c = &b->cells[icell - 1];
          if (txt_read(&tdir, 10, tok) != 10) { seterr("short %s", path); txt_close(&tdir); return E_IO; }
          int iindex = atoi(tok[0]), itype = atoi(tok[1]), isub = atoi(tok[2]), ith = atoi(tok[3]);
          c->nME = atoi(tok[5]);
          c->nx = atoi(tok[6]);
          c->xmax = tok_d(tok[7]);
          c->ny = atoi(tok[8]);
          c->ymax = tok_d(tok[9]);
          if (itype < 1 || itype > P_MAXTYPE3 || isub < 0 || isub > P_MAXSUB3 || ith < 1 ||
              ith > P_MAXTHETA || c->nME < 1 || c->nME > 128 || c->nx < 4 || c->ny < 4) {
            seterr("bad dir entry in %s", path); txt_close(&tdir); return E_IO;
          }
          size_t n = (size_t)c->nx * c->ny * c->nME;
          c->F = (double *)malloc(sizeof(double) * n);
          c->mu = (int *)malloc(sizeof(int) * c->nME);
          c->nu = (int *)malloc(sizeof(int) * c->nME);
          c->mvalue = (int *)malloc(sizeof(int) * c->nME);
          b->index[itype][isub][ith] = iindex;          /* :221 */
          char dpath[1200];
          snprintf(dpath, sizeof dpath, "%s/%s", dir, tok[4]);
          txt td;
          if (txt_open(&td, dpath)) { txt_close(&tdir); return E_IO; }
          double row[128];
          for (int iy = 1; iy <= c->ny; iy++)           /* :227-231 */
            for (int ix = 1; ix <= c->nx; ix++) {
              if (read_dbls(&td, c->nME, row)) { seterr("short data %s", dpath); txt_close(&td); txt_close(&tdir); return E_IO; }
              for (int m = 0; m < c->nME; m++)
                c->F[(ix - 1) + (size_t)c->nx * ((iy - 1) + (size_t)c->ny * m)] = row[m];
            }
          txt_close(&td);
          snprintf(dpath, sizeof dpath, "%s/%02d_munu_3c.%02d.%02d.%02d.dat", dir, itype, fd->sp[is].nZ,
                   fd->sp[js].nZ, fd->sp[ks].nZ);
          if (unit_open(&u13, dpath) || read_ints(&u13.t, c->nME, c->mu) ||
              read_ints(&u13.t, c->nME, c->nu) || read_ints(&u13.t, c->nME, c->mvalue)) {
            seterr("bad munu %s", dpath); unit_close(&u13); txt_close(&tdir); return E_IO;
          }
        }
        txt_close(&tdir);
        unit_close(&u13);
      }
  return OK;
}

/* read_Fdata_1c (e.FDATA/M_Fdata_1c_McWEDA_Harris.f90:99-136): vxc_1c.ZZ.dat
 * holds nssh records of E(issh, :) then nssh records of V(issh, :).  The
 * file is optional here: only the McWEDA assembler reads it. */
static int read_fdata_1c(or_fdata *fd, const char *dir) {
  for (int k = 1; k <= fd->nspecies; k++) {
    species_t *sp = &fd->sp[k];
    char path[1024];
    txt t;
    snprintf(path, sizeof path, "%s/vxc_1c.%02d.dat", dir, sp->nZ);
    sp->have_vxc1c = 0;
    FILE *f = fopen(path, "rb");
    if (!f) continue;
    fclose(f);
    if (txt_open(&t, path)) return E_IO;
    int n = sp->nssh, bad = 0;
    for (int a = 0; a < n && !bad; a++) bad = read_dbls(&t, n, &sp->vxc1c_E[a * MAXSH]);
    for (int a = 0; a < n && !bad; a++) bad = read_dbls(&t, n, &sp->vxc1c_V[a * MAXSH]);
    txt_close(&t);
    if (bad) { seterr("parse error in %s", path); return E_IO; }
    sp->have_vxc1c = 1;
  }
  return OK;
}

or_fdata *or_load_fdata(const char *dir, int nspecies, const int *nZ, char *err, int errlen) {
  if (nspecies < 1 || nspecies > MAXSP) {
    if (err) snprintf(err, (size_t)errlen, "nspecies out of range");
    return NULL;
  }
  or_fdata *fd = (or_fdata *)calloc(1, sizeof(or_fdata));
  fd->nspecies = nspecies;
  int st = read_info(fd, dir, nZ);
  if (!st) st = read_fdata_2c(fd, dir);
  if (!st) st = read_fdata_3c(fd, dir);
  if (!st) st = read_fdata_1c(fd, dir);
  if (st) {
    if (err) snprintf(err, (size_t)errlen, "%s", g_err);
    or_free_fdata(fd);
    return NULL;
  }
  return fd;
}

void or_free_fdata(or_fdata *fd) {
  if (!fd) return;
  for (int a = 1; a <= fd->nspecies; a++)
    for (int b = 1; b <= fd->nspecies; b++) {
      bundle2c *B = &fd->b2[a][b];
      for (int k = 0; B->cells && k < B->ncell; k++) {
        free(B->cells[k].F); free(B->cells[k].mu); free(B->cells[k].nu); free(B->cells[k].mvalue);
      }
      free(B->cells);
      for (int c = 1; c <= fd->nspecies; c++) {
        bundle3c *C = &fd->b3[a][b][c];
        for (int k = 0; C->cells && k < C->ncell; k++) {
          free(C->cells[k].F); free(C->cells[k].mu); free(C->cells[k].nu); free(C->cells[k].mvalue);
        }
        free(C->cells);
      }
    }
  free(fd);
}

int or_species_norb(const or_fdata *fd, int isp) { return fd->sp[isp].norb_max; }

/* ------------------------------------------------------------------------ */
/* interpolators                                                             */
/* ------------------------------------------------------------------------ */
static cell2c *get_cell2c(or_fdata *fd, int isp, int jsp, int iint, int isub) {
  bundle2c *b = &fd->b2[isp][jsp];
  if (iint < 1 || iint > P_MAXTYPE2 || isub < 0 || isub > P_MAXSUB2) return NULL;
  int k = b->index[iint][isub];
  if (k < 1 || k > b->ncell) return NULL;
  return &b->cells[k - 1];
}

/* getMEs_Fdata_2c (e.FDATA/M_Fdata_2c.f90:302-415) */
int or_getMEs_2c(or_fdata *fd, int isp, int jsp, int iint, int isub, double x, int norb_mu, int norb_nu,
                 double *hmbox) {
  const double P_tolerance = 1.0e-5;
  cell2c *c = get_cell2c(fd, isp, jsp, iint, isub);
  if (!c) { seterr("missing 2c cell (%d,%d) for species %d,%d", iint, isub, isp, jsp); return E_TABLE; }
  double Fdata[128], xx[7], pdenom[7];
  if (x < 0.0) { seterr("negative x"); return E_XNEG; }            /* :347-348 */
  if (x > c->xmax * (1.0 + P_tolerance)) {                          /* :349-353 */
    seterr("x too large: x=%.17g xmax=%.17g", x, c->xmax);
    return E_XLARGE;
  }
  /* :354-362 the x < tolerance branch fills hmbox but falls through, so the
   * interpolation below overwrites it; nothing to do here */
  int imid = (int)(x / c->dx) + 1;                                  /* :366-375 */
  int ileft = imid - 3, iright = imid + 3;
  if (ileft < 1) { ileft = 1; iright = 7; }
  else if (iright > c->nx) { ileft = c->nx - 6; iright = c->nx; }
  for (int ip = ileft; ip <= iright; ip++) xx[ip - ileft] = (double)(ip - 1) * c->dx;
  for (int m = 0; m < c->nME; m++) Fdata[m] = 0.0;
  for (int isum = ileft; isum <= iright; isum++) {                  /* :382-393 */
    double prod = 1.0;
    pdenom[isum - ileft] = 1.0;
    for (int iprod = ileft; iprod <= iright; iprod++) {
      if (iprod != isum) {
        double pden = 1.0 / (xx[isum - ileft] - xx[iprod - ileft]);
        pdenom[isum - ileft] = pdenom[isum - ileft] * pden;
        prod = prod * (x - xx[iprod - ileft]) * pden;
      }
    }
    for (int m = 0; m < c->nME; m++) Fdata[m] = Fdata[m] + c->F[(isum - 1) + (size_t)c->nx * m] * prod;
  }
  for (int k = 0; k < norb_mu * norb_nu; k++) hmbox[k] = 0.0;       /* :396-401 */
  for (int m = 0; m < c->nME; m++) {
    int imu = c->mu[m], inu = c->nu[m];
    if (imu < 1 || imu > norb_mu || inu < 1 || inu > norb_nu) { seterr("munu out of block"); return E_TABLE; }
    hmbox[(imu - 1) + norb_mu * (inu - 1)] = Fdata[m];
  }
  return OK;
}

/* getDMEs_Fdata_2c (e.FDATA/M_Fdata_2c.f90:446-600) */
int or_getDMEs_2c(or_fdata *fd, int isp, int jsp, int iint, int isub, double x, int norb_mu, int norb_nu,
                  double *hmbox, double *dhmbox) {
  const double P_tolerance = 1.0e-5;
  cell2c *c = get_cell2c(fd, isp, jsp, iint, isub);
  if (!c) { seterr("missing 2c cell (%d,%d)", iint, isub); return E_TABLE; }
  double Fdata[128], dF[128], xx[7] = {0}, pdenom[7] = {0};
  for (int m = 0; m < c->nME; m++) Fdata[m] = dF[m] = 0.0;
  if (x < 0.0) { seterr("negative x"); return E_XNEG; }
  if (x > c->xmax * (1.0 + P_tolerance)) {
    seterr("x too large: x=%.17g xmax=%.17g", x, c->xmax);
    return E_XLARGE;
  }
  if (x < P_tolerance) {                                            /* :510-520 early return */
    for (int k = 0; k < norb_mu * norb_nu; k++) hmbox[k] = 0.0;
    for (int m = 0; m < c->nME; m++) {
      int imu = c->mu[m], inu = c->nu[m];
      hmbox[(imu - 1) + norb_mu * (inu - 1)] = c->F[0 + (size_t)c->nx * m];
      dhmbox[(imu - 1) + norb_mu * (inu - 1)] = 0.0;
    }
    return OK;
  }
  int imid = (int)(x / c->dx) + 1;
  int ileft = imid - 3, iright = imid + 3;
  if (ileft < 1) { ileft = 1; iright = 7; }
  else if (iright > c->nx) { ileft = c->nx - 6; iright = c->nx; }
  for (int ip = ileft; ip <= iright; ip++) xx[ip - ileft] = (double)(ip - 1) * c->dx;
  for (int isum = ileft; isum <= iright; isum++) {
    double prod = 1.0;
    pdenom[isum - ileft] = 1.0;
    for (int iprod = ileft; iprod <= iright; iprod++) {
      if (iprod != isum) {
        double pden = 1.0 / (xx[isum - ileft] - xx[iprod - ileft]);
        pdenom[isum - ileft] = pdenom[isum - ileft] * pden;
        prod = prod * (x - xx[iprod - ileft]) * pden;
      }
    }
    for (int m = 0; m < c->nME; m++) Fdata[m] = Fdata[m] + c->F[(isum - 1) + (size_t)c->nx * m] * prod;
  }
  for (int k = 0; k < norb_mu * norb_nu; k++) hmbox[k] = 0.0;
  for (int m = 0; m < c->nME; m++) hmbox[(c->mu[m] - 1) + norb_mu * (c->nu[m] - 1)] = Fdata[m];
  for (int m = 0; m < c->nME; m++) dF[m] = 0.0;                     /* :561-577 */
  for (int ip = ileft; ip <= iright; ip++) {
    double xsumoverj = 0.0;
    for (int jp = ileft; jp <= iright; jp++) {
      if (ip == jp) continue;
      double xprod = 1.0;
      for (int kp = ileft; kp <= iright; kp++) {
        if (kp == jp) continue;
        if (kp == ip) continue;
        xprod = xprod * (x - xx[kp - ileft]);
      }
      xsumoverj = xsumoverj + xprod;
    }
    for (int m = 0; m < c->nME; m++)
      dF[m] = dF[m] + c->F[(ip - 1) + (size_t)c->nx * m] * pdenom[ip - ileft] * xsumoverj;
  }
  for (int k = 0; k < norb_mu * norb_nu; k++) dhmbox[k] = 0.0;      /* :580-585 */
  for (int m = 0; m < c->nME; m++) dhmbox[(c->mu[m] - 1) + norb_mu * (c->nu[m] - 1)] = dF[m];
  return OK;
}

static cell3c *get_cell3c(or_fdata *fd, int isp, int jsp, int ksp, int iint, int isub, int ith) {
  bundle3c *b = &fd->b3[isp][jsp][ksp];
  if (iint < 1 || iint > P_MAXTYPE3 || isub < 0 || isub > P_MAXSUB3) return NULL;
  int k = b->index[iint][isub][ith];
  if (k < 1 || k > b->ncell) return NULL;
  return &b->cells[k - 1];
}

#define F3(c, ix, iy, m) ((c)->F[((ix)-1) + (size_t)(c)->nx * (((iy)-1) + (size_t)(c)->ny * (m))])

/* getMEs_Fdata_3c (e.FDATA/M_Fdata_3c.f90:293-517) and getDMEs_Fdata_3c
 * (:549-846) share one body; deriv selects the derivative outputs. */
static int getMEs_3c_body(or_fdata *fd, int isp, int jsp, int ksp, int iint, int isub, double x, double y,
                          int norb_mu, int norb_nu, double cost, double *hmbox, double *dph, double *dxh,
                          double *dyh, int deriv) {
  const double P_tiny = 1.0e-6;
  const double P_small = 1.0 - 4; /* :317 "1.0d0-4" evaluates to -3 */
  double p[5], Dp[5];
  double cost2 = cost * cost;                                       /* :348-354 */
  double sint = sqrt(fmax(1.0e-5, 1.0 - cost2));
  p[0] = 1.0;
  p[1] = cost;
  p[2] = 0.5 * (3.0 * cost2 - 1.0);
  p[3] = 0.5 * cost * (5.0 * cost2 - 3.0);
  p[4] = 0.125 * (3.0 - cost2 * (30.0 - 35.0 * cost2));
  Dp[0] = 0.0;                                                      /* :625-629 */
  Dp[1] = 1.0;
  Dp[2] = 3.0 * cost;
  Dp[3] = (15.0 * cost2 - 3.0) / 2.0;
  Dp[4] = 0.5 * cost * (35.0 * cost2 - 15.0);
  cell3c *c = get_cell3c(fd, isp, jsp, ksp, iint, isub, 1);
  if (!c) { seterr("missing 3c cell"); return E_TABLE; }
  int nME = c->nME;
  double Fd[128], DpF[128], DxF[128], DyF[128], interim[128];
  for (int m = 0; m < nME; m++) Fd[m] = DpF[m] = DxF[m] = DyF[m] = 0.0;
  double dx = c->xmax / (c->nx - 1.0);                              /* :367-379 */
  double dy = c->ymax / (c->ny - 1.0);
  int ix = (int)(x / dx) + 1;
  int iy = (int)(y / dy) + 1;
  if (ix < 2) ix = 2;
  if (iy < 2) iy = 2;
  if (ix > c->nx - 2) ix = c->nx - 2;
  if (iy > c->ny - 2) iy = c->ny - 2;
  double px = x / dx - ix + 1.0;
  double py = y / dy - iy + 1.0;
  double gx = (F3(c, ix + 1, iy, 0) - F3(c, ix, iy, 0)) / dx;      /* :383-385 */
  double gy = (F3(c, ix, iy + 1, 0) - F3(c, ix, iy, 0)) / dy;
  double gg = gx * gx + gy * gy;
  for (int it = 1; it <= P_MAXTHETA; it++) {
    c = get_cell3c(fd, isp, jsp, ksp, iint, isub, it);
    if (!c || c->nME != nME) { seterr("missing 3c theta cell %d", it); return E_TABLE; }
    double pt = p[it - 1], Dpt = Dp[it - 1];
    if (!g_exact && gg < P_tiny) {                                  /* :406-410, :684-691 */
      for (int m = 0; m < nME; m++) {
        interim[m] = ((1.0 - px - py) * F3(c, ix, iy, m) + px * F3(c, ix + 1, iy, m) + py * F3(c, ix, iy + 1, m));
        Fd[m] = Fd[m] + pt * interim[m];
        if (deriv) {
          DpF[m] = DpF[m] + Dpt * interim[m];
          DxF[m] = DxF[m] + pt * gx;
          DyF[m] = DyF[m] + pt * gy;
        }
      }
    } else if (gg <= P_small) {                                     /* :415-422 dead: P_small = -3 */
      for (int m = 0; m < nME; m++) {
        interim[m] = (py * (py - 1) * 0.5 * F3(c, ix, iy - 1, m) + px * (px - 1) * 0.5 * F3(c, ix - 1, iy, m) +
                      (1.0 + px * py - px * px - py * py) * F3(c, ix, iy, m) +
                      px * (px - 2.0 * py + 1.0) * 0.5 * F3(c, ix + 1, iy, m) +
                      py * (py - 2.0 * px + 1.0) * 0.5 * F3(c, ix, iy + 1, m) + px * py * F3(c, ix + 1, iy + 1, m));
        Fd[m] = Fd[m] + pt * interim[m];
        if (deriv) {
          DpF[m] = DpF[m] + Dpt * interim[m];
          DxF[m] = DxF[m] + pt * (((F3(c, ix + 1, iy + 1, m) - F3(c, ix + 1, iy, m) - F3(c, ix, iy + 1, m) +
                                    F3(c, ix, iy, m)) * py +
                                   (F3(c, ix - 1, iy, m) + F3(c, ix + 1, iy, m) - 2.0 * F3(c, ix, iy, m)) * px -
                                   0.5 * (F3(c, ix - 1, iy, m) - F3(c, ix + 1, iy, m))) / dx);
          DyF[m] = DyF[m] + pt * (((F3(c, ix + 1, iy + 1, m) - F3(c, ix + 1, iy, m) - F3(c, ix, iy + 1, m) +
                                    F3(c, ix, iy, m)) * px +
                                   (F3(c, ix, iy - 1, m) + F3(c, ix, iy + 1, m) - 2.0 * F3(c, ix, iy, m)) * py -
                                   0.5 * (F3(c, ix, iy - 1, m) - F3(c, ix, iy + 1, m))) / dy);
        }
      }
    } else {                                                        /* :425-481, :721-798 */
      for (int m = 0; m < nME; m++) {
        double g[4], gp[4], f1m1, f1m2, f1m3, f0p3, f0p6, f1p3, f1p6, f2p1, bb0, bb1, bb2, bb3;
        for (int k = -1; k <= 2; k++) {
          f1m1 = F3(c, ix + k, iy - 1, m);
          f1m2 = 2.0 * f1m1;
          f1m3 = 3.0 * f1m1;
          f0p3 = 3.0 * F3(c, ix + k, iy, m);
          f0p6 = 2.0 * f0p3;
          f1p3 = 3.0 * F3(c, ix + k, iy + 1, m);
          f1p6 = 2.0 * f1p3;
          f2p1 = F3(c, ix + k, iy + 2, m);
          bb3 = -f1m1 + f0p3 - f1p3 + f2p1;
          bb2 = f1m3 - f0p6 + f1p3;
          bb1 = -f1m2 - f0p3 + f1p6 - f2p1;
          bb0 = f0p6;
          g[k + 1] = ((bb3 * py + bb2) * py + bb1) * py + bb0;
          gp[k + 1] = ((3 * bb3 * py + 2 * bb2) * py + bb1);
        }
        f1m1 = g[0];
        f1m2 = 2.0 * f1m1;
        f1m3 = 3.0 * f1m1;
        f0p3 = 3.0 * g[1];
        f0p6 = 2.0 * f0p3;
        f1p3 = 3.0 * g[2];
        f1p6 = 2.0 * f1p3;
        f2p1 = g[3];
        bb3 = -f1m1 + f0p3 - f1p3 + f2p1;
        bb2 = f1m3 - f0p6 + f1p3;
        bb1 = -f1m2 - f0p3 + f1p6 - f2p1;
        bb0 = f0p6;
        interim[m] = (((bb3 * px + bb2) * px + bb1) * px + bb0) / 36.0;
        Fd[m] = Fd[m] + pt * interim[m];
        if (deriv) {
          DpF[m] = DpF[m] + Dpt * interim[m];
          DxF[m] = DxF[m] + pt * ((3 * bb3 * px + 2 * bb2) * px + bb1) / (36.0 * dx);
          f1m1 = gp[0];
          f1m2 = 2 * f1m1;
          f1m3 = 3 * f1m1;
          f0p3 = 3 * gp[1];
          f0p6 = 2 * f0p3;
          f1p3 = 3 * gp[2];
          f1p6 = 2 * f1p3;
          f2p1 = gp[3];
          bb3 = -f1m1 + f0p3 - f1p3 + f2p1;
          bb2 = f1m3 - f0p6 + f1p3;
          bb1 = -f1m2 - f0p3 + f1p6 - f2p1;
          bb0 = f0p6;
          DyF[m] = DyF[m] + pt * (((bb3 * px + bb2) * px + bb1) * px + bb0) / (36.0 * dy);
        }
      }
    }
  }
  /* recover matrices (:497-507, :814-833); nME and the maps are taken from
   * the last theta cell */
  int nb = norb_mu * norb_nu;
  for (int k = 0; k < nb; k++) {
    hmbox[k] = 0.0;
    if (deriv) dph[k] = dxh[k] = dyh[k] = 0.0;
  }
  for (int m = 0; m < c->nME; m++) {
    int imu = c->mu[m], inu = c->nu[m];
    if (imu < 1 || imu > norb_mu || inu < 1 || inu > norb_nu) { seterr("munu out of block"); return E_TABLE; }
    int k = (imu - 1) + norb_mu * (inu - 1);
    if (c->mvalue[m] != 1) {
      hmbox[k] = Fd[m];
      if (deriv) { dph[k] = DpF[m]; dxh[k] = DxF[m]; dyh[k] = DyF[m]; }
    } else {
      hmbox[k] = Fd[m] * sint;
      if (deriv) {
        dph[k] = DpF[m] * sint - cost * Fd[m] / sint;
        dxh[k] = DxF[m] * sint;
        dyh[k] = DyF[m] * sint;
      }
    }
  }
  return OK;
}

int or_getMEs_3c(or_fdata *fd, int isp, int jsp, int ksp, int iint, int isub, double x, double y, int norb_mu,
                 int norb_nu, double cost, double *hmbox) {
  return getMEs_3c_body(fd, isp, jsp, ksp, iint, isub, x, y, norb_mu, norb_nu, cost, hmbox, NULL, NULL, NULL, 0);
}
int or_getDMEs_3c(or_fdata *fd, int isp, int jsp, int ksp, int iint, int isub, double x, double y, int norb_mu,
                  int norb_nu, double cost, double *hmbox, double *dph, double *dxh, double *dyh) {
  return getMEs_3c_body(fd, isp, jsp, ksp, iint, isub, x, y, norb_mu, norb_nu, cost, hmbox, dph, dxh, dyh, 1);
}

/* ------------------------------------------------------------------------ */
/* vector helpers: distance (b.FUNCTIONS/distance.f90:51-80), magnitude      */
/* (magnitude.f90:50-77), a_cross_b (a_cross_b.f90:49-79)                     */
/* ------------------------------------------------------------------------ */
static double distance3(const double *a, const double *b) {
  return sqrt((b[0] - a[0]) * (b[0] - a[0]) + (b[1] - a[1]) * (b[1] - a[1]) + (b[2] - a[2]) * (b[2] - a[2]));
}
static double magnitude3(const double *a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
static void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

/* eps and deps storage: eps[i + 3*j] = spe(i+1, j+1);                       */
/* deps[ix + 3*(imu + 3*k)] = deps(ix+1, imu+1, k+1)                          */
#define E2(a, i, j) (a)[(i) + 3 * (j)]
#define E3(a, i, j, k) (a)[(i) + 3 * ((j) + 3 * (k))]

/* epsilon_function (b.FUNCTIONS/epsilon.f90:73-202); the WARNINGS-file side
 * effects are not reproduced */
void or_epsilon(const double *r1, const double *r2, double *spe) {
  double r1_mag = magnitude3(r1), r2_mag = magnitude3(r2);
  double r1_hat[3], xp[3], yp[3] = {0, 0, 0}, zp[3], yp_mag;
  if (r2_mag < 1.0e-4) {                                            /* :123-133 */
    for (int k = 0; k < 9; k++) spe[k] = 0.0;
    for (int k = 0; k < 3; k++) E2(spe, k, k) = 1.0;
    return;
  }
  for (int k = 0; k < 3; k++) zp[k] = r2[k] / r2_mag;
  yp_mag = 0;
  if (r1_mag > 1.0e-4) {                                            /* :139-145 */
    for (int k = 0; k < 3; k++) r1_hat[k] = r1[k] / r1_mag;
    cross3(zp, r1_hat, yp);
    yp_mag = magnitude3(yp);
  }
  if (yp_mag < 1.0e-4) {                                            /* :148-168 */
    if (fabs(zp[0]) > 1.0e-4) {
      yp[0] = -(zp[1] + zp[2]) / zp[0];
      yp[1] = 1.0;
      yp[2] = 1.0;
    } else if (fabs(zp[1]) > 1.0e-4) {
      yp[0] = 1.0;
      yp[1] = -(zp[0] + zp[2]) / zp[1];
      yp[2] = 1.0;
    } else {
      yp[0] = 1.0;
      yp[1] = 1.0;
      yp[2] = -(zp[0] + zp[1]) / zp[2];
    }
    yp_mag = magnitude3(yp);
  }
  for (int k = 0; k < 3; k++) yp[k] = yp[k] / yp_mag;
  cross3(yp, zp, xp);
  for (int k = 0; k < 3; k++) {
    E2(spe, k, 0) = xp[k];
    E2(spe, k, 1) = yp[k];
    E2(spe, k, 2) = zp[k];
  }
}

/* constants.h:18-21 (delk), :24-28 (xlevi) */
static double delk(int i, int j) { return i == j ? 1.0 : 0.0; }
static double xlevi(int i, int j, int k) {
  if (i == j || j == k || i == k) return 0.0;
  if ((i == 0 && j == 1 && k == 2) || (i == 1 && j == 2 && k == 0) || (i == 2 && j == 0 && k == 1)) return 1.0;
  return -1.0;
}

/* Depsilon_2c (b.FUNCTIONS/Depsilon_2c.f90:46-140) */
void or_depsilon_2c(const double *r1, const double *r2, double z, const double *eps, double *deps) {
  for (int k = 0; k < 27; k++) deps[k] = 0.0;
  if (z < 1.0e-5) return;
  double crossa[3];
  crossa[0] = r2[1] * r1[2] - r2[2] * r1[1];
  crossa[1] = r2[2] * r1[0] - r2[0] * r1[2];
  crossa[2] = r2[0] * r1[1] - r2[1] * r1[0];
  double crossmag = sqrt(crossa[0] * crossa[0] + crossa[1] * crossa[1] + crossa[2] * crossa[2]);
  if (fabs(crossmag) < 1.0e-3) return;
  double r2mag2 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
  double r1dotr2 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
  for (int ix = 0; ix < 3; ix++)
    for (int imu = 0; imu < 3; imu++) {
      double sum = xlevi(ix, imu, 0) * r2[0] + xlevi(ix, imu, 1) * r2[1] + xlevi(ix, imu, 2) * r2[2];
      E3(deps, ix, imu, 0) = (E2(eps, imu, 0) * E2(eps, ix, 2) * (1.0 / z)) -
                             (E2(eps, imu, 0) * (1.0 / crossmag) * (1.0 / crossmag)) *
                                 (r2mag2 * r1[ix] - r1dotr2 * r2[ix]) +
                             (1.0 / z) * (1.0 / crossmag) *
                                 (delk(imu, ix) * (r2mag2 - r1dotr2) - r1[imu] * r2[ix] - r2[imu] * r2[ix] +
                                  2.0 * r1[ix] * r2[imu]);
      E3(deps, ix, imu, 1) =
          (1.0 / crossmag) * (sum + (E2(eps, imu, 1) * (1.0 / crossmag)) * (r1dotr2 * r2[ix] - r2mag2 * r1[ix]));
      E3(deps, ix, imu, 2) = -(delk(imu, ix) - E2(eps, imu, 2) * E2(eps, ix, 2)) * (1.0 / z);
    }
}

/* Depsilon_3c (b.FUNCTIONS/Depsilon_3c.f90:49-189) */
void or_depsilon_3c(const double *r1, const double *r2, const double *r21, double z, const double *ratm,
                    const double *rnabc, const double *eps3, double *dera3, double *der13) {
  for (int k = 0; k < 27; k++) dera3[k] = der13[k] = 0.0;
  double crossa[3];
  crossa[0] = r21[1] * rnabc[2] - r21[2] * rnabc[1];
  crossa[1] = r21[2] * rnabc[0] - r21[0] * rnabc[2];
  crossa[2] = r21[0] * rnabc[1] - r21[1] * rnabc[0];
  double crossmag = sqrt(crossa[0] * crossa[0] + crossa[1] * crossa[1] + crossa[2] * crossa[2]);
  if (fabs(crossmag) < 1.0e-3) return;
  double r2mag2 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
  double r1mag2 = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
  double ratmmag2 = ratm[0] * ratm[0] + ratm[1] * ratm[1] + ratm[2] * ratm[2];
  double r1dotr2 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
  double r2dotratm = r2[0] * ratm[0] + r2[1] * ratm[1] + r2[2] * ratm[2];
  double r1dotratm = r1[0] * ratm[0] + r1[1] * ratm[1] + r1[2] * ratm[2];
  for (int ix = 0; ix < 3; ix++)
    for (int imu = 0; imu < 3; imu++) {
      E3(dera3, ix, imu, 2) = 0.0;
      double sum = xlevi(ix, imu, 0) * (r2[0] - r1[0]) + xlevi(ix, imu, 1) * (r2[1] - r1[1]) +
                   xlevi(ix, imu, 2) * (r2[2] - r1[2]);
      E3(dera3, ix, imu, 1) =
          (1.0 / crossmag) *
          (sum - (E2(eps3, imu, 1) / crossmag) * ((r1mag2 + r2mag2 - 2.0 * r1dotr2) * ratm[ix] +
                                                  (r1dotr2 - r1mag2 - r2dotratm + r1dotratm) * r2[ix] +
                                                  (r1dotr2 - r2mag2 + r2dotratm - r1dotratm) * r1[ix]));
    }
  for (int a = 0; a < 3; a++) {
    E3(dera3, a, 0, 0) = E2(eps3, 2, 2) * E3(dera3, a, 1, 1) - E2(eps3, 1, 2) * E3(dera3, a, 2, 1);
    E3(dera3, a, 1, 0) = E2(eps3, 0, 2) * E3(dera3, a, 2, 1) - E2(eps3, 2, 2) * E3(dera3, a, 0, 1);
    E3(dera3, a, 2, 0) = E2(eps3, 1, 2) * E3(dera3, a, 0, 1) - E2(eps3, 0, 2) * E3(dera3, a, 1, 1);
  }
  for (int ix = 0; ix < 3; ix++)
    for (int imu = 0; imu < 3; imu++) {
      E3(der13, ix, imu, 2) = (1.0 / z) * (E2(eps3, imu, 2) * E2(eps3, ix, 2) - delk(imu, ix));
      double sum = xlevi(ix, imu, 0) * (ratm[0] - r2[0]) + xlevi(ix, imu, 1) * (ratm[1] - r2[1]) +
                   xlevi(ix, imu, 2) * (ratm[2] - r2[2]);
      E3(der13, ix, imu, 1) =
          (1.0 / crossmag) *
          (sum - (E2(eps3, imu, 1) / crossmag) * ((r2dotratm - r1dotratm + r1dotr2 - r2mag2) * ratm[ix] +
                                                  (r2dotratm + r1dotratm - r1dotr2 - ratmmag2) * r2[ix] +
                                                  (ratmmag2 - 2.0 * r2dotratm + r2mag2) * r1[ix]));
    }
  for (int a = 0; a < 3; a++) {
    E3(der13, a, 0, 0) = E2(eps3, 2, 2) * E3(der13, a, 1, 1) - E2(eps3, 2, 1) * E3(der13, a, 1, 2) -
                         E2(eps3, 1, 2) * E3(der13, a, 2, 1) + E2(eps3, 1, 1) * E3(der13, a, 2, 2);
    E3(der13, a, 1, 0) = E2(eps3, 0, 2) * E3(der13, a, 2, 1) - E2(eps3, 0, 1) * E3(der13, a, 2, 2) -
                         E2(eps3, 2, 2) * E3(der13, a, 0, 1) + E2(eps3, 2, 1) * E3(der13, a, 0, 2);
    E3(der13, a, 2, 0) = E2(eps3, 1, 2) * E3(der13, a, 0, 1) - E2(eps3, 1, 1) * E3(der13, a, 0, 2) -
                         E2(eps3, 0, 2) * E3(der13, a, 1, 1) + E2(eps3, 0, 1) * E3(der13, a, 1, 2);
  }
}

/* ------------------------------------------------------------------------ */
/* rotations: twister/chooser (c.SYSTEM/M_rotations.f90:221-382), rotate     */
/* (:98-177), Dtwister/Dchooser/Dmatrix/Drotate (M_Drotations.f90:102-482)   */
/* ------------------------------------------------------------------------ */
/* amat(3,3,5) of include/constants.h:30-38, stored amat[imu][ix][jx] */
static double amat(int ix, int jx, int imu) {
  static const double v = 0.28867513459481287; /* 1/(2*sqrt(3)) */
  switch (imu) {
  case 0: return ((ix == 0 && jx == 1) || (ix == 1 && jx == 0)) ? 0.5 : 0.0;
  case 1: return ((ix == 1 && jx == 2) || (ix == 2 && jx == 1)) ? 0.5 : 0.0;
  case 2: return (ix == jx) ? (ix == 2 ? 2.0 * v : -v) : 0.0;
  case 3: return ((ix == 0 && jx == 2) || (ix == 2 && jx == 0)) ? 0.5 : 0.0;
  case 4: return (ix == jx && ix < 2) ? (ix == 0 ? 0.5 : -0.5) : 0.0;
  }
  return 0.0;
}

/* dmat[a + 5*b] = dmat(a+1, b+1); pmat[a + 3*b] = pmat(a+1,b+1) */
static void twister(const double *eps, int have_d, double *dmat, double *pmat) {
  pmat[0 + 3 * 0] = E2(eps, 1, 1);
  pmat[0 + 3 * 1] = E2(eps, 1, 2);
  pmat[0 + 3 * 2] = E2(eps, 1, 0);
  pmat[1 + 3 * 0] = E2(eps, 2, 1);
  pmat[1 + 3 * 1] = E2(eps, 2, 2);
  pmat[1 + 3 * 2] = E2(eps, 2, 0);
  pmat[2 + 3 * 0] = E2(eps, 0, 1);
  pmat[2 + 3 * 1] = E2(eps, 0, 2);
  pmat[2 + 3 * 2] = E2(eps, 0, 0);
  if (!have_d) return;
  for (int imu = 0; imu < 5; imu++) {
    double l11 = 0, l12 = 0, l13 = 0, l32 = 0, l33 = 0;
    for (int jx = 0; jx < 3; jx++)
      for (int ix = 0; ix < 3; ix++) {
        double a = amat(ix, jx, imu);
        if (a != 0.0) {
          l11 = l11 + a * E2(eps, jx, 0) * E2(eps, ix, 0);
          l12 = l12 + a * E2(eps, jx, 0) * E2(eps, ix, 1);
          l13 = l13 + a * E2(eps, jx, 0) * E2(eps, ix, 2);
          l32 = l32 + a * E2(eps, jx, 2) * E2(eps, ix, 1);
          l33 = l33 + a * E2(eps, jx, 2) * E2(eps, ix, 2);
        }
      }
    dmat[imu + 5 * 0] = 2.0 * l12;
    dmat[imu + 5 * 1] = 2.0 * l32;
    dmat[imu + 5 * 2] = sqrt(3.0) * l33;
    dmat[imu + 5 * 3] = 2.0 * l13;
    dmat[imu + 5 * 4] = 2.0 * l11 + l33;
  }
}

/* chooser: rm[a + 5*b] */
static void chooser(int l, const double *dmat, const double *pmat, double *rm) {
  for (int k = 0; k < 25; k++) rm[k] = 0.0;
  if (l == 0) rm[0] = 1.0;
  else if (l == 1) {
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) rm[a + 5 * b] = pmat[a + 3 * b];
  } else if (l == 2) {
    for (int k = 0; k < 25; k++) rm[k] = dmat[k];
  }
}

/* rotate (M_rotations.f90:98-177) with the shells of in1 on the left and
 * the shell list (n2sh, l2s) on the right: the basis of in3, or the
 * projector shells for rotate_PP (c.SYSTEM/rotate_PP.f90:60-156) */
static void rotate_shells(or_fdata *fd, int in1, int n2sh, const int *l2s, int have_d, const double *eps,
                          int norb_mu, int norb_nu, const double *mm, double *xm) {
  double dmat[25] = {0}, pmat[9], left[25], right[25];
  twister(eps, have_d, dmat, pmat);
  for (int k = 0; k < norb_mu * norb_nu; k++) xm[k] = 0.0;
  int n1 = 0;
  for (int issh = 0; issh < fd->sp[in1].nssh; issh++) {
    int l1 = fd->sp[in1].lssh[issh];
    chooser(l1, dmat, pmat, left);
    int n2 = 0;
    for (int jssh = 0; jssh < n2sh; jssh++) {
      int l2 = l2s[jssh];
      chooser(l2, dmat, pmat, right);
      for (int m2 = 0; m2 < 2 * l2 + 1; m2++)
        for (int m1 = 0; m1 < 2 * l1 + 1; m1++)
          for (int k2 = 0; k2 < 2 * l2 + 1; k2++)
            for (int k1 = 0; k1 < 2 * l1 + 1; k1++)
              xm[(n1 + k1) + norb_mu * (n2 + k2)] = xm[(n1 + k1) + norb_mu * (n2 + k2)] +
                                                    left[k1 + 5 * m1] * mm[(n1 + m1) + norb_mu * (n2 + m2)] *
                                                        right[k2 + 5 * m2];
      n2 += 2 * l2 + 1;
    }
    n1 += 2 * l1 + 1;
  }
}

void or_rotate(or_fdata *fd, int in1, int in3, const double *eps, int norb_mu, int norb_nu, const double *mm,
               double *xm) {
  rotate_shells(fd, in1, fd->sp[in3].nssh, fd->sp[in3].lssh, fd->have_dorbitals, eps, norb_mu, norb_nu, mm, xm);
}

static void rotate_pp(or_fdata *fd, int in1, int in2, const double *eps, int norb_mu, int norb_nu, const double *mm,
                      double *xm) {
  rotate_shells(fd, in1, fd->sp[in2].nssh_PP, fd->sp[in2].lssh_PP, fd->have_dorbitals || fd->have_dorbitals_PP, eps,
                norb_mu, norb_nu, mm, xm);
}

/* Dtwister: Ddmat[ix + 3*(a + 5*b)], Dpmat[ix + 3*(a + 3*b)] */
static void dtwister(const double *eps, const double *deps, double *Ddmat, double *Dpmat) {
  for (int k = 0; k < 3; k++) {
    Dpmat[k + 3 * (0 + 3 * 0)] = E3(deps, k, 1, 1);
    Dpmat[k + 3 * (0 + 3 * 1)] = E3(deps, k, 1, 2);
    Dpmat[k + 3 * (0 + 3 * 2)] = E3(deps, k, 1, 0);
    Dpmat[k + 3 * (1 + 3 * 0)] = E3(deps, k, 2, 1);
    Dpmat[k + 3 * (1 + 3 * 1)] = E3(deps, k, 2, 2);
    Dpmat[k + 3 * (1 + 3 * 2)] = E3(deps, k, 2, 0);
    Dpmat[k + 3 * (2 + 3 * 0)] = E3(deps, k, 0, 1);
    Dpmat[k + 3 * (2 + 3 * 1)] = E3(deps, k, 0, 2);
    Dpmat[k + 3 * (2 + 3 * 2)] = E3(deps, k, 0, 0);
  }
  for (int imu = 0; imu < 5; imu++)
    for (int kx = 0; kx < 3; kx++) {
      double a12 = 0, a32 = 0, a33 = 0, a13 = 0, a11 = 0;
      for (int ix = 0; ix < 3; ix++)
        for (int jx = 0; jx < 3; jx++) {
          double a = amat(jx, ix, imu);
          if (a != 0.0) {
            a12 = a12 + a * (E3(deps, kx, ix, 0) * E2(eps, jx, 1) + E2(eps, ix, 0) * E3(deps, kx, jx, 1));
            a32 = a32 + a * (E3(deps, kx, ix, 2) * E2(eps, jx, 1) + E2(eps, ix, 2) * E3(deps, kx, jx, 1));
            a33 = a33 + a * (E3(deps, kx, ix, 2) * E2(eps, jx, 2) + E2(eps, ix, 2) * E3(deps, kx, jx, 2));
            a13 = a13 + a * (E3(deps, kx, ix, 0) * E2(eps, jx, 2) + E2(eps, ix, 0) * E3(deps, kx, jx, 2));
            a11 = a11 + a * (E3(deps, kx, ix, 0) * E2(eps, jx, 0) + E2(eps, ix, 0) * E3(deps, kx, jx, 0));
          }
        }
      Ddmat[kx + 3 * (imu + 5 * 0)] = 2.0 * a12;
      Ddmat[kx + 3 * (imu + 5 * 1)] = 2.0 * a32;
      Ddmat[kx + 3 * (imu + 5 * 2)] = sqrt(3.0) * a33;
      Ddmat[kx + 3 * (imu + 5 * 3)] = 2.0 * a13;
      Ddmat[kx + 3 * (imu + 5 * 4)] = 2.0 * a11 + a33;
    }
}

static void dchooser(int l, const double *Ddmat, const double *Dpmat, double *Dm) {
  for (int k = 0; k < 75; k++) Dm[k] = 0.0;
  if (l == 1) {
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++)
        for (int x = 0; x < 3; x++) Dm[x + 3 * (a + 5 * b)] = Dpmat[x + 3 * (a + 3 * b)];
  } else if (l == 2) {
    for (int k = 0; k < 75; k++) Dm[k] = Ddmat[k];
  }
}

/* Drotate = twister + Dtwister + Dmatrix; matm (norb_mu,norb_nu), Dmatm and
 * Dmatx (3,norb_mu,norb_nu) */
static void drotate_shells(or_fdata *fd, int in1, int n2sh, const int *l2s, int have_d, const double *eps,
                           const double *deps, int norb_mu, int norb_nu, const double *matm, const double *Dmatm,
                           double *term) {
  double dmat[25] = {0}, pmat[9], Ddmat[75], Dpmat[27];
  double left[25], right[25], Dleft[75], Dright[75];
  twister(eps, have_d, dmat, pmat);
  dtwister(eps, deps, Ddmat, Dpmat);
  int n1 = 0;
  for (int issh = 0; issh < fd->sp[in1].nssh; issh++) {
    int l1 = fd->sp[in1].lssh[issh];
    chooser(l1, dmat, pmat, left);
    dchooser(l1, Ddmat, Dpmat, Dleft);
    int n2 = 0;
    for (int jssh = 0; jssh < n2sh; jssh++) {
      int l2 = l2s[jssh];
      chooser(l2, dmat, pmat, right);
      dchooser(l2, Ddmat, Dpmat, Dright);
      for (int k2 = 0; k2 < 2 * l2 + 1; k2++)
        for (int k1 = 0; k1 < 2 * l1 + 1; k1++)
          for (int x = 0; x < 3; x++) term[x + 3 * ((n1 + k1) + norb_mu * (n2 + k2))] = 0.0;
      for (int m2 = 0; m2 < 2 * l2 + 1; m2++)
        for (int k2 = 0; k2 < 2 * l2 + 1; k2++)
          for (int m1 = 0; m1 < 2 * l1 + 1; m1++)
            for (int k1 = 0; k1 < 2 * l1 + 1; k1++)
              for (int x = 0; x < 3; x++) {
                double mv = matm[(n1 + m1) + norb_mu * (n2 + m2)];
                size_t ko = x + 3 * ((n1 + k1) + norb_mu * (n2 + k2));
                term[ko] = term[ko] + Dleft[x + 3 * (k1 + 5 * m1)] * right[k2 + 5 * m2] * mv +
                           left[k1 + 5 * m1] * Dright[x + 3 * (k2 + 5 * m2)] * mv +
                           left[k1 + 5 * m1] * right[k2 + 5 * m2] * Dmatm[x + 3 * ((n1 + m1) + norb_mu * (n2 + m2))];
              }
      n2 += 2 * l2 + 1;
    }
    n1 += 2 * l1 + 1;
  }
}

static void drotate(or_fdata *fd, int in1, int in2, const double *eps, const double *deps, int norb_mu,
                    int norb_nu, const double *matm, const double *Dmatm, double *term) {
  drotate_shells(fd, in1, fd->sp[in2].nssh, fd->sp[in2].lssh, fd->have_dorbitals, eps, deps, norb_mu, norb_nu, matm,
                 Dmatm, term);
}

/* Drotate_PP (c.SYSTEM/M_Drotations_PP.f90:103-271) */
static void drotate_pp(or_fdata *fd, int in1, int in2, const double *eps, const double *deps, int norb_mu,
                       int norb_nu, const double *matm, const double *Dmatm, double *term) {
  drotate_shells(fd, in1, fd->sp[in2].nssh_PP, fd->sp[in2].lssh_PP, fd->have_dorbitals || fd->have_dorbitals_PP, eps,
                 deps, norb_mu, norb_nu, matm, Dmatm, term);
}

/* ------------------------------------------------------------------------ */
/* structure and neighbor maps                                               */
/* ------------------------------------------------------------------------ */
or_sys *or_create_system(or_fdata *fd, int natoms, const double *ratom, const int *imass, const double *lattice,
                         int icluster) {
  if (!fd || natoms < 1) return NULL;
  or_sys *s = (or_sys *)calloc(1, sizeof(or_sys));
  s->fd = fd;
  s->natoms = natoms;
  s->icluster = icluster;
  s->ratom = (double *)malloc(sizeof(double) * 3 * natoms);
  s->imass = (int *)malloc(sizeof(int) * natoms);
  memcpy(s->ratom, ratom, sizeof(double) * 3 * natoms);
  memcpy(s->imass, imass, sizeof(int) * natoms);
  for (int i = 0; i < natoms; i++)
    if (imass[i] < 1 || imass[i] > fd->nspecies) { free(s->ratom); free(s->imass); free(s); return NULL; }
  memcpy(s->lattice, lattice, sizeof(double) * 9);
  /* make_cells (c.SYSTEM/make_cells.f90:112-144) */
  if (icluster == 1) {
    s->mbeta_max = 0;
    s->xl = (double(*)[3])calloc(1, sizeof(double[3]));
  } else {
    int mbox = P_mbox;
    s->mbeta_max = (2 * P_mbox + 1) * (2 * P_mbox + 1) * (2 * P_mbox + 1) - 1;
    s->xl = (double(*)[3])calloc((size_t)s->mbeta_max + 1, sizeof(double[3]));
    int mbeta = 1;
    for (int iz = -mbox; iz <= mbox; iz++)
      for (int iy = -mbox; iy <= mbox; iy++)
        for (int ix = -mbox; ix <= mbox; ix++)
          if (!(ix == 0 && iy == 0 && iz == 0)) {
            for (int k = 0; k < 3; k++)
              s->xl[mbeta][k] = (double)ix * lattice[0 * 3 + k] + (double)iy * lattice[1 * 3 + k] +
                                (double)iz * lattice[2 * 3 + k];
            mbeta++;
          }
  }
  return s;
}

static void free_neigh(or_sys *s) {
  free(s->neighn); free(s->pair_off); free(s->neigh_j); free(s->neigh_b); free(s->neigh_back);
  free(s->neigh_self); free(s->blk_off); free(s->ncommon); free(s->trip_off); free(s->ci_j);
  free(s->ci_b); free(s->cj_j); free(s->cj_b); free(s->cneigh);
  s->neighn = s->pair_off = s->neigh_j = s->neigh_b = s->neigh_back = s->neigh_self = NULL;
  s->ncommon = s->trip_off = s->ci_j = s->ci_b = s->cj_j = s->cj_b = s->cneigh = NULL;
  s->blk_off = NULL;
}

static void free_pp(or_sys *s) {
  void *v[] = {s->pp_off, s->pp_j, s->pp_b, s->pp_self, s->pp_map, s->ppx_off, s->ppx_j, s->ppx_b, s->ppx_self,
               s->ppx_map, s->ppx_point, s->ppp_off, s->ppp_j, s->ppp_b, s->ppp_self, s->svnl_off, s->vnl_off,
               s->ppc_off, s->ppc_i, s->ppc_ib, s->ppc_j, s->ppc_jb, s->ppc_m, s->ppc_m31, s->ppc_m32};
  for (size_t k = 0; k < sizeof v / sizeof v[0]; k++) free(v[k]);
  s->pp_off = s->pp_j = s->pp_b = s->pp_self = s->pp_map = NULL;
  s->ppx_off = s->ppx_j = s->ppx_b = s->ppx_self = s->ppx_map = s->ppx_point = NULL;
  s->ppp_off = s->ppp_j = s->ppp_b = s->ppp_self = NULL;
  s->svnl_off = s->vnl_off = NULL;
  s->ppc_off = s->ppc_i = s->ppc_ib = s->ppc_j = s->ppc_jb = s->ppc_m = s->ppc_m31 = s->ppc_m32 = NULL;
  s->have_pp = 0;
}

void or_free_system(or_sys *s) {
  if (!s) return;
  free_neigh(s);
  free_pp(s);
  free(s->ratom); free(s->imass); free(s->xl); free(s->dQ);
  free(s);
}

static double rcut_of(const or_sys *s, int iatom) { return s->fd->sp[s->imass[iatom]].rcutoffA_max; }
#define RAT(s, i) (&(s)->ratom[3 * (i)])

/* find_neigh_max + find_neighbors + neigh_self/neigh_back
 * (c.SYSTEM/M_neighbors.f90:246-519), then find_common_max +
 * find_common_neighbors (:548-812) */
int or_neighbors(or_sys *s) {
  free_neigh(s);
  int N = s->natoms;
  s->neighn = (int *)calloc((size_t)N, sizeof(int));
  s->pair_off = (int *)calloc((size_t)N + 1, sizeof(int));
  s->neigh_self = (int *)malloc(sizeof(int) * N);
  /* counting pass (find_neigh_max :289-330); atoms are independent, so the
   * CPU baseline runs this loop on all threads */
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
  for (int i = 0; i < N; i++) {
    int num = 0;
    double rci = rcut_of(s, i), r2[3];
    for (int mb = 0; mb <= s->mbeta_max; mb++)
      for (int j = 0; j < N; j++) {
        for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[mb][k];
        double z = distance3(RAT(s, i), r2);
        double range_max = rci + rcut_of(s, j) - 0.01;
        if (z < range_max) num++;
      }
    s->neighn[i] = num;
  }
  for (int i = 0; i < N; i++) s->pair_off[i + 1] = s->pair_off[i] + s->neighn[i];
  int P = s->pair_off[N];
  s->npairs = P;
  s->neigh_j = (int *)malloc(sizeof(int) * (P ? P : 1));
  s->neigh_b = (int *)malloc(sizeof(int) * (P ? P : 1));
  s->neigh_back = (int *)malloc(sizeof(int) * (P ? P : 1));
  int close_err = 0;
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
  for (int i = 0; i < N; i++) {                                     /* :392-439 */
    int num = 0;
    double rci = rcut_of(s, i), r2[3];
    for (int mb = 0; mb <= s->mbeta_max; mb++)
      for (int j = 0; j < N; j++) {
        for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[mb][k];
        double z = distance3(RAT(s, i), r2);
        double range_max = rci + rcut_of(s, j) - 0.01;
        if (i != j && z < 0.5) {
#pragma omp critical
          {
            if (!close_err) seterr("atoms dangerously close: %d %d z=%g mbeta=%d", i + 1, j + 1, z, mb);
            close_err = 1;
          }
        }
        if (z < range_max) {
          s->neigh_j[s->pair_off[i] + num] = j;
          s->neigh_b[s->pair_off[i] + num] = mb;
          num++;
        }
      }
  }
  if (close_err) return E_CLOSE;
  for (int i = 0; i < N; i++) s->neigh_self[i] = -999;              /* :456-505 */
  for (int i = 0; i < N; i++) {
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, mb = s->neigh_b[p], j = s->neigh_j[p];
      s->neigh_back[p] = -999;
      if (i == j && mb == 0) {
        if (s->neigh_self[i] != -999) { seterr("neigh_self found twice for %d", i + 1); return E_SELF; }
        s->neigh_self[i] = in;
      }
      for (int jn = 0; jn < s->neighn[j]; jn++) {
        int q = s->pair_off[j] + jn, jb = s->neigh_b[q], k = s->neigh_j[q];
        if (i != k || fabs(s->xl[mb][0] + s->xl[jb][0]) > 1.0e-3 || fabs(s->xl[mb][1] + s->xl[jb][1]) > 1.0e-3 ||
            fabs(s->xl[mb][2] + s->xl[jb][2]) > 1.0e-3) {
        } else {
          if (s->neigh_back[p] != -999) { seterr("neigh_back found twice for %d", i + 1); return E_BACK; }
          s->neigh_back[p] = jn;
        }
      }
    }
    for (int in = 0; in < s->neighn[i]; in++)
      if (s->neigh_back[s->pair_off[i] + in] == -999) { seterr("no neigh_back for %d", i + 1); return E_BACK; }
  }
  for (int i = 0; i < N; i++)
    if (s->neigh_self[i] == -999) { seterr("no neigh_self for %d", i + 1); return E_SELF; }
  /* block offsets */
  s->blk_off = (long long *)malloc(sizeof(long long) * (P + 1));
  long long off = 0;
  for (int i = 0; i < N; i++)
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in;
      s->blk_off[p] = off;
      off += (long long)s->fd->sp[s->imass[i]].norb_max * s->fd->sp[s->imass[s->neigh_j[p]]].norb_max;
    }
  s->blk_off[P] = off;
  s->nblock = off;
  /* common neighbors (:681-812): a counting pass and a filling pass, both
   * parallel over ialpha, give the reference order */
  s->ncommon = (int *)calloc((size_t)N, sizeof(int));
  s->trip_off = (int *)calloc((size_t)N + 1, sizeof(int));
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) {
      for (int ia = 0; ia < N; ia++) s->trip_off[ia + 1] = s->trip_off[ia] + s->ncommon[ia];
      int T = s->trip_off[N] ? s->trip_off[N] : 1;
      s->ci_j = (int *)malloc(sizeof(int) * T);
      s->ci_b = (int *)malloc(sizeof(int) * T);
      s->cj_j = (int *)malloc(sizeof(int) * T);
      s->cj_b = (int *)malloc(sizeof(int) * T);
      s->cneigh = (int *)malloc(sizeof(int) * T);
    }
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
    for (int ia = 0; ia < N; ia++) {
      int num = 0;
      for (int in = 0; in < s->neighn[ia]; in++) {
        int p = s->pair_off[ia] + in, iat = s->neigh_j[p], ib = s->neigh_b[p];
        if (iat == ia && ib == 0) continue;
        double r1[3], r2[3], r3[3];
        for (int k = 0; k < 3; k++) r1[k] = RAT(s, iat)[k] + s->xl[ib][k];
        double rci = rcut_of(s, iat);
        for (int jn = 0; jn < s->neighn[ia]; jn++) {
          int q = s->pair_off[ia] + jn, jat = s->neigh_j[q], jb = s->neigh_b[q];
          if ((jat == ia && jb == 0) || in == jn) continue;
          for (int k = 0; k < 3; k++) r2[k] = RAT(s, jat)[k] + s->xl[jb][k];
          double z = distance3(r1, r2);
          double range_max = rci + rcut_of(s, jat) - 0.01;
          if (z < range_max) {
            int found = -9999;
            for (int kn = 0; kn < s->neighn[iat]; kn++) {
              int r = s->pair_off[iat] + kn, kat = s->neigh_j[r], kb = s->neigh_b[r];
              for (int k = 0; k < 3; k++) r3[k] = s->xl[kb][k] + RAT(s, kat)[k] - RAT(s, iat)[k];
              if ((fabs(r3[0] - r2[0] + r1[0]) < 1.0e-4) && (fabs(r3[1] - r2[1] + r1[1]) < 1.0e-4) &&
                  (fabs(r3[2] - r2[2] + r1[2]) < 1.0e-4)) {
                found = kn;
                break;
              }
            }
            if (found == -9999) continue;
            if (pass == 1) {
              int t = s->trip_off[ia] + num;
              s->ci_j[t] = iat;
              s->ci_b[t] = ib;
              s->cj_j[t] = jat;
              s->cj_b[t] = jb;
              s->cneigh[t] = found;
            }
            num++;
          }
        }
      }
      if (pass == 0) s->ncommon[ia] = num;
    }
  }
  int nt = s->trip_off[N];
  s->ntrip = nt;
  return OK;
}

int or_npairs(const or_sys *s) { return s->npairs; }
int or_ntriplets(const or_sys *s) { return s->ntrip; }
long long or_nblock(const or_sys *s) { return s->nblock; }

void or_get_pairs(const or_sys *s, int *pair_off, int *neigh_j, int *neigh_b, int *neigh_back, int *neigh_self,
                  long long *blk_off) {
  int N = s->natoms, P = s->npairs;
  if (pair_off) memcpy(pair_off, s->pair_off, sizeof(int) * (N + 1));
  if (neigh_j) memcpy(neigh_j, s->neigh_j, sizeof(int) * P);
  if (neigh_b) memcpy(neigh_b, s->neigh_b, sizeof(int) * P);
  if (neigh_back) memcpy(neigh_back, s->neigh_back, sizeof(int) * P);
  if (neigh_self) memcpy(neigh_self, s->neigh_self, sizeof(int) * N);
  if (blk_off) memcpy(blk_off, s->blk_off, sizeof(long long) * (P + 1));
}

void or_get_triplets(const or_sys *s, int *trip_off, int *iatom_j, int *iatom_b, int *jatom_j, int *jatom_b,
                     int *neigh_common) {
  int N = s->natoms, T = s->ntrip;
  if (trip_off) memcpy(trip_off, s->trip_off, sizeof(int) * (N + 1));
  if (iatom_j) memcpy(iatom_j, s->ci_j, sizeof(int) * T);
  if (iatom_b) memcpy(iatom_b, s->ci_b, sizeof(int) * T);
  if (jatom_j) memcpy(jatom_j, s->cj_j, sizeof(int) * T);
  if (jatom_b) memcpy(jatom_b, s->cj_b, sizeof(int) * T);
  if (neigh_common) memcpy(neigh_common, s->cneigh, sizeof(int) * T);
}

/* ------------------------------------------------------------------------ */
/* assemblers                                                                */
/* ------------------------------------------------------------------------ */
/* pair set-up shared by all 2c assemblers: z, sighat, eps = epsilon(r2,
 * sighat) (e.g. j.ASSEMBLERS/M_assemble_2c_Harris.f90:170-177) */
static void pair_frame(const or_sys *s, int i, int p, double *r1, double *r2, double *z, double *eps) {
  double sighat[3];
  int j = s->neigh_j[p], mb = s->neigh_b[p];
  for (int k = 0; k < 3; k++) {
    r1[k] = RAT(s, i)[k];
    r2[k] = RAT(s, j)[k] + s->xl[mb][k];
  }
  *z = distance3(r1, r2);
  if (*z < 1.0e-05) {
    sighat[0] = 0.0;
    sighat[1] = 0.0;
    sighat[2] = 1.0;
  } else {
    for (int k = 0; k < 3; k++) sighat[k] = (r2[k] - r1[k]) / *z;
  }
  or_epsilon(r2, sighat, eps);
}

/* assemble_S (:89-209), assemble_T (:233-353), assemble_vna_2c (:435-649) of
 * j.ASSEMBLERS/M_assemble_2c_Harris.f90 */
int or_assemble_2c(or_sys *s, double *S, double *T, double *vb, double *vbo) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK;
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
  for (int i = 0; i < N; i++) {
    double r1[3], r2[3], z, eps[9], mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      long long o = s->blk_off[p];
      pair_frame(s, i, p, r1, r2, &z, eps);
      if (S) {
        if ((st = or_getMEs_2c(fd, in1, in2, P_overlap, 0, z, nmu, nnu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        memcpy(S + o, xm, sizeof(double) * nmu * nnu);
      }
      if (T) {
        if ((st = or_getMEs_2c(fd, in1, in2, P_kinetic, 0, z, nmu, nnu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        memcpy(T + o, xm, sizeof(double) * nmu * nnu);
      }
      if (vb) {
        for (int k = 0; k < nmu * nnu; k++) vb[o + k] = 0.0, vbo[o + k] = 0.0;
        if (!(i == j && s->neigh_b[p] == 0)) {
          if ((st = or_getMEs_2c(fd, in1, in2, P_vna_ontopL, 0, z, nmu, nnu, mm))) { err = st; continue; }
          or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
          for (int k = 0; k < nmu * nnu; k++) vbo[o + k] = vbo[o + k] + xm[k] * P_eq2;
          if ((st = or_getMEs_2c(fd, in1, in2, P_vna_ontopR, 0, z, nmu, nnu, mm))) { err = st; continue; }
          or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
          for (int k = 0; k < nmu * nnu; k++) vbo[o + k] = vbo[o + k] + xm[k] * P_eq2;
        }
      }
    }
    if (vb) {
      /* atom case (:584-636): <i|v(j)|i> summed into block(neigh_self(i)) */
      long long os = s->blk_off[s->pair_off[i] + s->neigh_self[i]];
      for (int k = 0; k < nmu * nmu; k++) vb[os + k] = 0.0;
      for (int in = 0; in < s->neighn[i]; in++) {
        int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
        pair_frame(s, i, p, r1, r2, &z, eps);
        if ((st = or_getMEs_2c(fd, in1, in2, P_vna_atom, 0, z, nmu, nmu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in1, eps, nmu, nmu, mm, xm);
        for (int k = 0; k < nmu * nmu; k++) vb[os + k] = vb[os + k] + xm[k] * P_eq2;
      }
    }
  }
  return err;
}

/* triplet set-up shared by assemble_vna_3c and Dassemble_vna_3c
 * (j.ASSEMBLERS/M_assemble_3c_Harris.f90:154-189) */
typedef struct {
  double r1[3], r2[3], rna[3], r21[3], rnabc[3], sighat[3], rhat[3], z, x, cost, eps[9];
  int iatom, jatom, in1, in2, indna, mneigh;
} trip_t;

static void trip_frame(const or_sys *s, int ia, int t, trip_t *g) {
  g->indna = s->imass[ia];
  for (int k = 0; k < 3; k++) g->rna[k] = RAT(s, ia)[k];
  g->mneigh = s->cneigh[t];
  g->iatom = s->ci_j[t];
  g->jatom = s->cj_j[t];
  for (int k = 0; k < 3; k++) {
    g->r1[k] = RAT(s, g->iatom)[k] + s->xl[s->ci_b[t]][k];
    g->r2[k] = RAT(s, g->jatom)[k] + s->xl[s->cj_b[t]][k];
  }
  g->in1 = s->imass[g->iatom];
  g->in2 = s->imass[g->jatom];
  for (int k = 0; k < 3; k++) g->r21[k] = g->r2[k] - g->r1[k];
  g->z = distance3(g->r1, g->r2);
  if (g->z < 1.0e-05) {
    g->sighat[0] = 0.0; g->sighat[1] = 0.0; g->sighat[2] = 1.0;
  } else {
    for (int k = 0; k < 3; k++) g->sighat[k] = g->r21[k] / g->z;
  }
  for (int k = 0; k < 3; k++) g->rnabc[k] = g->rna[k] - (g->r1[k] + g->r21[k] / 2.0);
  g->x = sqrt(g->rnabc[0] * g->rnabc[0] + g->rnabc[1] * g->rnabc[1] + g->rnabc[2] * g->rnabc[2]);
  if (g->x < 1.0e-05) {
    g->rhat[0] = g->rhat[1] = g->rhat[2] = 0.0;
  } else {
    for (int k = 0; k < 3; k++) g->rhat[k] = g->rnabc[k] / g->x;
  }
  g->cost = g->sighat[0] * g->rhat[0] + g->sighat[1] * g->rhat[1] + g->sighat[2] * g->rhat[2];
  or_epsilon(g->rhat, g->sighat, g->eps);
}

/* assemble_vna_3c (j.ASSEMBLERS/M_assemble_3c_Harris.f90:82-227) */
int or_assemble_3c(or_sys *s, double *vb) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK, nthr = g_threads;
  long long nb = s->nblock;
  double *acc = NULL;
  if (nthr > 1) acc = (double *)calloc((size_t)nthr * nb, sizeof(double));
#pragma omp parallel num_threads(nthr) if (nthr > 1)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *dst = nthr > 1 ? acc + (size_t)tid * nb : vb;
#pragma omp for schedule(dynamic, 2)
    for (int ia = 0; ia < N; ia++) {
      double mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
      for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
        trip_t g;
        trip_frame(s, ia, t, &g);
        int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
        int st = or_getMEs_3c(fd, g.in1, g.in2, g.indna, P_bcna, 0, g.x, g.z, nmu, nnu, g.cost, mm);
        if (st) { err = st; continue; }
        or_rotate(fd, g.in1, g.in2, g.eps, nmu, nnu, mm, xm);
        long long o = s->blk_off[s->pair_off[g.iatom] + g.mneigh];
        for (int k = 0; k < nmu * nnu; k++) dst[o + k] = dst[o + k] + xm[k] * P_eq2;
      }
    }
  }
  if (nthr > 1) {
    for (int t = 0; t < nthr; t++)
#pragma omp parallel for num_threads(nthr)
      for (long long k = 0; k < nb; k++) vb[k] += acc[(size_t)t * nb + k];
    free(acc);
  }
  return err;
}

/* Dassemble_S/T (k.DASSEMBLERS/M_Dassemble_2c_Harris.f90:96-263, :289-456)
 * and Dassemble_vna_2c (:538-869) */
int or_dassemble_2c(or_sys *s, const double *rho, double *dS, double *dT, double *vna_ontop, double *vna_atom) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK;
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
  for (int i = 0; i < N; i++) {
    double r1[3], r2[3], z, eps[9], deps[27], eta[3];
    double mm[MAXORB * MAXORB], dm[MAXORB * MAXORB], vdm[3 * MAXORB * MAXORB], vdx[3 * MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, st;
    const int ints[2] = {P_overlap, P_kinetic};
    double *outs[2] = {dS, dT};
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      long long o = s->blk_off[p];
      pair_frame(s, i, p, r1, r2, &z, eps);
      or_depsilon_2c(r1, r2, z, eps, deps);
      for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
      for (int w = 0; w < 2; w++) {
        if (!outs[w]) continue;
        for (int k = 0; k < nmu * nnu; k++) mm[k] = dm[k] = 0.0;
        if ((st = or_getDMEs_2c(fd, in1, in2, ints[w], 0, z, nmu, nnu, mm, dm))) { err = st; continue; }
        for (int k = 0; k < 3 * nmu * nnu; k++) vdm[k] = 0.0;
        for (int inu = 0; inu < nnu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            if (z > 1.0e-3)
              for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
        drotate(fd, in1, in2, eps, deps, nmu, nnu, mm, vdm, vdx);
        memcpy(outs[w] + 3 * o, vdx, sizeof(double) * 3 * nmu * nnu);
      }
      if (vna_ontop) {
        double *f = vna_ontop + 3 * (size_t)p;
        f[0] = f[1] = f[2] = 0.0;
        if (!(i == j && s->neigh_b[p] == 0)) {
          const int vi[2] = {P_vna_ontopL, P_vna_ontopR};
          for (int w = 0; w < 2; w++) {
            for (int k = 0; k < nmu * nnu; k++) mm[k] = dm[k] = 0.0;
            for (int k = 0; k < 3 * nmu * nnu; k++) vdm[k] = vdx[k] = 0.0;
            if ((st = or_getDMEs_2c(fd, in1, in2, vi[w], 0, z, nmu, nnu, mm, dm))) { err = st; continue; }
            for (int inu = 0; inu < nnu; inu++)
              for (int imu = 0; imu < nmu; imu++)
                if (z > 1.0e-3)
                  for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
            drotate(fd, in1, in2, eps, deps, nmu, nnu, mm, vdm, vdx);
            for (int inu = 0; inu < nnu; inu++)
              for (int imu = 0; imu < nmu; imu++)
                for (int c = 0; c < 3; c++)
                  f[c] = f[c] - rho[o + imu + nmu * inu] * vdx[c + 3 * (imu + nmu * inu)] * P_eq2;
          }
        }
      }
    }
    if (vna_atom) {
      /* atom case (:784-859), contracted with the self block of rho */
      long long os = s->blk_off[s->pair_off[i] + s->neigh_self[i]];
      for (int in = 0; in < s->neighn[i]; in++) {
        int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
        double *f = vna_atom + 3 * (size_t)p;
        f[0] = f[1] = f[2] = 0.0;
        pair_frame(s, i, p, r1, r2, &z, eps);
        or_depsilon_2c(r1, r2, z, eps, deps);
        for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
        for (int k = 0; k < nmu * nmu; k++) mm[k] = dm[k] = 0.0;
        for (int k = 0; k < 3 * nmu * nmu; k++) vdm[k] = vdx[k] = 0.0;
        if ((st = or_getDMEs_2c(fd, in1, in2, P_vna_atom, 0, z, nmu, nmu, mm, dm))) { err = st; continue; }
        for (int inu = 0; inu < nmu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            if (z > 1.0e-3)
              for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
        drotate(fd, in1, in1, eps, deps, nmu, nmu, mm, vdm, vdx);
        for (int inu = 0; inu < nmu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            for (int c = 0; c < 3; c++)
              f[c] = f[c] - rho[os + imu + nmu * inu] * vdx[c + 3 * (imu + nmu * inu)] * P_eq2;
      }
    }
  }
  return err;
}

/* Dassemble_vna_3c (k.DASSEMBLERS/M_Dassemble_3c_Harris.f90:136-408) */
int or_dassemble_3c(or_sys *s, const double *rho, double *f3naa, double *f3nab, double *f3nac) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK, nthr = g_threads;
  double *acc = (double *)calloc((size_t)nthr * 9 * N, sizeof(double));
#pragma omp parallel num_threads(nthr) if (nthr > 1)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *fa = acc + (size_t)tid * 9 * N, *fb = fa + 3 * N, *fc = fb + 3 * N;
#pragma omp for schedule(dynamic, 2)
    for (int ia = 0; ia < N; ia++) {
      double mm[MAXORB * MAXORB], dpm[MAXORB * MAXORB], dxm[MAXORB * MAXORB], dym[MAXORB * MAXORB];
      double Ma[3 * MAXORB * MAXORB], Mb[3 * MAXORB * MAXORB], Xa[3 * MAXORB * MAXORB], Xb[3 * MAXORB * MAXORB];
      double depsA[27], depsB[27], amt[3], bmt[3];
      for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
        trip_t g;
        trip_frame(s, ia, t, &g);
        int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
        or_depsilon_3c(g.r1, g.r2, g.r21, g.z, g.rna, g.rnabc, g.eps, depsA, depsB);
        if (g.x > 1.0e-5)                                           /* :285-292 */
          for (int k = 0; k < 3; k++) amt[k] = (g.sighat[k] - g.cost * g.rhat[k]) / g.x;
        else
          amt[0] = amt[1] = amt[2] = 0.0;
        for (int k = 0; k < 3; k++) bmt[k] = (g.cost * g.sighat[k] - g.rhat[k]) / g.z;
        int st = or_getDMEs_3c(fd, g.in1, g.in2, g.indna, P_bcna, 0, g.x, g.z, nmu, nnu, g.cost, mm, dpm, dxm, dym);
        if (st) { err = st; continue; }
        for (int k = 0; k < 3 * nmu * nnu; k++) Ma[k] = Mb[k] = 0.0;
        cell3c *c = get_cell3c(fd, g.in1, g.in2, g.indna, P_bcna, 0, 1);
        for (int m = 0; m < c->nME; m++) {                          /* :330-345 */
          int k = (c->mu[m] - 1) + nmu * (c->nu[m] - 1);
          for (int q = 0; q < 3; q++) Ma[q + 3 * k] = g.rhat[q] * dxm[k] + amt[q] * dpm[k];
          for (int q = 0; q < 3; q++) Mb[q + 3 * k] = -g.sighat[q] * dym[k] + bmt[q] * dpm[k] - Ma[q + 3 * k] / 2.0;
        }
        drotate(fd, g.in1, g.in2, g.eps, depsA, nmu, nnu, mm, Ma, Xa);
        drotate(fd, g.in1, g.in2, g.eps, depsB, nmu, nnu, mm, Mb, Xb);
        long long o = s->blk_off[s->pair_off[g.iatom] + g.mneigh];
        for (int inu = 0; inu < nnu; inu++)                         /* :379-388 */
          for (int imu = 0; imu < nmu; imu++) {
            double r = rho[o + imu + nmu * inu];
            for (int q = 0; q < 3; q++) {
              double xa = Xa[q + 3 * (imu + nmu * inu)], xb = Xb[q + 3 * (imu + nmu * inu)];
              double xc = -xa - xb;
              fa[3 * ia + q] = fa[3 * ia + q] - r * xa * P_eq2;
              fb[3 * g.iatom + q] = fb[3 * g.iatom + q] - r * xb * P_eq2;
              fc[3 * g.jatom + q] = fc[3 * g.jatom + q] - r * xc * P_eq2;
            }
          }
      }
    }
  }
  for (int k = 0; k < 3 * N; k++) {
    double a = 0, b = 0, cc = 0;
    for (int t = 0; t < nthr; t++) {
      a += acc[(size_t)t * 9 * N + k];
      b += acc[(size_t)t * 9 * N + 3 * N + k];
      cc += acc[(size_t)t * 9 * N + 6 * N + k];
    }
    if (f3naa) f3naa[k] = a;
    if (f3nab) f3nab[k] = b;
    if (f3nac) f3nac[k] = cc;
  }
  free(acc);
  return err;
}

/* build_forces (c.SYSTEM/M_build_forces.f90:172-588), assembly terms only:
 * kinetic (:234-301), vna atom/ontop (:310-345), f3na (:444-451), Pulay
 * (:473-537).  The vxc, ewald, vnl, usr and vdW terms belong to assemblers
 * outside this library and are left to the caller. */
int or_build_forces(or_sys *s, const double *rho, const double *cape, const double *dS, const double *dT,
                    const double *vna_ontop, const double *vna_atom, const double *f3naa, const double *f3nab,
                    const double *f3nac, double *kinetic, double *vna, double *pulay, double *ftot) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  for (int k = 0; k < 3 * N; k++) kinetic[k] = vna[k] = pulay[k] = ftot[k] = 0.0;
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], nnu = fd->sp[s->imass[j]].norb_max;
      long long o = s->blk_off[p];
      for (int ix = 0; ix < 3; ix++) {
        double sumT = 0.0;
        for (int inu = 0; inu < nnu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            sumT = sumT + rho[o + imu + nmu * inu] * dT[3 * (o + imu + nmu * inu) + ix];
        kinetic[3 * i + ix] = kinetic[3 * i + ix] + (-1.0) * sumT;
        kinetic[3 * j + ix] = kinetic[3 * j + ix] - (-1.0) * sumT;
      }
    }
  }
  for (int k = 0; k < 3 * N; k++) ftot[k] = ftot[k] + kinetic[k];
  for (int i = 0; i < N; i++)
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p];
      for (int q = 0; q < 3; q++) {
        vna[3 * i + q] = vna[3 * i + q] + vna_atom[3 * p + q];
        vna[3 * j + q] = vna[3 * j + q] - vna_atom[3 * p + q];
        ftot[3 * i + q] = ftot[3 * i + q] + vna_atom[3 * p + q];
        ftot[3 * j + q] = ftot[3 * j + q] - vna_atom[3 * p + q];
        vna[3 * i + q] = vna[3 * i + q] + vna_ontop[3 * p + q];
        vna[3 * j + q] = vna[3 * j + q] - vna_ontop[3 * p + q];
        ftot[3 * i + q] = ftot[3 * i + q] + vna_ontop[3 * p + q];
        ftot[3 * j + q] = ftot[3 * j + q] - vna_ontop[3 * p + q];
      }
    }
  for (int k = 0; k < 3 * N; k++) ftot[k] = ftot[k] + f3naa[k] + f3nab[k] + f3nac[k];
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], nnu = fd->sp[s->imass[j]].norb_max;
      long long o = s->blk_off[p];
      for (int ix = 0; ix < 3; ix++) {
        double sumT = 0.0;
        for (int inu = 0; inu < nnu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            sumT = sumT + cape[o + imu + nmu * inu] * dS[3 * (o + imu + nmu * inu) + ix];
        pulay[3 * i + ix] = pulay[3 * i + ix] + (-1.0) * sumT;
        pulay[3 * j + ix] = pulay[3 * j + ix] - (-1.0) * sumT;
      }
    }
  }
  for (int k = 0; k < 3 * N; k++) ftot[k] = ftot[k] - pulay[k];
  return OK;
}

/* ------------------------------------------------------------------------ */
/* Bloch sums (h.SOLVESH/M_kspace_Lowdin.f90:680-708, :796-853)              */
/* ------------------------------------------------------------------------ */
/* out: nk column-major n x n complex matrices (re, im interleaved),
 * M(jmu,jnu) += phase(dot) * block(imu,inu) over every pair, with
 * vec = xl(mbeta) + ratom(jatom) - ratom(iatom), dot = k . vec and
 * phase(dot) = cmplx(cos(dot), sin(dot))
 * (M_diagonalization_Lowdin_kpoints.f90:413-442); jmu = imu + iblock_slot
 * (M_configuraciones.f90:778-783). */
int or_bloch(or_sys *s, int nk, const double *kpts, const double *blocks, double *out) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  int *slot = (int *)malloc(sizeof(int) * (N + 1));
  if (!slot) return E_ARG;
  slot[0] = 0;
  for (int i = 0; i < N; i++) slot[i + 1] = slot[i] + fd->sp[s->imass[i]].norb_max;
  long long n = slot[N];
  for (long long q = 0; q < (long long)nk * 2 * n * n; q++) out[q] = 0.0;
  for (int kk = 0; kk < nk; kk++) {
    const double *k = kpts + 3 * kk;
    double *M = out + (long long)kk * 2 * n * n;
    for (int i = 0; i < N; i++) {
      int ni = fd->sp[s->imass[i]].norb_max;
      for (int p = s->pair_off[i]; p < s->pair_off[i + 1]; p++) {
        int j = s->neigh_j[p], mb = s->neigh_b[p];
        int nj = fd->sp[s->imass[j]].norb_max;
        double vec[3], dot = 0.0;
        for (int c = 0; c < 3; c++) {
          vec[c] = (s->xl[mb][c] + s->ratom[3 * j + c]) - s->ratom[3 * i + c];
          dot += k[c] * vec[c];
        }
        double cs = cos(dot), sn = sin(dot);
        for (int nu = 0; nu < nj; nu++)
          for (int mu = 0; mu < ni; mu++) {
            double v = blocks[s->blk_off[p] + mu + (long long)ni * nu];
            long long e = (slot[i] + mu) + n * (long long)(slot[j] + nu);
            M[2 * e] += cs * v;
            M[2 * e + 1] += sn * v;
          }
      }
    }
  }
  free(slot);
  return 0;
}
/* ------------------------------------------------------------------------ */
/* DOGS: charge-weighted neutral-atom terms                                  */
/* ------------------------------------------------------------------------ */
int or_set_charges(or_sys *s, const double *dq, int nssh_max) {
  if (!s || !dq || nssh_max < 1) return E_ARG;
  free(s->dQ);
  s->dQ = (double *)malloc(sizeof(double) * (size_t)s->natoms * nssh_max);
  memcpy(s->dQ, dq, sizeof(double) * (size_t)s->natoms * nssh_max);
  s->nssh_max = nssh_max;
  return OK;
}

/* s%atom(iatom)%shell(isorp)%dQ */
static double shell_dq(const or_sys *s, int iatom, int isorp) {
  if (!s->dQ || isorp > s->nssh_max) return 0.0;
  return s->dQ[(size_t)iatom * s->nssh_max + isorp - 1];
}

/* smoother (b.FUNCTIONS/smoother.f90:100-146), scaler = 1 */
static double smoother(double r, double rend, double x) {
  double rbegin = x * rend;
  if (r > rend) return 0.0;
  if (r < rbegin) return 1.0;
  double ratio = (r - rbegin) / (rend - rbegin);
  double sm = 1.0 - ratio * ratio;
  return sm * sm;
}

/* smallest shell cutoff of a species, starting from 99
 * (j.ASSEMBLERS/M_assemble_2c_DOGS.f90:746-754) */
static double rcutoff_min(const species_t *sp) {
  double r = 99.0;
  for (int k = 0; k < sp->nssh; k++) r = fmin(r, sp->rcutoffA[k]);
  return r;
}

/* assemble_dipole_z (j.ASSEMBLERS/M_assemble_2c_DOGS.f90:376-499) */
int or_assemble_dipole_z(or_sys *s, double *dip) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int i = 0; i < s->natoms; i++) {
    double r1[3], r2[3], z, eps[9], mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      pair_frame(s, i, p, r1, r2, &z, eps);
      if ((st = or_getMEs_2c(fd, in1, in2, P_dipole_z, 0, z, nmu, nnu, mm))) { err = st; continue; }
      or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
      memcpy(dip + s->blk_off[p], xm, sizeof(double) * nmu * nnu);
    }
  }
  return err;
}

/* assemble_vna_2c, DOGS (j.ASSEMBLERS/M_assemble_2c_DOGS.f90:640-814): the
 * Harris ontop and atom terms plus the charged shells -- ontop L weighted by
 * the shells of iatom, ontop R and atom by those of jatom, the atom terms
 * smoothed into the effective monopole S(i, self) / z.  S is the overlap
 * block set. */
int or_assemble_vna_2c_dogs(or_sys *s, const double *S, double *vb, double *vbo) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int i = 0; i < s->natoms; i++) {
    double r1[3], r2[3], z, eps[9], mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      long long o = s->blk_off[p];
      for (int k = 0; k < nmu * nnu; k++) vb[o + k] = 0.0, vbo[o + k] = 0.0;
      if (i == j && s->neigh_b[p] == 0) continue;
      pair_frame(s, i, p, r1, r2, &z, eps);
      /* ontop L: neutral, then the charged shells of iatom */
      for (int isorp = 0; isorp <= fd->sp[in1].nssh; isorp++) {
        if ((st = or_getMEs_2c(fd, in1, in2, P_vna_ontopL, isorp, z, nmu, nnu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        double w = isorp == 0 ? 1.0 : shell_dq(s, i, isorp);
        for (int k = 0; k < nmu * nnu; k++) vbo[o + k] = vbo[o + k] + w * xm[k] * P_eq2;
      }
      /* ontop R: neutral, then the charged shells of jatom */
      for (int isorp = 0; isorp <= fd->sp[in2].nssh; isorp++) {
        if ((st = or_getMEs_2c(fd, in1, in2, P_vna_ontopR, isorp, z, nmu, nnu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        double w = isorp == 0 ? 1.0 : shell_dq(s, j, isorp);
        for (int k = 0; k < nmu * nnu; k++) vbo[o + k] = vbo[o + k] + w * xm[k] * P_eq2;
      }
    }
    /* atom case (:704-814) into block(neigh_self(i)) */
    long long os = s->blk_off[s->pair_off[i] + s->neigh_self[i]];
    for (int k = 0; k < nmu * nmu; k++) vb[os + k] = 0.0;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
      pair_frame(s, i, p, r1, r2, &z, eps);
      double rend = rcutoff_min(&fd->sp[in1]) + rcutoff_min(&fd->sp[in2]);
      double smooth = smoother(z, rend, 0.8);
      double emnpl[MAXORB * MAXORB];
      for (int k = 0; k < nmu * nmu; k++) emnpl[k] = z > 1.0e-4 ? S[os + k] / z : 0.0;
      for (int isorp = 0; isorp <= fd->sp[in2].nssh; isorp++) {
        if ((st = or_getMEs_2c(fd, in1, in2, P_vna_atom, isorp, z, nmu, nmu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in1, eps, nmu, nmu, mm, xm);
        if (isorp == 0) {
          for (int k = 0; k < nmu * nmu; k++) vb[os + k] = vb[os + k] + xm[k] * P_eq2;
        } else {
          double dq = shell_dq(s, j, isorp);
          for (int k = 0; k < nmu * nmu; k++)
            vb[os + k] = vb[os + k] + P_eq2 * dq * ((1.0 - smooth) * emnpl[k] + smooth * xm[k]);
        }
      }
    }
  }
  return err;
}

/* assemble_vna_3c, DOGS (j.ASSEMBLERS/M_assemble_3c_DOGS.f90:158-322),
 * accumulating: the neutral bcna term plus, for the charged shells of
 * ialpha, the dQ-weighted sub-cells smoothed (stinky = smoother(d13) *
 * smoother(d23)) into the effective monopole
 * emnpl = (S/2 - dip/z)/d13 + (S/2 + dip/z)/d23 of the pair (i, mneigh). */
int or_assemble_vna_3c_dogs(or_sys *s, const double *S, const double *dip, double *vb) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int ia = 0; ia < s->natoms; ia++) {
    double mm[MAXORB * MAXORB], xm[MAXORB * MAXORB], emnpl[MAXORB * MAXORB];
    for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
      trip_t g;
      trip_frame(s, ia, t, &g);
      int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
      long long o = s->blk_off[s->pair_off[g.iatom] + g.mneigh];
      double d13 = distance3(g.rna, g.r1), d23 = distance3(g.rna, g.r2);
      double rc3 = rcutoff_min(&fd->sp[g.indna]);
      double stinky = smoother(d13, rcutoff_min(&fd->sp[g.in1]) + rc3, 0.8) *
                      smoother(d23, rcutoff_min(&fd->sp[g.in2]) + rc3, 0.8);
      for (int k = 0; k < nmu * nnu; k++) {
        double sterm = S[o + k] / 2.0, dterm = dip[o + k] / g.z;
        emnpl[k] = (sterm - dterm) / d13 + (sterm + dterm) / d23;
      }
      for (int isorp = 0; isorp <= fd->sp[g.indna].nssh; isorp++) {
        int st = or_getMEs_3c(fd, g.in1, g.in2, g.indna, P_bcna, isorp, g.x, g.z, nmu, nnu, g.cost, mm);
        if (st) { err = st; continue; }
        or_rotate(fd, g.in1, g.in2, g.eps, nmu, nnu, mm, xm);
        if (isorp == 0) {
          for (int k = 0; k < nmu * nnu; k++) vb[o + k] = vb[o + k] + xm[k] * P_eq2;
        } else {
          double dq = shell_dq(s, ia, isorp);
          for (int k = 0; k < nmu * nnu; k++)
            vb[o + k] = vb[o + k] + dq * (stinky * xm[k] + (1.0 - stinky) * emnpl[k]) * P_eq2;
        }
      }
    }
  }
  return err;
}

/* Dsmoother (b.FUNCTIONS/Dsmoother.f90:102-135), scaler = 1 */
static double dsmoother(double r, double rend, double x) {
  double rbegin = x * rend;
  if (r > rend) return 0.0;
  if (r < rbegin) return 0.0;
  double ratio = (r - rbegin) / (rend - rbegin);
  return -2.0 * (1.0 - ratio * ratio) * (2.0 * ratio) / (rend - rbegin);
}

/* Dassemble_dipole_z (k.DASSEMBLERS/M_Dassemble_2c_DOGS.f90:487-655):
 * Dblock(3, mu, nu) of the z-dipole, layout of dS */
int or_dassemble_dipole_z(or_sys *s, double *ddip) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int i = 0; i < s->natoms; i++) {
    double r1[3], r2[3], z, eps[9], deps[27], eta[3];
    double mm[MAXORB * MAXORB], dm[MAXORB * MAXORB], vdm[3 * MAXORB * MAXORB], vdx[3 * MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      pair_frame(s, i, p, r1, r2, &z, eps);
      or_depsilon_2c(r1, r2, z, eps, deps);
      for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
      for (int k = 0; k < nmu * nnu; k++) mm[k] = dm[k] = 0.0;
      for (int k = 0; k < 3 * nmu * nnu; k++) vdm[k] = 0.0;
      if ((st = or_getDMEs_2c(fd, in1, in2, P_dipole_z, 0, z, nmu, nnu, mm, dm))) { err = st; continue; }
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++)
          if (z > 1.0e-3)
            for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
      drotate(fd, in1, in2, eps, deps, nmu, nnu, mm, vdm, vdx);
      memcpy(ddip + 3 * s->blk_off[p], vdx, sizeof(double) * 3 * nmu * nnu);
    }
  }
  return err;
}

/* Dassemble_vna_2c, DOGS (k.DASSEMBLERS/M_Dassemble_2c_DOGS.f90:679-1199):
 * the Harris ontop and atom derivatives plus the charged shells -- ontop L
 * weighted by the shells of iatom, ontop R by those of jatom; the atom terms
 * smoothed, with the derivative of the smoother and of the monopole S/z.
 * S is the overlap block set. */
int or_dassemble_vna_2c_dogs(or_sys *s, const double *rho, const double *S, double *vna_ontop, double *vna_atom) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int i = 0; i < s->natoms; i++) {
    double r1[3], r2[3], z, eps[9], deps[27], eta[3];
    double mm[MAXORB * MAXORB], dm[MAXORB * MAXORB], vdm[3 * MAXORB * MAXORB], vdx[3 * MAXORB * MAXORB];
    double xm[MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      long long o = s->blk_off[p];
      double *f = vna_ontop + 3 * (size_t)p;
      f[0] = f[1] = f[2] = 0.0;
      if (i == j && s->neigh_b[p] == 0) continue;
      pair_frame(s, i, p, r1, r2, &z, eps);
      or_depsilon_2c(r1, r2, z, eps, deps);
      for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
      const int vi[2] = {P_vna_ontopL, P_vna_ontopR};
      for (int w = 0; w < 2; w++) {
        int owner = w == 0 ? i : j, nsh = fd->sp[w == 0 ? in1 : in2].nssh;
        for (int isorp = 0; isorp <= nsh; isorp++) {
          double dq = isorp == 0 ? 1.0 : shell_dq(s, owner, isorp);
          for (int k = 0; k < nmu * nnu; k++) mm[k] = dm[k] = 0.0;
          for (int k = 0; k < 3 * nmu * nnu; k++) vdm[k] = vdx[k] = 0.0;
          if ((st = or_getDMEs_2c(fd, in1, in2, vi[w], isorp, z, nmu, nnu, mm, dm))) { err = st; continue; }
          for (int inu = 0; inu < nnu; inu++)
            for (int imu = 0; imu < nmu; imu++)
              if (z > 1.0e-3)
                for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
          drotate(fd, in1, in2, eps, deps, nmu, nnu, mm, vdm, vdx);
          for (int inu = 0; inu < nnu; inu++)
            for (int imu = 0; imu < nmu; imu++)
              for (int c = 0; c < 3; c++) {
                double r = rho[o + imu + nmu * inu];
                if (isorp == 0) f[c] = f[c] - r * vdx[c + 3 * (imu + nmu * inu)] * P_eq2;
                else f[c] = f[c] - r * dq * vdx[c + 3 * (imu + nmu * inu)] * P_eq2;
              }
        }
      }
    }
    /* atom case (:1004-1196), contracted with the self blocks of rho and S */
    long long os = s->blk_off[s->pair_off[i] + s->neigh_self[i]];
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
      double *f = vna_atom + 3 * (size_t)p;
      f[0] = f[1] = f[2] = 0.0;
      pair_frame(s, i, p, r1, r2, &z, eps);
      or_depsilon_2c(r1, r2, z, eps, deps);
      for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
      double rend = rcutoff_min(&fd->sp[in1]) + rcutoff_min(&fd->sp[in2]);
      double smooth = smoother(z, rend, 0.8), dsmooth = dsmoother(z, rend, 0.8);
      for (int isorp = 0; isorp <= fd->sp[in2].nssh; isorp++) {
        for (int k = 0; k < nmu * nmu; k++) mm[k] = dm[k] = xm[k] = 0.0;
        for (int k = 0; k < 3 * nmu * nmu; k++) vdm[k] = vdx[k] = 0.0;
        if ((st = or_getDMEs_2c(fd, in1, in2, P_vna_atom, isorp, z, nmu, nmu, mm, dm))) { err = st; continue; }
        if (isorp == 0) {
          for (int inu = 0; inu < nmu; inu++)
            for (int imu = 0; imu < nmu; imu++)
              if (z > 1.0e-3)
                for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
          drotate(fd, in1, in1, eps, deps, nmu, nmu, mm, vdm, vdx);
          for (int inu = 0; inu < nmu; inu++)
            for (int imu = 0; imu < nmu; imu++)
              for (int c = 0; c < 3; c++)
                f[c] = f[c] - rho[os + imu + nmu * inu] * vdx[c + 3 * (imu + nmu * inu)] * P_eq2;
          continue;
        }
        double dq = shell_dq(s, j, isorp);
        double emnpl[MAXORB * MAXORB], vdemnpl[3 * MAXORB * MAXORB];
        for (int k = 0; k < nmu * nmu; k++) emnpl[k] = 0.0;
        for (int k = 0; k < 3 * nmu * nmu; k++) vdemnpl[k] = 0.0;
        for (int inu = 0; inu < nmu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            if (z > 1.0e-4) {
              int k = imu + nmu * inu;
              for (int c = 0; c < 3; c++) vdm[c + 3 * k] = -eta[c] * dm[k];
              emnpl[k] = S[os + k] / z;
              for (int c = 0; c < 3; c++) vdemnpl[c + 3 * k] = eta[c] * S[os + k] / (z * z);
            }
        or_rotate(fd, in1, in1, eps, nmu, nmu, mm, xm);
        drotate(fd, in1, in1, eps, deps, nmu, nmu, mm, vdm, vdx);
        for (int inu = 0; inu < nmu; inu++)
          for (int imu = 0; imu < nmu; imu++) {
            int k = imu + nmu * inu;
            for (int c = 0; c < 3; c++)
              f[c] = f[c] - rho[os + k] * P_eq2 * dq *
                                (smooth * vdx[c + 3 * k] - eta[c] * dsmooth * xm[k] +
                                 (1.0 - smooth) * vdemnpl[c + 3 * k] + eta[c] * dsmooth * emnpl[k]);
          }
      }
    }
  }
  return err;
}

/* Dassemble_vna_3c, DOGS (k.DASSEMBLERS/M_Dassemble_3c_DOGS.f90:136-520):
 * the Harris (neutral) term plus, for the charged shells of ialpha, the
 * smoothed sub-cell derivatives with the derivatives of the smoothers
 * (dstn) and of the effective monopole (demnpl), from the overlap and
 * z-dipole blocks of the pair (i, mneigh) and their Dblocks dS, ddip. */
int or_dassemble_vna_3c_dogs(or_sys *s, const double *rho, const double *S, const double *dS, const double *dip,
                             const double *ddip, double *f3naa, double *f3nab, double *f3nac) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK;
  if ((err = or_dassemble_3c(s, rho, f3naa, f3nab, f3nac))) return err;
  for (int ia = 0; ia < N; ia++) {
    double mm[MAXORB * MAXORB], xm[MAXORB * MAXORB], dpm[MAXORB * MAXORB], dxm[MAXORB * MAXORB],
        dym[MAXORB * MAXORB];
    double Ma[3 * MAXORB * MAXORB], Mb[3 * MAXORB * MAXORB], Xa[3 * MAXORB * MAXORB], Xb[3 * MAXORB * MAXORB];
    double emnpl[MAXORB * MAXORB], dA[3 * MAXORB * MAXORB], dB[3 * MAXORB * MAXORB];
    double depsA[27], depsB[27], amt[3], bmt[3], rA1[3] = {0, 0, 0}, rA2[3] = {0, 0, 0};
    for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
      trip_t g;
      trip_frame(s, ia, t, &g);
      int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
      or_depsilon_3c(g.r1, g.r2, g.r21, g.z, g.rna, g.rnabc, g.eps, depsA, depsB);
      double d13 = distance3(g.rna, g.r1), d23 = distance3(g.rna, g.r2);
      if (d13 > 1.0e-5)
        for (int k = 0; k < 3; k++) rA1[k] = (g.rna[k] - g.r1[k]) / d13;
      if (d23 > 1.0e-5)
        for (int k = 0; k < 3; k++) rA2[k] = (g.rna[k] - g.r2[k]) / d23;
      if (g.x > 1.0e-5)
        for (int k = 0; k < 3; k++) amt[k] = (g.sighat[k] - g.cost * g.rhat[k]) / g.x;
      else
        amt[0] = amt[1] = amt[2] = 0.0;
      for (int k = 0; k < 3; k++) bmt[k] = (g.cost * g.sighat[k] - g.rhat[k]) / g.z;
      double rc3 = rcutoff_min(&fd->sp[g.indna]);
      double rend1 = rcutoff_min(&fd->sp[g.in1]) + rc3, rend2 = rcutoff_min(&fd->sp[g.in2]) + rc3;
      double s13 = smoother(d13, rend1, 0.8), ds13 = dsmoother(d13, rend1, 0.8);
      double s23 = smoother(d23, rend2, 0.8), ds23 = dsmoother(d23, rend2, 0.8);
      double stinky = s13 * s23, dstnA[3], dstnB[3], dstnC[3];
      for (int k = 0; k < 3; k++) {
        dstnB[k] = -ds13 * s23 * rA1[k];
        dstnC[k] = -s13 * ds23 * rA2[k];
        dstnA[k] = -dstnB[k] - dstnC[k];
      }
      long long o = s->blk_off[s->pair_off[g.iatom] + g.mneigh];
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          int k = imu + nmu * inu;
          double sterm = S[o + k] / 2.0, dterm = dip[o + k] / g.z;
          emnpl[k] = (sterm - dterm) / d13 + (sterm + dterm) / d23;
          for (int c = 0; c < 3; c++) {
            double spterm = dS[3 * (o + k) + c] / 2.0;
            double dpterm = ddip[3 * (o + k) + c] / g.z + dterm * g.sighat[c] / g.z;
            dA[c + 3 * k] = -(sterm - dterm) * rA1[c] / (d13 * d13) - (sterm + dterm) * rA2[c] / (d23 * d23);
            dB[c + 3 * k] = (sterm - dterm) * rA1[c] / (d13 * d13) + (spterm - dpterm) / d13 +
                            (spterm + dpterm) / d23;
          }
        }
      for (int isorp = 1; isorp <= fd->sp[g.indna].nssh; isorp++) {
        int st = or_getDMEs_3c(fd, g.in1, g.in2, g.indna, P_bcna, isorp, g.x, g.z, nmu, nnu, g.cost, mm, dpm, dxm,
                               dym);
        if (st) { err = st; continue; }
        or_rotate(fd, g.in1, g.in2, g.eps, nmu, nnu, mm, xm);
        for (int k = 0; k < 3 * nmu * nnu; k++) Ma[k] = Mb[k] = 0.0;
        cell3c *c = get_cell3c(fd, g.in1, g.in2, g.indna, P_bcna, isorp, 1);
        for (int m = 0; m < c->nME; m++) {
          int k = (c->mu[m] - 1) + nmu * (c->nu[m] - 1);
          for (int q = 0; q < 3; q++) Ma[q + 3 * k] = g.rhat[q] * dxm[k] + amt[q] * dpm[k];
          for (int q = 0; q < 3; q++) Mb[q + 3 * k] = -g.sighat[q] * dym[k] + bmt[q] * dpm[k] - Ma[q + 3 * k] / 2.0;
        }
        drotate(fd, g.in1, g.in2, g.eps, depsA, nmu, nnu, mm, Ma, Xa);
        drotate(fd, g.in1, g.in2, g.eps, depsB, nmu, nnu, mm, Mb, Xb);
        double dq = shell_dq(s, ia, isorp);
        for (int inu = 0; inu < nnu; inu++)
          for (int imu = 0; imu < nmu; imu++) {
            int k = imu + nmu * inu;
            double r = rho[o + k];
            for (int q = 0; q < 3; q++) {
              double xa = Xa[q + 3 * k], xb = Xb[q + 3 * k], xc = -xa - xb;
              double dC = -dA[q + 3 * k] - dB[q + 3 * k];
              f3naa[3 * ia + q] = f3naa[3 * ia + q] - P_eq2 * dq * r *
                  (stinky * xa + dstnA[q] * xm[k] - dstnA[q] * emnpl[k] + (1.0 - stinky) * dA[q + 3 * k]);
              f3nab[3 * g.iatom + q] = f3nab[3 * g.iatom + q] - P_eq2 * dq * r *
                  (stinky * xb + dstnB[q] * xm[k] - dstnB[q] * emnpl[k] + (1.0 - stinky) * dB[q + 3 * k]);
              f3nac[3 * g.jatom + q] = f3nac[3 * g.jatom + q] - P_eq2 * dq * r *
                  (stinky * xc + dstnC[q] * xm[k] - dstnC[q] * emnpl[k] + (1.0 - stinky) * dC);
            }
          }
      }
    }
  }
  return err;
}

/* ------------------------------------------------------------------------ */
/* Non-local pseudopotential (vnl)                                           */
/* ------------------------------------------------------------------------ */
/* growable int list */
typedef struct { int *v; int n, cap; } ivec;
static void ivec_push(ivec *a, int x) {
  if (a->n == a->cap) {
    a->cap = a->cap ? 2 * a->cap : 256;
    a->v = (int *)realloc(a->v, sizeof(int) * a->cap);
  }
  a->v[a->n++] = x;
}

/* pairs (i, j, mbeta) with |r_j + xl - r_i| < rc_i + rc_j - 0.01, mbeta
 * outer and jatom inner, and the self index; ri / rj the two cutoffs
 * (find_neighbors_PP, M_neighbors_PP.f90:409-516, ri = basis, rj = PP;
 * find_neighbors_PPx, :672-778, ri = PP, rj = basis) */
static int pp_pairs(or_sys *s, int kind, int **off, int **jj, int **bb, int **self) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  ivec J = {0}, B = {0};
  *off = (int *)malloc(sizeof(int) * (N + 1));
  *self = (int *)malloc(sizeof(int) * N);
  (*off)[0] = 0;
  for (int i = 0; i < N; i++) {
    const species_t *a = &fd->sp[s->imass[i]];
    double rci = kind == 0 ? a->rcutoffA_max : a->rcutoff_PP;
    (*self)[i] = -1;
    for (int mb = 0; mb <= s->mbeta_max; mb++)
      for (int j = 0; j < N; j++) {
        const species_t *b = &fd->sp[s->imass[j]];
        double rcj = kind == 0 ? b->rcutoff_PP : b->rcutoffA_max;
        double r2[3];
        for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[mb][k];
        double z = distance3(RAT(s, i), r2);
        if (z < rci + rcj - 0.01) {
          if (j == i && mb == 0 && (*self)[i] < 0) (*self)[i] = J.n - (*off)[i];
          ivec_push(&J, j);
          ivec_push(&B, mb);
        }
      }
    (*off)[i + 1] = J.n;
    if ((*self)[i] < 0) { seterr("no PP self pair for atom %d", i + 1); return E_SELF; }
  }
  *jj = J.v ? J.v : (int *)malloc(sizeof(int));
  *bb = B.v ? B.v : (int *)malloc(sizeof(int));
  return OK;
}

/* the image index of a lattice vector (distance < 1e-4), or -1 */
static int image_of(const or_sys *s, const double *r) {
  for (int mb = 0; mb <= s->mbeta_max; mb++)
    if (distance3(s->xl[mb], r) < 1.0e-04) return mb;
  return -1;
}

/* driver_neighbors_PP (c.SYSTEM/M_neighbors_PP.f90:98-151): PP and PPx
 * pairs, PPp with the PP/PPx maps and the PPx point (find_neighbors_PPp,
 * :922-1123), and the PP common-neighbor triplets (find_common_neighbors_PP,
 * :1301-1420) with the svnl indices mpairnay gives
 * (M_assemble_PP_3c.f90:266-365) */
int or_neighbors_pp(or_sys *s) {
  or_fdata *fd = s->fd;
  int N = s->natoms, st;
  free_pp(s);
  if ((st = pp_pairs(s, 0, &s->pp_off, &s->pp_j, &s->pp_b, &s->pp_self))) return st;
  if ((st = pp_pairs(s, 1, &s->ppx_off, &s->ppx_j, &s->ppx_b, &s->ppx_self))) return st;
  /* PPp: for each PP neighbor alpha of i, each PPx neighbor j of alpha,
   * image xl(jbeta) + xl(ibeta); first occurrences in that order */
  ivec J = {0}, B = {0};
  s->ppp_off = (int *)malloc(sizeof(int) * (N + 1));
  s->ppp_self = (int *)malloc(sizeof(int) * N);
  s->ppp_off[0] = 0;
  for (int i = 0; i < N; i++) {
    int start = J.n;
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      int al = s->pp_j[p], ib = s->pp_b[p];
      for (int q = s->ppx_off[al]; q < s->ppx_off[al + 1]; q++) {
        int j = s->ppx_j[q], jb = s->ppx_b[q];
        double r3[3];
        for (int k = 0; k < 3; k++) r3[k] = s->xl[jb][k] + s->xl[ib][k];
        int mb = image_of(s, r3);
        if (mb < 0) {
          seterr("PPp image of atom %d outside the %d-image box", j + 1, s->mbeta_max + 1);
          return E_BACK;
        }
        int found = 0;
        for (int k = start; k < J.n; k++)
          if (J.v[k] == j && B.v[k] == mb) { found = 1; break; }
        if (!found) { ivec_push(&J, j); ivec_push(&B, mb); }
      }
    }
    s->ppp_off[i + 1] = J.n;
    s->ppp_self[i] = -1;
    for (int k = start; k < J.n; k++)
      if (J.v[k] == i && B.v[k] == 0) { s->ppp_self[i] = k - start; break; }
    if (s->ppp_self[i] < 0) { seterr("no PPp self pair for atom %d", i + 1); return E_SELF; }
  }
  s->ppp_j = J.v;
  s->ppp_b = B.v;
  /* maps of PP and PPx pairs into PPp, and PPx point into PP(j) */
  s->pp_map = (int *)malloc(sizeof(int) * (s->pp_off[N] + 1));
  s->ppx_map = (int *)malloc(sizeof(int) * (s->ppx_off[N] + 1));
  s->ppx_point = (int *)malloc(sizeof(int) * (s->ppx_off[N] + 1));
  for (int i = 0; i < N; i++) {
    for (int w = 0; w < 2; w++) {
      int *off = w ? s->ppx_off : s->pp_off, *jj = w ? s->ppx_j : s->pp_j, *bb = w ? s->ppx_b : s->pp_b;
      int *map = w ? s->ppx_map : s->pp_map;
      for (int p = off[i]; p < off[i + 1]; p++) {
        map[p] = -1;
        for (int k = s->ppp_off[i]; k < s->ppp_off[i + 1]; k++)
          if (s->ppp_j[k] == jj[p] && s->ppp_b[k] == bb[p]) { map[p] = k - s->ppp_off[i]; break; }
        if (map[p] < 0) { seterr("PP map of atom %d not found", i + 1); return E_BACK; }
      }
    }
    for (int p = s->ppx_off[i]; p < s->ppx_off[i + 1]; p++) {
      int j = s->ppx_j[p], jb = s->ppx_b[p];
      s->ppx_point[p] = -1;
      for (int k = s->pp_off[j]; k < s->pp_off[j + 1]; k++) {
        double r2[3];
        for (int c = 0; c < 3; c++) r2[c] = RAT(s, s->pp_j[k])[c] + s->xl[s->pp_b[k]][c] + s->xl[jb][c];
        if (distance3(RAT(s, i), r2) < 1.0e-04) { s->ppx_point[p] = k - s->pp_off[j]; break; }
      }
      if (s->ppx_point[p] < 0) { seterr("PPx point of atom %d not found", i + 1); return E_BACK; }
    }
  }
  /* block offsets: svnl norb_i x norb_PP_j per PP pair, vnl norb_i x norb_j per PPp pair */
  s->svnl_off = (long long *)malloc(sizeof(long long) * (s->pp_off[N] + 1));
  s->vnl_off = (long long *)malloc(sizeof(long long) * (s->ppp_off[N] + 1));
  long long o = 0;
  for (int i = 0; i < N; i++)
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      s->svnl_off[p] = o;
      o += (long long)fd->sp[s->imass[i]].norb_max * fd->sp[s->imass[s->pp_j[p]]].norb_PP_max;
    }
  s->svnl_off[s->pp_off[N]] = o;
  s->nsvnl = o;
  o = 0;
  for (int i = 0; i < N; i++)
    for (int p = s->ppp_off[i]; p < s->ppp_off[i + 1]; p++) {
      s->vnl_off[p] = o;
      o += (long long)fd->sp[s->imass[i]].norb_max * fd->sp[s->imass[s->ppp_j[p]]].norb_max;
    }
  s->vnl_off[s->ppp_off[N]] = o;
  s->nvnl = o;
  /* common PP triplets of each alpha */
  ivec CI = {0}, CIB = {0}, CJ = {0}, CJB = {0}, CM = {0}, C31 = {0}, C32 = {0};
  s->ppc_off = (int *)malloc(sizeof(int) * (N + 1));
  s->ppc_off[0] = 0;
  for (int al = 0; al < N; al++) {
    for (int a = s->ppx_off[al]; a < s->ppx_off[al + 1]; a++) {
      int i = s->ppx_j[a], ib = s->ppx_b[a];
      if (i == al && ib == 0) continue;
      double r1[3];
      for (int k = 0; k < 3; k++) r1[k] = RAT(s, i)[k] + s->xl[ib][k];
      for (int b = s->ppx_off[al]; b < s->ppx_off[al + 1]; b++) {
        int j = s->ppx_j[b], jb = s->ppx_b[b];
        if ((j == al && jb == 0) || a == b) continue;
        double r2[3], r[3];
        for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[jb][k], r[k] = r2[k] - r1[k];
        int m = -1;
        for (int k = s->ppp_off[i]; k < s->ppp_off[i + 1]; k++) {
          double r3[3];
          for (int c = 0; c < 3; c++) r3[c] = s->xl[s->ppp_b[k]][c] + RAT(s, s->ppp_j[k])[c] - RAT(s, i)[c];
          if (distance3(r, r3) < 1.0e-4) { m = k - s->ppp_off[i]; break; }
        }
        if (m < 0) continue;
        /* mpairnay: alpha in PP(i) and in PP(j) at the triplet's vectors */
        int mm[2];
        for (int w = 0; w < 2; w++) {
          int at = w ? j : i;
          const double *rr = w ? r2 : r1;
          double r12[3];
          for (int k = 0; k < 3; k++) r12[k] = RAT(s, al)[k] - rr[k];
          int imatch = 0;
          mm[w] = -1;
          for (int k = s->pp_off[at]; k < s->pp_off[at + 1]; k++) {
            if (s->pp_j[k] != al) continue;
            double r21[3];
            for (int c = 0; c < 3; c++) r21[c] = RAT(s, al)[c] + s->xl[s->pp_b[k]][c] - RAT(s, at)[c];
            if (distance3(r12, r21) < 0.0001) { imatch++; mm[w] = k - s->pp_off[at]; }
          }
          if (imatch != 1) { seterr("mpairnay: imatch = %d for atoms %d, %d", imatch, at + 1, al + 1); return E_BACK; }
        }
        ivec_push(&CI, i); ivec_push(&CIB, ib); ivec_push(&CJ, j); ivec_push(&CJB, jb);
        ivec_push(&CM, m); ivec_push(&C31, mm[0]); ivec_push(&C32, mm[1]);
      }
    }
    s->ppc_off[al + 1] = CI.n;
  }
  s->ppc_i = CI.v; s->ppc_ib = CIB.v; s->ppc_j = CJ.v; s->ppc_jb = CJB.v;
  s->ppc_m = CM.v; s->ppc_m31 = C31.v; s->ppc_m32 = C32.v;
  s->have_pp = 1;
  return OK;
}

void or_pp_sizes(const or_sys *s, int *npp, int *nppx, int *nppp, int *ntrip, long long *nsvnl, long long *nvnl) {
  int N = s->natoms;
  *npp = s->pp_off[N];
  *nppx = s->ppx_off[N];
  *nppp = s->ppp_off[N];
  *ntrip = s->ppc_off[N];
  *nsvnl = s->nsvnl;
  *nvnl = s->nvnl;
}

/* which: 0 PP (off, j, b, self, map), 1 PPx (off, j, b, self, map, point),
 * 2 PPp (off, j, b, self); 0-based */
void or_get_pp(const or_sys *s, int which, int *off, int *jj, int *bb, int *self, int *map, int *point) {
  int N = s->natoms;
  const int *o = which == 0 ? s->pp_off : which == 1 ? s->ppx_off : s->ppp_off;
  const int *J = which == 0 ? s->pp_j : which == 1 ? s->ppx_j : s->ppp_j;
  const int *B = which == 0 ? s->pp_b : which == 1 ? s->ppx_b : s->ppp_b;
  const int *S = which == 0 ? s->pp_self : which == 1 ? s->ppx_self : s->ppp_self;
  memcpy(off, o, sizeof(int) * (N + 1));
  memcpy(jj, J, sizeof(int) * o[N]);
  memcpy(bb, B, sizeof(int) * o[N]);
  memcpy(self, S, sizeof(int) * N);
  if (map && which < 2) memcpy(map, which == 0 ? s->pp_map : s->ppx_map, sizeof(int) * o[N]);
  if (point && which == 1) memcpy(point, s->ppx_point, sizeof(int) * o[N]);
}

void or_get_pp_common(const or_sys *s, int *off, int *ci, int *cib, int *cj, int *cjb, int *m, int *m31, int *m32) {
  int N = s->natoms, T = s->ppc_off[N];
  memcpy(off, s->ppc_off, sizeof(int) * (N + 1));
  memcpy(ci, s->ppc_i, sizeof(int) * T); memcpy(cib, s->ppc_ib, sizeof(int) * T);
  memcpy(cj, s->ppc_j, sizeof(int) * T); memcpy(cjb, s->ppc_jb, sizeof(int) * T);
  memcpy(m, s->ppc_m, sizeof(int) * T); memcpy(m31, s->ppc_m31, sizeof(int) * T);
  memcpy(m32, s->ppc_m32, sizeof(int) * T);
}

/* the PP pair frame: z, sighat, eps = epsilon(r2, sighat) */
static void pp_frame(const or_sys *s, int i, int j, int mb, double *r1, double *r2, double *z, double *eps) {
  double sighat[3];
  for (int k = 0; k < 3; k++) {
    r1[k] = RAT(s, i)[k];
    r2[k] = RAT(s, j)[k] + s->xl[mb][k];
  }
  *z = distance3(r1, r2);
  if (*z < 1.0e-05) {
    sighat[0] = 0.0; sighat[1] = 0.0; sighat[2] = 1.0;
  } else {
    for (int k = 0; k < 3; k++) sighat[k] = (r2[k] - r1[k]) / *z;
  }
  or_epsilon(r2, sighat, eps);
}

/* cl(ispecies) (b.FUNCTIONS/cl.f90:50-90): the shell's cl for each of its
 * 2l+1 projector orbitals */
static void cl_values(const species_t *sp, double *cl) {
  int k = 0;
  for (int issh = 0; issh < sp->nssh_PP; issh++)
    for (int m = 0; m < 2 * sp->lssh_PP[issh] + 1; m++) cl[k++] = sp->cl_PP[issh];
}

/* assemble_svnl (j.ASSEMBLERS/M_assemble_PP_2c.f90:86-206) */
int or_assemble_svnl(or_sys *s, double *svnl) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int i = 0; i < s->natoms; i++) {
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max;
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      int j = s->pp_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_PP_max, st;
      double r1[3], r2[3], z, eps[9], mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
      pp_frame(s, i, j, s->pp_b[p], r1, r2, &z, eps);
      if ((st = or_getMEs_2c(fd, in1, in2, P_vnl, 0, z, nmu, nnu, mm))) { err = st; continue; }
      rotate_pp(fd, in1, in2, eps, nmu, nnu, mm, xm);
      memcpy(svnl + s->svnl_off[p], xm, sizeof(double) * nmu * nnu);
    }
  }
  return err;
}

/* PPx(imu, inu) = sum_ncc cl(ncc) A(imu, ncc) B(inu, ncc), A, B column-major
 * with leading dimensions na, nb */
static void cl_product(const double *cl, int ncl, const double *A, int na, const double *B, int nb, double *out) {
  for (int inu = 0; inu < nb; inu++)
    for (int imu = 0; imu < na; imu++) {
      double acc = 0.0;
      for (int ncc = 0; ncc < ncl; ncc++) acc = acc + cl[ncc] * A[imu + na * ncc] * B[inu + nb * ncc];
      out[imu + na * inu] = acc;
    }
}

/* assemble_vnl_2c (j.ASSEMBLERS/M_assemble_PP_2c.f90:232-511): the vnl
 * blocks over PPp, the atom (both orbitals on i, projector on a PP
 * neighbor), ontop left (projector on i, PPx pairs) and ontop right
 * (projector on j, PP pairs) terms */
int or_assemble_vnl_2c(or_sys *s, const double *svnl, double *vnl) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double cl[MAXORB], PPx[MAXORB * MAXORB];
  for (long long k = 0; k < s->nvnl; k++) vnl[k] = 0.0;
  for (int i = 0; i < N; i++) {  /* atom */
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max;
    double *dst = vnl + s->vnl_off[s->ppp_off[i] + s->ppp_self[i]];
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      int in2 = s->imass[s->pp_j[p]];
      cl_values(&fd->sp[in2], cl);
      const double *b = svnl + s->svnl_off[p];
      cl_product(cl, fd->sp[in2].norb_PP_max, b, nmu, b, nmu, PPx);
      for (int k = 0; k < nmu * nmu; k++) dst[k] = dst[k] + PPx[k];
    }
  }
  for (int i = 0; i < N; i++) {  /* ontop left */
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max;
    cl_values(&fd->sp[in1], cl);
    for (int p = s->ppx_off[i]; p < s->ppx_off[i + 1]; p++) {
      int j = s->ppx_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      if (j == i && s->ppx_b[p] == 0) continue;
      const double *b1 = svnl + s->svnl_off[s->pp_off[i] + s->pp_self[i]];
      const double *b2 = svnl + s->svnl_off[s->pp_off[j] + s->ppx_point[p]];
      cl_product(cl, fd->sp[in1].norb_PP_max, b1, nmu, b2, nnu, PPx);
      double *dst = vnl + s->vnl_off[s->ppp_off[i] + s->ppx_map[p]];
      for (int k = 0; k < nmu * nnu; k++) dst[k] = dst[k] + PPx[k];
    }
  }
  for (int i = 0; i < N; i++) {  /* ontop right */
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max;
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      int j = s->pp_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      if (j == i && s->pp_b[p] == 0) continue;
      cl_values(&fd->sp[in2], cl);
      const double *b1 = svnl + s->svnl_off[p];
      const double *b2 = svnl + s->svnl_off[s->pp_off[j] + s->pp_self[j]];
      cl_product(cl, fd->sp[in2].norb_PP_max, b1, nmu, b2, nnu, PPx);
      double *dst = vnl + s->vnl_off[s->ppp_off[i] + s->pp_map[p]];
      for (int k = 0; k < nmu * nnu; k++) dst[k] = dst[k] + PPx[k];
    }
  }
  return OK;
}

/* assemble_vnl_3c (j.ASSEMBLERS/M_assemble_PP_3c.f90:94-229), accumulating */
int or_assemble_vnl_3c(or_sys *s, const double *svnl, double *vnl) {
  or_fdata *fd = s->fd;
  double cl[MAXORB], PPx[MAXORB * MAXORB];
  for (int al = 0; al < s->natoms; al++) {
    int indna = s->imass[al];
    cl_values(&fd->sp[indna], cl);
    for (int t = s->ppc_off[al]; t < s->ppc_off[al + 1]; t++) {
      int i = s->ppc_i[t], j = s->ppc_j[t];
      int nmu = fd->sp[s->imass[i]].norb_max, nnu = fd->sp[s->imass[j]].norb_max;
      const double *b1 = svnl + s->svnl_off[s->pp_off[i] + s->ppc_m31[t]];
      const double *b2 = svnl + s->svnl_off[s->pp_off[j] + s->ppc_m32[t]];
      cl_product(cl, fd->sp[indna].norb_PP_max, b1, nmu, b2, nnu, PPx);
      double *dst = vnl + s->vnl_off[s->ppp_off[i] + s->ppc_m[t]];
      for (int k = 0; k < nmu * nnu; k++) dst[k] = dst[k] + PPx[k];
    }
  }
  return OK;
}

/* Dassemble_svnl (k.DASSEMBLERS/M_Dassemble_PP_2c.f90:296-380): Dblock(3,
 * mu, ncc) of svnl, the derivative with respect to the basis atom i */
int or_dassemble_svnl(or_sys *s, double *dsvnl) {
  or_fdata *fd = s->fd;
  int err = OK;
  for (int i = 0; i < s->natoms; i++) {
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max;
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      int j = s->pp_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_PP_max, st;
      double r1[3], r2[3], z, eps[9], deps[27], eta[3];
      double mm[MAXORB * MAXORB], dm[MAXORB * MAXORB], vdm[3 * MAXORB * MAXORB], vdx[3 * MAXORB * MAXORB];
      pp_frame(s, i, j, s->pp_b[p], r1, r2, &z, eps);
      or_depsilon_2c(r1, r2, z, eps, deps);
      for (int k = 0; k < nmu * nnu; k++) mm[k] = dm[k] = 0.0;
      for (int k = 0; k < 3 * nmu * nnu; k++) vdm[k] = 0.0;
      if ((st = or_getDMEs_2c(fd, in1, in2, P_vnl, 0, z, nmu, nnu, mm, dm))) { err = st; continue; }
      for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++)
          if (z > 1.0e-3)
            for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
      drotate_pp(fd, in1, in2, eps, deps, nmu, nnu, mm, vdm, vdx);
      memcpy(dsvnl + 3 * s->svnl_off[p], vdx, sizeof(double) * 3 * nmu * nnu);
    }
  }
  return err;
}

/* Dassemble_vnl_2c (k.DASSEMBLERS/M_Dassemble_PP_2c.f90:420-745): vnl_atom
 * per PP pair (self skipped), vnl_ontop per PPx pair (ontop left; the ontop
 * right force is commented out in the reference, :737-738, and build_forces
 * doubles the left one instead); rho_pp is the density over PPp */
int or_dassemble_vnl_2c(or_sys *s, const double *rho_pp, const double *svnl, const double *dsvnl, double *vnl_atom,
                        double *vnl_ontop) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double cl[MAXORB];
  for (int k = 0; k < 3 * s->pp_off[N]; k++) vnl_atom[k] = 0.0;
  for (int k = 0; k < 3 * s->ppx_off[N]; k++) vnl_ontop[k] = 0.0;
  for (int i = 0; i < N; i++) {
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max;
    const double *rs = rho_pp + s->vnl_off[s->ppp_off[i] + s->ppp_self[i]];
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      if (p - s->pp_off[i] == s->pp_self[i]) continue;
      int in2 = s->imass[s->pp_j[p]], ncl = fd->sp[in2].norb_PP_max;
      cl_values(&fd->sp[in2], cl);
      const double *b = svnl + s->svnl_off[p], *D = dsvnl + 3 * s->svnl_off[p];
      double *f = vnl_atom + 3 * (size_t)p;
      for (int inu = 0; inu < nmu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          double x[3] = {0, 0, 0};
          for (int ncc = 0; ncc < ncl; ncc++)
            for (int c = 0; c < 3; c++)
              x[c] = x[c] + cl[ncc] * (D[c + 3 * (imu + nmu * ncc)] * b[inu + nmu * ncc] +
                                       b[imu + nmu * ncc] * D[c + 3 * (inu + nmu * ncc)]);
          for (int c = 0; c < 3; c++) f[c] = f[c] - rs[imu + nmu * inu] * x[c];
        }
    }
  }
  for (int i = 0; i < N; i++) {
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, ncl = fd->sp[in1].norb_PP_max;
    cl_values(&fd->sp[in1], cl);
    for (int p = s->ppx_off[i]; p < s->ppx_off[i + 1]; p++) {
      int j = s->ppx_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      if (j == i && s->ppx_b[p] == 0) continue;
      const double *b1 = svnl + s->svnl_off[s->pp_off[i] + s->pp_self[i]];
      const double *D2 = dsvnl + 3 * s->svnl_off[s->pp_off[j] + s->ppx_point[p]];
      const double *r = rho_pp + s->vnl_off[s->ppp_off[i] + s->ppx_map[p]];
      double *f = vnl_ontop + 3 * (size_t)p;
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          double x[3] = {0, 0, 0};
          for (int ncc = 0; ncc < ncl; ncc++)
            for (int c = 0; c < 3; c++)
              x[c] = x[c] - cl[ncc] * b1[imu + nmu * ncc] * D2[c + 3 * (inu + nnu * ncc)];
          for (int c = 0; c < 3; c++) f[c] = f[c] - r[imu + nmu * inu] * x[c];
        }
    }
  }
  return OK;
}

/* Dassemble_vnl_3c (k.DASSEMBLERS/M_Dassemble_PP_3c.f90:127-265) */
int or_dassemble_vnl_3c(or_sys *s, const double *rho_pp, const double *svnl, const double *dsvnl, double *f3nla,
                        double *f3nlb, double *f3nlc) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double cl[MAXORB];
  for (int k = 0; k < 3 * N; k++) f3nla[k] = f3nlb[k] = f3nlc[k] = 0.0;
  for (int al = 0; al < N; al++) {
    int indna = s->imass[al], ncl = fd->sp[indna].norb_PP_max;
    cl_values(&fd->sp[indna], cl);
    for (int t = s->ppc_off[al]; t < s->ppc_off[al + 1]; t++) {
      int i = s->ppc_i[t], j = s->ppc_j[t];
      int nmu = fd->sp[s->imass[i]].norb_max, nnu = fd->sp[s->imass[j]].norb_max;
      long long o1 = s->svnl_off[s->pp_off[i] + s->ppc_m31[t]], o2 = s->svnl_off[s->pp_off[j] + s->ppc_m32[t]];
      const double *b1 = svnl + o1, *b2 = svnl + o2, *D1 = dsvnl + 3 * o1, *D2 = dsvnl + 3 * o2;
      const double *r = rho_pp + s->vnl_off[s->ppp_off[i] + s->ppc_m[t]];
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          double xb[3] = {0, 0, 0}, xc[3] = {0, 0, 0};
          for (int ncc = 0; ncc < ncl; ncc++)
            for (int c = 0; c < 3; c++) {
              xb[c] = xb[c] + cl[ncc] * D1[c + 3 * (imu + nmu * ncc)] * b2[inu + nnu * ncc];
              xc[c] = xc[c] + cl[ncc] * b1[imu + nmu * ncc] * D2[c + 3 * (inu + nnu * ncc)];
            }
          double rr = r[imu + nmu * inu];
          for (int c = 0; c < 3; c++) {
            double xa = -xb[c] - xc[c];
            f3nla[3 * al + c] = f3nla[3 * al + c] - rr * xa;
            f3nlb[3 * i + c] = f3nlb[3 * i + c] - rr * xb[c];
            f3nlc[3 * j + c] = f3nlc[3 * j + c] - rr * xc[c];
          }
        }
    }
  }
  return OK;
}

/* build_forces, vnl terms (c.SYSTEM/M_build_forces.f90:395-461): vnl(i) =
 * sum of vnl_atom over PP pairs (i +, j -) and 2 vnl_ontop over PPx pairs
 * (i +, j -); ftot_add = vnl + f3nla + f3nlb + f3nlc */
int or_build_forces_vnl(or_sys *s, const double *vnl_atom, const double *vnl_ontop, const double *f3nla,
                        const double *f3nlb, const double *f3nlc, double *vnl, double *ftot_add) {
  int N = s->natoms;
  for (int k = 0; k < 3 * N; k++) vnl[k] = 0.0;
  for (int i = 0; i < N; i++) {
    for (int p = s->pp_off[i]; p < s->pp_off[i + 1]; p++) {
      int j = s->pp_j[p];
      for (int c = 0; c < 3; c++) {
        vnl[3 * i + c] = vnl[3 * i + c] + vnl_atom[3 * p + c];
        vnl[3 * j + c] = vnl[3 * j + c] - vnl_atom[3 * p + c];
      }
    }
    for (int p = s->ppx_off[i]; p < s->ppx_off[i + 1]; p++) {
      int j = s->ppx_j[p];
      for (int c = 0; c < 3; c++) {
        vnl[3 * i + c] = vnl[3 * i + c] + 2.0 * vnl_ontop[3 * p + c];
        vnl[3 * j + c] = vnl[3 * j + c] - 2.0 * vnl_ontop[3 * p + c];
      }
    }
  }
  for (int k = 0; k < 3 * N; k++) ftot_add[k] = vnl[k] + f3nla[k] + f3nlb[k] + f3nlc[k];
  return OK;
}

/* ------------------------------------------------------------------------ */
/* Ewald (DOGS): the long-range Coulomb matrix and the ewaldsr / ewaldlr     */
/* blocks (j.ASSEMBLERS/M_assemble_ewald_DOGS.f90)                           */
/* ------------------------------------------------------------------------ */
/* total charge of each atom, dQ(i) = sum over its shells of Qin - Qneutral */
static void atom_dq(const or_sys *s, double *dq) {
  for (int i = 0; i < s->natoms; i++) {
    dq[i] = 0.0;
    for (int k = 1; k <= s->fd->sp[s->imass[i]].nssh; k++) dq[i] = dq[i] + shell_dq(s, i, k);
  }
}

/* assemble_ewald (:633-918): ewald(i, j) (row-major N x N here) */
int or_assemble_ewald(or_sys *s, double *ewald) {
  int N = s->natoms;
  const double pi = 3.141592653589793238462643;
  double a1[3], a2[3], a3[3], c[3], g1[3], g2[3], g3[3];
  for (int k = 0; k < 3; k++) a1[k] = s->lattice[0][k], a2[k] = s->lattice[1][k], a3[k] = s->lattice[2][k];
  for (long long k = 0; k < (long long)N * N; k++) ewald[k] = 0.0;
  cross3(a2, a3, c);
  double volume = a1[0] * c[0] + a1[1] * c[1] + a1[2] * c[2];
  for (int k = 0; k < 3; k++) g1[k] = 2.0 * pi * c[k] / volume;
  cross3(a3, a1, c);
  for (int k = 0; k < 3; k++) g2[k] = 2.0 * pi * c[k] / volume;
  cross3(a1, a2, c);
  for (int k = 0; k < 3; k++) g3[k] = 2.0 * pi * c[k] / volume;
  volume = fabs(volume);
  double gmax = 5.0, rmax = 5.0;
  double g1m2 = pow(magnitude3(g1), 2), g2m2 = pow(magnitude3(g2), 2), g3m2 = pow(magnitude3(g3), 2);
  double r1m2 = pow(magnitude3(a1), 2), r2m2 = pow(magnitude3(a2), 2), r3m2 = pow(magnitude3(a3), 2);
  double rmin2 = r1m2;
  if (r2m2 < rmin2) rmin2 = r2m2;
  if (r3m2 < rmin2) rmin2 = r3m2;
  double gmin2 = g1m2;
  if (g2m2 < gmin2) gmin2 = g2m2;
  if (g3m2 < gmin2) gmin2 = g3m2;
  double kappa = sqrt(sqrt(gmin2 / (4.0 * rmin2)));
  int ig1 = (int)(gmax * sqrt(4.0 * kappa * kappa / g1m2) + 1.0);
  int ig2 = (int)(gmax * sqrt(4.0 * kappa * kappa / g2m2) + 1.0);
  int ig3 = (int)(gmax * sqrt(4.0 * kappa * kappa / g3m2) + 1.0);
  if (ig1 <= 1) ig1 = 2;
  if (ig2 <= 1) ig2 = 2;
  if (ig3 <= 1) ig3 = 2;
  int il1 = (int)(rmax * sqrt(1.0 / (kappa * kappa * r1m2)) + 1.0);
  int il2 = (int)(rmax * sqrt(1.0 / (kappa * kappa * r2m2)) + 1.0);
  int il3 = (int)(rmax * sqrt(1.0 / (kappa * kappa * r3m2)) + 1.0);
  if (il1 <= 1) il1 = 2;
  if (il2 <= 1) il2 = 2;
  if (il3 <= 1) il3 = 2;
  if (s->icluster == 1) ig1 = ig2 = ig3 = 0;
  for (int n1 = -ig1; n1 <= ig1; n1++)
    for (int n2 = -ig2; n2 <= ig2; n2++)
      for (int n3 = -ig3; n3 <= ig3; n3++) {
        if (n1 == 0 && n2 == 0 && n3 == 0) continue;
        double g[3];
        for (int k = 0; k < 3; k++) g[k] = n1 * g1[k] + n2 * g2[k] + n3 * g3[k];
        double gm2 = pow(magnitude3(g), 2);
        double argument = gm2 / (4.0 * kappa * kappa);
        double stuff = 4.0 * pi * exp(-argument) / (gm2 * volume);
        for (int i = 0; i < N; i++)
          for (int j = i; j < N; j++) {
            double factor = j == i ? 0.5 * stuff : 1.0 * stuff;
            double gdotb = g[0] * (RAT(s, i)[0] - RAT(s, j)[0]) + g[1] * (RAT(s, i)[1] - RAT(s, j)[1]) +
                           g[2] * (RAT(s, i)[2] - RAT(s, j)[2]);
            ewald[(size_t)i * N + j] = ewald[(size_t)i * N + j] + factor * cos(gdotb);
            ewald[(size_t)j * N + i] = ewald[(size_t)j * N + i] + factor * cos(gdotb);
          }
      }
  if (s->icluster == 1) {
    il1 = il2 = il3 = 0;
    kappa = 0.0;
  }
  for (int n1 = -il1; n1 <= il1; n1++)
    for (int n2 = -il2; n2 <= il2; n2++)
      for (int n3 = -il3; n3 <= il3; n3++)
        for (int i = 0; i < N; i++)
          for (int j = i; j < N; j++) {
            double factor = j == i ? 0.5 : 1.0;
            double cv[3];
            for (int k = 0; k < 3; k++) cv[k] = n1 * a1[k] + n2 * a2[k] + n3 * a3[k];
            for (int k = 0; k < 3; k++) cv[k] = cv[k] + RAT(s, i)[k] - RAT(s, j)[k];
            double z = sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
            if (z > 0.0001) {
              double argument = kappa * z;
              ewald[(size_t)i * N + j] = ewald[(size_t)i * N + j] + factor * erfc(argument) / z;
              ewald[(size_t)j * N + i] = ewald[(size_t)j * N + i] + factor * erfc(argument) / z;
            }
          }
  for (int i = 0; i < N; i++) ewald[(size_t)i * N + i] = ewald[(size_t)i * N + i] - 2.0 * kappa / sqrt(pi);
  return OK;
}

/* assemble_ewaldsr (:98-378): per pair of the neighbor map (S and dip are
 * the overlap and z-dipole block sets), the atom term into the self block
 * (dQ_j S(i,self)/z), the ontop terms (dQ_i (S/2z + dip/z^2) + dQ_j (S/2z -
 * dip/z^2)) and the three-center terms over the common neighbors
 * ((sterm - dterm)/d13 + (sterm + dterm)/d23 with sterm = dQ_alpha S/2,
 * dterm = dQ_alpha dip/z), all times eq2 */
int or_assemble_ewaldsr(or_sys *s, const double *S, const double *dip, double *sr) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double *dq = (double *)malloc(sizeof(double) * N);
  atom_dq(s, dq);
  for (long long k = 0; k < s->nblock; k++) sr[k] = 0.0;
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    long long os = s->blk_off[s->pair_off[i] + s->neigh_self[i]];
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p];
      if (i == j && s->neigh_b[p] == 0) continue;
      double r2[3];
      for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[s->neigh_b[p]][k];
      double z = distance3(RAT(s, i), r2);
      for (int k = 0; k < nmu * nmu; k++) sr[os + k] = sr[os + k] + dq[j] * (S[os + k] / z) * P_eq2;
    }
  }
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], nnu = fd->sp[s->imass[j]].norb_max;
      if (i == j && s->neigh_b[p] == 0) continue;
      long long o = s->blk_off[p];
      double r2[3];
      for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[s->neigh_b[p]][k];
      double z = distance3(RAT(s, i), r2);
      for (int k = 0; k < nmu * nnu; k++) {
        double sterm = S[o + k] / (2.0 * z), dterm = dip[o + k] / (z * z);
        sr[o + k] = sr[o + k] + dq[i] * (sterm + dterm) * P_eq2;
        sr[o + k] = sr[o + k] + dq[j] * (sterm - dterm) * P_eq2;
      }
    }
  }
  for (int ia = 0; ia < N; ia++) {
    for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
      trip_t g;
      trip_frame(s, ia, t, &g);
      int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
      long long o = s->blk_off[s->pair_off[g.iatom] + g.mneigh];
      double d13 = distance3(g.rna, g.r1), d23 = distance3(g.rna, g.r2);
      for (int k = 0; k < nmu * nnu; k++) {
        double sterm = dq[ia] * S[o + k] / 2.0, dterm = dq[ia] * dip[o + k] / g.z;
        sr[o + k] = sr[o + k] + ((sterm - dterm) / d13 + (sterm + dterm) / d23) * P_eq2;
      }
    }
  }
  free(dq);
  return OK;
}

/* assemble_ewaldlr (:404-592): sum_ewald(i) = sum_j dQ_j ewald(i, j); per
 * pair (S/2 - dip/z) sum_ewald(i) eq2 + (S/2 + dip/z) sum_ewald(j) eq2, the
 * dipole term left out on the self pair */
int or_assemble_ewaldlr(or_sys *s, const double *ewald, const double *S, const double *dip, double *lr) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double *dq = (double *)malloc(sizeof(double) * N), *se = (double *)calloc(N, sizeof(double));
  atom_dq(s, dq);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) se[i] = se[i] + dq[j] * ewald[(size_t)i * N + j];
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], nnu = fd->sp[s->imass[j]].norb_max;
      long long o = s->blk_off[p];
      double r2[3];
      for (int k = 0; k < 3; k++) r2[k] = RAT(s, j)[k] + s->xl[s->neigh_b[p]][k];
      double z = distance3(RAT(s, i), r2);
      int self = i == j && s->neigh_b[p] == 0;
      for (int k = 0; k < nmu * nnu; k++) {
        double sterm = S[o + k] / 2.0, dterm = self ? 0.0 : dip[o + k] / z;
        lr[o + k] = 0.0 + (sterm - dterm) * se[i] * P_eq2 + (sterm + dterm) * se[j] * P_eq2;
      }
    }
  }
  free(dq);
  free(se);
  return OK;
}

/* ------------------------------------------------------------------------ */
/* Ewald force pass (DOGS, k.DASSEMBLERS/M_Dassemble_ewald_DOGS.f90)         */
/* ------------------------------------------------------------------------ */
/* Dassemble_ewald (:878-1236): dewald(:, i, j) = derivative of ewald(i, j)
 * with respect to r_i ([(i * N + j) * 3 + c]), and the Ewald energy force
 * fewald(i) with qq = Q_i Q_j - Q0_i Q0_j (Q = Q0 + dQ) */
int or_dassemble_ewald(or_sys *s, double *dewald, double *fewald) {
  int N = s->natoms;
  const double pi = 3.141592653589793238462643;
  double *dq = (double *)malloc(sizeof(double) * N), *Q = (double *)malloc(sizeof(double) * N),
         *Q0 = (double *)malloc(sizeof(double) * N);
  atom_dq(s, dq);
  for (int i = 0; i < N; i++) Q0[i] = s->fd->sp[s->imass[i]].Q0, Q[i] = Q0[i] + dq[i];
  for (long long k = 0; k < 3LL * N * N; k++) dewald[k] = 0.0;
  for (int k = 0; k < 3 * N; k++) fewald[k] = 0.0;
  double a1[3], a2[3], a3[3], c[3], g1[3], g2[3], g3[3];
  for (int k = 0; k < 3; k++) a1[k] = s->lattice[0][k], a2[k] = s->lattice[1][k], a3[k] = s->lattice[2][k];
  cross3(a2, a3, c);
  double volume = a1[0] * c[0] + a1[1] * c[1] + a1[2] * c[2];
  for (int k = 0; k < 3; k++) g1[k] = 2.0 * pi * c[k] / volume;
  cross3(a3, a1, c);
  for (int k = 0; k < 3; k++) g2[k] = 2.0 * pi * c[k] / volume;
  cross3(a1, a2, c);
  for (int k = 0; k < 3; k++) g3[k] = 2.0 * pi * c[k] / volume;
  volume = fabs(volume);
  double gmax = 5.0, rmax = 5.0;
  double g1m2 = pow(magnitude3(g1), 2), g2m2 = pow(magnitude3(g2), 2), g3m2 = pow(magnitude3(g3), 2);
  double r1m2 = pow(magnitude3(a1), 2), r2m2 = pow(magnitude3(a2), 2), r3m2 = pow(magnitude3(a3), 2);
  double rmin2 = r1m2;
  if (r2m2 < rmin2) rmin2 = r2m2;
  if (r3m2 < rmin2) rmin2 = r3m2;
  double gmin2 = g1m2;
  if (g2m2 < gmin2) gmin2 = g2m2;
  if (g3m2 < gmin2) gmin2 = g3m2;
  double kappa = sqrt(sqrt(gmin2 / (4.0 * rmin2)));
  int ig1 = (int)(gmax * sqrt(4.0 * kappa * kappa / g1m2) + 1.0);
  int ig2 = (int)(gmax * sqrt(4.0 * kappa * kappa / g2m2) + 1.0);
  int ig3 = (int)(gmax * sqrt(4.0 * kappa * kappa / g3m2) + 1.0);
  if (ig1 <= 1) ig1 = 2;
  if (ig2 <= 1) ig2 = 2;
  if (ig3 <= 1) ig3 = 2;
  int il1 = (int)(rmax * sqrt(1.0 / (kappa * kappa * r1m2)) + 1.0);
  int il2 = (int)(rmax * sqrt(1.0 / (kappa * kappa * r2m2)) + 1.0);
  int il3 = (int)(rmax * sqrt(1.0 / (kappa * kappa * r3m2)) + 1.0);
  if (il1 <= 1) il1 = 2;
  if (il2 <= 1) il2 = 2;
  if (il3 <= 1) il3 = 2;
  if (s->icluster == 1) ig1 = ig2 = ig3 = 0;
  for (int n1 = -ig1; n1 <= ig1; n1++)
    for (int n2 = -ig2; n2 <= ig2; n2++)
      for (int n3 = -ig3; n3 <= ig3; n3++) {
        if (n1 == 0 && n2 == 0 && n3 == 0) continue;
        double g[3];
        for (int k = 0; k < 3; k++) g[k] = n1 * g1[k] + n2 * g2[k] + n3 * g3[k];
        double gm2 = pow(magnitude3(g), 2);
        double stuff = 4.0 * pi * exp(-gm2 / (4.0 * kappa * kappa)) / (gm2 * volume);
        for (int i = 0; i < N; i++)
          for (int j = i; j < N; j++) {
            double factor = j == i ? 0.5 * stuff : 1.0 * stuff, factorf = 2.0 * stuff;
            double gdotb = g[0] * (RAT(s, i)[0] - RAT(s, j)[0]) + g[1] * (RAT(s, i)[1] - RAT(s, j)[1]) +
                           g[2] * (RAT(s, i)[2] - RAT(s, j)[2]);
            double qq = Q[i] * Q[j] - Q0[i] * Q0[j], sn = sin(gdotb);
            for (int k = 0; k < 3; k++) {
              fewald[3 * i + k] = fewald[3 * i + k] + qq * factorf * sn * g[k];
              fewald[3 * j + k] = fewald[3 * j + k] - qq * factorf * sn * g[k];
              dewald[((size_t)i * N + j) * 3 + k] = dewald[((size_t)i * N + j) * 3 + k] - factor * sn * g[k];
              dewald[((size_t)j * N + i) * 3 + k] = dewald[((size_t)j * N + i) * 3 + k] + factor * sn * g[k];
            }
          }
      }
  if (s->icluster == 1) {
    il1 = il2 = il3 = 0;
    kappa = 0.0;
  }
  for (int n1 = -il1; n1 <= il1; n1++)
    for (int n2 = -il2; n2 <= il2; n2++)
      for (int n3 = -il3; n3 <= il3; n3++)
        for (int i = 0; i < N; i++)
          for (int j = i; j < N; j++) {
            double factor = j == i ? 0.5 : 1.0, factorf = 2.0;
            double cv[3];
            for (int k = 0; k < 3; k++) cv[k] = n1 * a1[k] + n2 * a2[k] + n3 * a3[k];
            for (int k = 0; k < 3; k++) cv[k] = cv[k] + RAT(s, i)[k] - RAT(s, j)[k];
            double z = sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
            if (z > 0.0001) {
              double argument = kappa * z, qq = Q[i] * Q[j] - Q0[i] * Q0[j];
              double F = (2.0 * exp(-argument * argument) * kappa * z / sqrt(pi) + erfc(argument)) / (z * z * z);
              for (int k = 0; k < 3; k++) {
                fewald[3 * i + k] = fewald[3 * i + k] + qq * factorf * cv[k] * F;
                fewald[3 * j + k] = fewald[3 * j + k] - qq * factorf * cv[k] * F;
                dewald[((size_t)i * N + j) * 3 + k] = dewald[((size_t)i * N + j) * 3 + k] - factor * cv[k] * F;
                dewald[((size_t)j * N + i) * 3 + k] = dewald[((size_t)j * N + i) * 3 + k] + factor * cv[k] * F;
              }
            }
          }
  free(dq); free(Q); free(Q0);
  return OK;
}

/* Dassemble_ewaldsr (:94-527): per pair fsr(3, pair) (atom and ontop terms,
 * the self pair zero) and the three-center terms added into f3naa/b/c */
int or_dassemble_ewaldsr(or_sys *s, const double *rho, const double *S, const double *dS, const double *dip,
                         const double *ddip, double *fsr, double *f3naa, double *f3nab, double *f3nac) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double *dq = (double *)malloc(sizeof(double) * N);
  atom_dq(s, dq);
  for (int k = 0; k < 3 * s->npairs; k++) fsr[k] = 0.0;
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    long long os = s->blk_off[s->pair_off[i] + s->neigh_self[i]];
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p];
      double r1[3], r2[3], z, eps[9], sig[3];
      pair_frame(s, i, p, r1, r2, &z, eps);
      if (z < 1.0e-05) sig[0] = 0.0, sig[1] = 0.0, sig[2] = 1.0;
      else for (int k = 0; k < 3; k++) sig[k] = (r2[k] - r1[k]) / z;
      if (i == j && s->neigh_b[p] == 0) continue;
      for (int inu = 0; inu < nmu; inu++)
        for (int imu = 0; imu < nmu; imu++)
          for (int k = 0; k < 3; k++)
            fsr[3 * p + k] = fsr[3 * p + k] - P_eq2 * rho[os + imu + nmu * inu] * dq[j] *
                                                  (S[os + imu + nmu * inu] / (z * z)) * sig[k];
    }
  }
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], nnu = fd->sp[s->imass[j]].norb_max;
      if (i == j && s->neigh_b[p] == 0) continue;
      double r1[3], r2[3], z, eps[9], sig[3];
      pair_frame(s, i, p, r1, r2, &z, eps);
      if (z < 1.0e-05) sig[0] = 0.0, sig[1] = 0.0, sig[2] = 1.0;
      else for (int k = 0; k < 3; k++) sig[k] = (r2[k] - r1[k]) / z;
      long long o = s->blk_off[p];
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          long long e = o + imu + nmu * inu;
          double r = rho[e], sterm = S[e] / (2.0 * z), dterm = dip[e] / (z * z);
          for (int k = 0; k < 3; k++) {
            double spterm = dS[3 * e + k] / (2.0 * z), dpterm = ddip[3 * e + k] / (z * z);
            fsr[3 * p + k] = fsr[3 * p + k] - P_eq2 * r * dq[i] * (spterm + dpterm) -
                             P_eq2 * r * dq[i] * (sterm + 2.0 * dterm) * (sig[k] / z) -
                             P_eq2 * r * dq[j] * (spterm - dpterm) -
                             P_eq2 * r * dq[j] * (sterm - 2.0 * dterm) * (sig[k] / z);
          }
        }
    }
  }
  for (int ia = 0; ia < N; ia++) {
    for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
      trip_t g;
      trip_frame(s, ia, t, &g);
      int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
      long long o = s->blk_off[s->pair_off[g.iatom] + g.mneigh];
      double d13 = distance3(g.rna, g.r1), d23 = distance3(g.rna, g.r2), rA1[3] = {0, 0, 0}, rA2[3] = {0, 0, 0};
      if (d13 > 1.0e-05) for (int k = 0; k < 3; k++) rA1[k] = (g.rna[k] - g.r1[k]) / d13;
      if (d23 > 1.0e-05) for (int k = 0; k < 3; k++) rA2[k] = (g.rna[k] - g.r2[k]) / d23;
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          long long e = o + imu + nmu * inu;
          double r = rho[e], sterm = S[e] / 2.0, dterm = dip[e] / g.z;
          for (int k = 0; k < 3; k++) {
            double spterm = dS[3 * e + k] / 2.0;
            double dpterm = ddip[3 * e + k] / g.z + dterm * g.sighat[k] / g.z;
            double A = -dq[ia] * (sterm - dterm) * rA1[k] / (d13 * d13) - dq[ia] * (sterm + dterm) * rA2[k] / (d23 * d23);
            double B = dq[ia] * (sterm - dterm) * rA1[k] / (d13 * d13) + dq[ia] * (spterm - dpterm) / d13 +
                       dq[ia] * (spterm + dpterm) / d23;
            A = -A;
            B = -B;
            double Cc = -A - B;
            f3naa[3 * ia + k] = f3naa[3 * ia + k] - P_eq2 * r * A;
            f3nab[3 * g.iatom + k] = f3nab[3 * g.iatom + k] - P_eq2 * r * B;
            f3nac[3 * g.jatom + k] = f3nac[3 * g.jatom + k] - P_eq2 * r * Cc;
          }
        }
    }
  }
  free(dq);
  return OK;
}

/* Dassemble_ewaldlr (:553-837): flr(3, atom), with sum_ewald = ewald dQ and
 * sum_dewald = dewald dQ (dewald from or_dassemble_ewald) */
int or_dassemble_ewaldlr(or_sys *s, const double *rho, const double *ewald, const double *dewald, const double *S,
                         const double *dS, const double *dip, const double *ddip, double *flr) {
  or_fdata *fd = s->fd;
  int N = s->natoms;
  double *dq = (double *)malloc(sizeof(double) * N), *se = (double *)calloc(N, sizeof(double)),
         *sd = (double *)calloc(3 * (size_t)N, sizeof(double));
  atom_dq(s, dq);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      se[i] = se[i] + dq[j] * ewald[(size_t)i * N + j];
      for (int k = 0; k < 3; k++) sd[3 * i + k] = sd[3 * i + k] + dq[j] * dewald[((size_t)i * N + j) * 3 + k];
    }
  for (int k = 0; k < 3 * N; k++) flr[k] = 0.0;
#define DEW(a, b, k) dewald[((size_t)(a) * N + (b)) * 3 + (k)]
  for (int i = 0; i < N; i++) {
    int nmu = fd->sp[s->imass[i]].norb_max;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], nnu = fd->sp[s->imass[j]].norb_max;
      double r1[3], r2[3], z, eps[9], sig[3];
      pair_frame(s, i, p, r1, r2, &z, eps);
      if (z < 1.0e-05) sig[0] = 0.0, sig[1] = 0.0, sig[2] = 1.0;
      else for (int k = 0; k < 3; k++) sig[k] = (r2[k] - r1[k]) / z;
      long long o = s->blk_off[p];
      int self = i == j && s->neigh_b[p] == 0;
      for (int inu = 0; inu < nnu; inu++)
        for (int imu = 0; imu < nmu; imu++) {
          long long e = o + imu + nmu * inu;
          double r = rho[e], sterm = S[e] / 2.0, dterm = self ? 0.0 : dip[e] / z;
          for (int k = 0; k < 3; k++) {
            if (self) {
              flr[3 * i + k] = flr[3 * i + k] - P_eq2 * r * sterm * sd[3 * i + k];
              flr[3 * j + k] = flr[3 * j + k] - P_eq2 * r * sterm * sd[3 * j + k];
            } else {
              double spterm = dS[3 * e + k] / 2.0;
              double dpterm = ddip[3 * e + k] / z + dip[e] * sig[k] / (z * z);
              flr[3 * i + k] = flr[3 * i + k] - P_eq2 * r * (sterm - dterm) * sd[3 * i + k] -
                               P_eq2 * r * (spterm - dpterm) * se[i] -
                               P_eq2 * r * (sterm + dterm) * dq[i] * DEW(i, j, k) -
                               P_eq2 * r * (spterm + dpterm) * se[j];
              flr[3 * j + k] = flr[3 * j + k] - P_eq2 * r * (sterm - dterm) * dq[j] * DEW(j, i, k) +
                               P_eq2 * r * (spterm - dpterm) * se[i] -
                               P_eq2 * r * (sterm + dterm) * sd[3 * j + k] +
                               P_eq2 * r * (spterm + dpterm) * se[j];
            }
          }
          for (int ka = 0; ka < N; ka++) {
            if (ka == i || ka == j) continue;
            for (int k = 0; k < 3; k++)
              flr[3 * ka + k] = flr[3 * ka + k] - r * dq[ka] * P_eq2 * (sterm - dterm) * DEW(ka, i, k) -
                                r * dq[ka] * P_eq2 * (sterm + dterm) * DEW(ka, j, k);
          }
        }
    }
  }
#undef DEW
  free(dq); free(se); free(sd);
  return OK;
}

/* ======================================================================== */
/* McWEDA exchange-correlation, Harris (PRB 71, 235101 (2005)):             */
/* j.ASSEMBLERS/M_assemble_rho_McWEDA_Harris.f90 (input densities) and      */
/* j.ASSEMBLERS/M_assemble_vxc_McWEDA_Harris.f90 (the vxc blocks).          */
/* Orbital blocks use the pair layout (blk_off); the shell-level weighted   */
/* densities use 9 doubles per pair, element (issh, jssh) at                */
/* [9 p + issh + nssh_i jssh] (column-major nssh_i x nssh_j).               */
/* ======================================================================== */
#define P_vxc_ontop 7
#define P_rho_ontopL 15
#define P_rho_ontopR 16
#define P_rho_atom 17
#define P_rhoS_ontopL 19
#define P_rhoS_ontopR 20
#define P_rhoS_atom 21
#define P_rho_3c 1
#define P_rhoS_3c 2
#define P_Hartree (P_eq2 / P_abohr) /* include/constants.h:5 */
#define WSH 9                       /* doubles per pair of a shell-level block */

/* lda_ceperley_alder (g.XC_FUNCTIONALS/lda_ceperley_alder.f90:56-190):
 * out = exc, muxc, dexc, d2exc, dmuxc, d2muxc.  The low-density branch's
 * d2dec keeps the reference's (dden*3) factor (:142). */
void or_lda_ceperley_alder(double rh, double *out) {
  const double delta_rh = 1.0e-6;
  double exc, muxc, dexc, d2exc, dmuxc, d2muxc;
  double dec, ddec, d2dec, den, dden, d2den, d3den, ex, rho_third, rho, rhx, rs, rsl, sqrs;
  double d2nec, d2nex, d3nec, d3nex;
  rhx = sqrt(rh * rh + delta_rh);
  rho = rhx * (P_abohr * P_abohr * P_abohr);
  rho_third = pow(rho, 1.0 / 3.0);
  rs = 0.62035049 / rho_third;
  if (rho < 0.23873241) {
    sqrs = sqrt(rs);
    den = 1.0 + 1.0529 * sqrs + 0.3334 * rs;
    exc = -0.4581652 / rs - 0.1423 / den;
    muxc = exc - rs * (0.15273333 / (rs * rs) + (0.02497128 / sqrs + 0.01581427) / (den * den));
    dden = 1.0529 / (2.0 * sqrs) + 0.3334;
    d2den = (-0.5) * 1.0529 / (2.0 * rs * sqrs);
    d3den = (0.75) * 1.0529 / (2.0 * (rs * rs) * sqrs);
    dec = 0.1423 * dden / (den * den);
    ddec = -2.0 * 0.1423 * dden * dden / (den * den * den) + 0.1423 * d2den / (den * den);
    double dd3 = g_exact ? dden * dden * dden : dden * 3; /* the reference's form is (dden*3) */
    d2dec = 6.0 * 0.1423 * dd3 / (den * den * den * den) - 6.0 * 0.1423 * dden * d2den / (den * den * den) +
            0.1423 * d3den / (den * den);
  } else {
    rsl = log(rs);
    exc = -0.4581652 / rs - 0.0480 + 0.0311 * rsl - 0.0116 * rs + 0.002 * rs * rsl;
    muxc = exc - rs * (0.15273333 / (rs * rs) + 0.01036667 / rs - 0.003866667 + 0.00066667 * (1.0 + rsl));
    dec = 0.0311 / rs - 0.0116 + 0.0020 * (rsl + 1.0);
    ddec = -0.0311 / (rs * rs) + 0.0020 / rs;
    d2dec = 2.0 * 0.0311 / (rs * rs * rs) - 0.0020 / (rs * rs);
  }
  ex = -0.7385587664 * rho_third;
  dexc = (muxc - exc) / rho;
  d2nec = (4.0 * rs / (9.0 * rho * rho)) * dec + (rs * rs / (9.0 * rho * rho)) * ddec;
  d2nex = -(2.0 / (9.0 * rho * rho)) * ex;
  dmuxc = 2.0 * dexc + rho * (d2nex + d2nec);
  d3nec = (-28.0 * rs / (27.0 * rho * rho * rho)) * dec + (-4.0 * rs * rs / (9.0 * rho * rho * rho)) * ddec +
          ((rs * rs * rs) / (-27.0 * rho * rho * rho)) * d2dec;
  d3nex = (10.0 / (27.0 * rho * rho * rho)) * ex;
  d2muxc = 3.0 * (d2nex + d2nec) + rho * (d3nex + d3nec);
  d2exc = d2nex + d2nec;
  {
    const double a3 = P_abohr * P_abohr * P_abohr, a6 = a3 * a3;
    out[0] = exc * P_Hartree;
    out[1] = muxc * P_Hartree;
    out[2] = dexc * P_Hartree * a3;
    out[3] = d2exc * P_Hartree * a6;
    out[4] = dmuxc * P_Hartree * a3;
    out[5] = d2muxc * P_Hartree * a6;
  }
}

/* assemble_rho_2c (:81-276) and assemble_rho_weighted_2c (:427-622) of
 * M_assemble_rho_McWEDA_Harris.f90: rho_in = rho_bond = sum over the shells
 * of both atoms of Qneutral * <i|rho_shell|j> (ontop left + right) for
 * i != j; into the self block sum over every neighbor j of the atom case
 * <i|rho_shell(j)|i> rotated with (in1, in1), rho_bond taking only the self
 * pair's term.  The weighted (shell-level) densities follow the same
 * pattern without rotations. */
int or_assemble_rho_2c(or_sys *s, double *rho_in, double *rho_bond, double *wrho_in, double *wrho_bond) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK;
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
  for (int i = 0; i < N; i++) {
    double r1[3], r2[3], z, eps[9], mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, ni = fd->sp[in1].nssh, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j], nnu = fd->sp[in2].norb_max;
      int nj = fd->sp[in2].nssh;
      long long o = s->blk_off[p];
      for (int k = 0; k < nmu * nnu; k++) rho_in[o + k] = 0.0, rho_bond[o + k] = 0.0;
      for (int k = 0; k < WSH; k++) wrho_in[WSH * p + k] = 0.0, wrho_bond[WSH * p + k] = 0.0;
      if (i == j && s->neigh_b[p] == 0) continue;
      pair_frame(s, i, p, r1, r2, &z, eps);
      for (int isorp = 1; isorp <= ni; isorp++) { /* :189-200 */
        double Q = fd->sp[in1].qn[isorp - 1];
        if ((st = or_getMEs_2c(fd, in1, in2, P_rho_ontopL, isorp, z, nmu, nnu, mm))) { err = st; break; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        for (int k = 0; k < nmu * nnu; k++) rho_in[o + k] = rho_in[o + k] + xm[k] * Q;
        for (int k = 0; k < nmu * nnu; k++) rho_bond[o + k] = rho_bond[o + k] + xm[k] * Q;
      }
      for (int isorp = 1; isorp <= nj; isorp++) { /* :206-217 */
        double Q = fd->sp[in2].qn[isorp - 1];
        if ((st = or_getMEs_2c(fd, in1, in2, P_rho_ontopR, isorp, z, nmu, nnu, mm))) { err = st; break; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        for (int k = 0; k < nmu * nnu; k++) rho_in[o + k] = rho_in[o + k] + xm[k] * Q;
        for (int k = 0; k < nmu * nnu; k++) rho_bond[o + k] = rho_bond[o + k] + xm[k] * Q;
      }
      for (int isorp = 1; isorp <= ni; isorp++) { /* weighted :528-539 */
        double Q = fd->sp[in1].qn[isorp - 1];
        if ((st = or_getMEs_2c(fd, in1, in2, P_rhoS_ontopL, isorp, z, ni, nj, mm))) { err = st; break; }
        for (int k = 0; k < ni * nj; k++) wrho_in[WSH * p + k] = wrho_in[WSH * p + k] + mm[k] * Q;
        for (int k = 0; k < ni * nj; k++) wrho_bond[WSH * p + k] = wrho_bond[WSH * p + k] + mm[k] * Q;
      }
      for (int isorp = 1; isorp <= nj; isorp++) { /* :544-554 */
        double Q = fd->sp[in2].qn[isorp - 1];
        if ((st = or_getMEs_2c(fd, in1, in2, P_rhoS_ontopR, isorp, z, ni, nj, mm))) { err = st; break; }
        for (int k = 0; k < ni * nj; k++) wrho_in[WSH * p + k] = wrho_in[WSH * p + k] + mm[k] * Q;
        for (int k = 0; k < ni * nj; k++) wrho_bond[WSH * p + k] = wrho_bond[WSH * p + k] + mm[k] * Q;
      }
    }
    /* self block: the atom case (:222-276, :560-621) */
    int ps = s->pair_off[i] + s->neigh_self[i];
    long long os = s->blk_off[ps];
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
      int self = (i == j && s->neigh_b[p] == 0);
      pair_frame(s, i, p, r1, r2, &z, eps);
      for (int isorp = 1; isorp <= fd->sp[in2].nssh; isorp++) {
        double Q = fd->sp[in2].qn[isorp - 1];
        if ((st = or_getMEs_2c(fd, in1, in2, P_rho_atom, isorp, z, nmu, nmu, mm))) { err = st; break; }
        or_rotate(fd, in1, in1, eps, nmu, nmu, mm, xm);
        for (int k = 0; k < nmu * nmu; k++) rho_in[os + k] = rho_in[os + k] + xm[k] * Q;
        if (self)
          for (int k = 0; k < nmu * nmu; k++) rho_bond[os + k] = rho_bond[os + k] + xm[k] * Q;
      }
      for (int isorp = 1; isorp <= fd->sp[in2].nssh; isorp++) {
        double Q = fd->sp[in2].qn[isorp - 1];
        if ((st = or_getMEs_2c(fd, in1, in2, P_rhoS_atom, isorp, z, ni, ni, mm))) { err = st; break; }
        for (int k = 0; k < ni * ni; k++) wrho_in[WSH * ps + k] = wrho_in[WSH * ps + k] + mm[k] * Q;
        if (self)
          for (int k = 0; k < ni * ni; k++) wrho_bond[WSH * ps + k] = wrho_bond[WSH * ps + k] + mm[k] * Q;
      }
    }
  }
  return err;
}

/* assemble_rho_3c (:298-403) and assemble_rho_weighted_3c (:645-741):
 * rho_in(iatom, mneigh) += sum over the shells of ialpha of Qneutral *
 * rotate(den3), and the weighted density += Qneutral * denS3 (no rotation).
 * Accumulates onto the 2c values. */
int or_assemble_rho_3c(or_sys *s, double *rho_in, double *wrho_in) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK;
  /* serial over ialpha: the triplets of different ialpha write the same
   * pair blocks */
  for (int ia = 0; ia < N; ia++) {
    double mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
    for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1]; t++) {
      trip_t g;
      trip_frame(s, ia, t, &g);
      int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
      int ni = fd->sp[g.in1].nssh, nj = fd->sp[g.in2].nssh, st;
      int p = s->pair_off[g.iatom] + g.mneigh;
      long long o = s->blk_off[p];
      for (int isorp = 1; isorp <= fd->sp[g.indna].nssh; isorp++) {
        double Q = fd->sp[g.indna].qn[isorp - 1];
        st = or_getMEs_3c(fd, g.in1, g.in2, g.indna, P_rho_3c, isorp, g.x, g.z, nmu, nnu, g.cost, mm);
        if (st) { err = st; break; }
        or_rotate(fd, g.in1, g.in2, g.eps, nmu, nnu, mm, xm);
        for (int k = 0; k < nmu * nnu; k++) rho_in[o + k] = rho_in[o + k] + xm[k] * Q;
      }
      for (int isorp = 1; isorp <= fd->sp[g.indna].nssh; isorp++) {
        double Q = fd->sp[g.indna].qn[isorp - 1];
        st = or_getMEs_3c(fd, g.in1, g.in2, g.indna, P_rhoS_3c, isorp, g.x, g.z, ni, nj, g.cost, mm);
        if (st) { err = st; break; }
        for (int k = 0; k < ni * nj; k++) wrho_in[WSH * p + k] = wrho_in[WSH * p + k] + mm[k] * Q;
      }
    }
  }
  return err;
}

/* orbital imu (0-based) of species sp: its shell, l and m
 * (c.SYSTEM/M_species.f90:1196-1208) */
static void orb_of(const species_t *sp, int imu, int *issh, int *l, int *m) {
  int n = 0;
  for (int a = 0; a < sp->nssh; a++) {
    int w = 2 * sp->lssh[a] + 1;
    if (imu < n + w) { *issh = a; *l = sp->lssh[a]; *m = imu - n - sp->lssh[a]; return; }
    n += w;
  }
  *issh = -1; *l = -1; *m = 0;
}

/* assemble_vxc (M_assemble_vxc_McWEDA_Harris.f90:102-191): vxc = vxc_bond +
 * vxc_SN - vxc_SN_bond, with assemble_vxc_SN (:212-486), the generalized
 * Sankey-Niklewski terms at the weighted densities, and assemble_vxc_bond
 * (:507-640), the one-center V for the self block and the rotated
 * vxc_ontop table otherwise.  The optional outputs take vxc_SN,
 * vxc_SN_bond and vxc_bond. */
int or_assemble_vxc(or_sys *s, const double *S, const double *rho_in, const double *rho_bond,
                    const double *wrho_in, const double *wrho_bond, double *vxc, double *sn, double *snb,
                    double *bond) {
  or_fdata *fd = s->fd;
  int N = s->natoms, err = OK;
  for (int k = 1; k <= fd->nspecies; k++)
    if (!fd->sp[k].have_vxc1c) { seterr("no vxc_1c.%02d.dat", fd->sp[k].nZ); return E_TABLE; }
#pragma omp parallel for schedule(dynamic, 4) num_threads(g_threads) if (g_threads > 1)
  for (int i = 0; i < N; i++) {
    double r1[3], r2[3], z, eps[9], mm[MAXORB * MAXORB], xm[MAXORB * MAXORB];
    double vsn[MAXORB * MAXORB], vsnb[MAXORB * MAXORB], vb[MAXORB * MAXORB];
    double lin[6], lbo[6];
    const species_t *A = &fd->sp[s->imass[i]];
    int in1 = s->imass[i], nmu = A->norb_max, ni = A->nssh, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
      const species_t *B = &fd->sp[in2];
      int nnu = B->norb_max;
      long long o = s->blk_off[p];
      const double *Wi = wrho_in + WSH * p, *Wb = wrho_bond + WSH * p;
      for (int k = 0; k < nmu * nnu; k++) vsn[k] = 0.0, vsnb[k] = 0.0, vb[k] = 0.0;
      if (!(i == j && s->neigh_b[p] == 0)) {
        /* off-site SN (:286-357) */
        int n1 = 0;
        for (int a = 0; a < ni; a++) {
          int l1 = A->lssh[a];
          n1 = n1 + l1 + 1;
          int n2 = 0;
          for (int b = 0; b < B->nssh; b++) {
            int l2 = B->lssh[b];
            n2 = n2 + l2 + 1;
            double wi = Wi[a + ni * b], wb = Wb[a + ni * b];
            or_lda_ceperley_alder(wi, lin);
            or_lda_ceperley_alder(wb, lbo);
            for (int m1 = -l1; m1 <= l1; m1++)
              for (int m2 = -l2; m2 <= l2; m2++) {
                int imu = n1 + m1 - 1, inu = n2 + m2 - 1, q = imu + nmu * inu;
                double ov = S[o + q], ri = rho_in[o + q], rb = rho_bond[o + q];
                vsn[q] = lin[1] * ov + lin[4] * (ri - wi * ov);
                vsnb[q] = lbo[1] * ov + lbo[4] * (rb - wb * ov);
              }
            n2 = n2 + l2;
          }
          n1 = n1 + l1;
        }
        /* vxc_bond ontop (:612-627) */
        pair_frame(s, i, p, r1, r2, &z, eps);
        if ((st = or_getMEs_2c(fd, in1, in2, P_vxc_ontop, 0, z, nmu, nnu, mm))) { err = st; continue; }
        or_rotate(fd, in1, in2, eps, nmu, nnu, mm, xm);
        for (int k = 0; k < nmu * nnu; k++) vb[k] = xm[k];
      } else {
        /* on-site SN (:365-480) */
        int n1 = 0;
        for (int a = 0; a < ni; a++) {
          int l1 = A->lssh[a];
          n1 = n1 + l1 + 1;
          double wi = Wi[a + ni * a], wb = Wb[a + ni * a];
          or_lda_ceperley_alder(wi, lin);
          or_lda_ceperley_alder(wb, lbo);
          for (int m1 = -l1; m1 <= l1; m1++) {
            int imu = n1 + m1 - 1, q = imu + nmu * imu;
            vsn[q] = lin[1] + lin[4] * (rho_in[o + q] - wi);
            vsnb[q] = lbo[1] + lbo[4] * (rho_bond[o + q] - wb);
          }
          int n2 = 0;
          for (int b = 0; b < ni; b++) {
            int l2 = A->lssh[b];
            n2 = n2 + l2 + 1;
            double wi2 = Wi[a + ni * b], wb2 = Wb[a + ni * b];
            or_lda_ceperley_alder(wi2, lin);
            or_lda_ceperley_alder(wb2, lbo);
            for (int m1 = -l1; m1 <= l1; m1++)
              for (int m2 = -l2; m2 <= l2; m2++) {
                int imu = n1 + m1 - 1, inu = n2 + m2 - 1, q = imu + nmu * inu;
                if (imu != inu) {
                  vsn[q] = lin[4] * rho_in[o + q];
                  vsnb[q] = lbo[4] * rho_bond[o + q];
                }
              }
            n2 = n2 + l2;
          }
          n1 = n1 + l1;
        }
        /* vxc_bond on-site: V(issh, jssh) where l and m agree (:590-605) */
        for (int inu = 0; inu < nmu; inu++)
          for (int imu = 0; imu < nmu; imu++) {
            int sa, la, ma, sb, lb, mb;
            orb_of(A, imu, &sa, &la, &ma);
            orb_of(A, inu, &sb, &lb, &mb);
            if (la == lb && ma == mb) vb[imu + nmu * inu] = A->vxc1c_V[sa * MAXSH + sb];
          }
      }
      for (int k = 0; k < nmu * nnu; k++) vxc[o + k] = vb[k] + vsn[k] - vsnb[k];
      if (sn) for (int k = 0; k < nmu * nnu; k++) sn[o + k] = vsn[k];
      if (snb) for (int k = 0; k < nmu * nnu; k++) snb[o + k] = vsnb[k];
      if (bond) for (int k = 0; k < nmu * nnu; k++) bond[o + k] = vb[k];
    }
  }
  return err;
}

/* ------------------------------------------------------------------------ */
/* McWEDA force pass (Harris): Dassemble_vxc                                 */
/* (k.DASSEMBLERS/M_Dassemble_vxc_McWEDA_Harris.f90:102-810, with            */
/* Dassemble_rho_2c / Dassemble_rho_weighted_2c of                           */
/* k.DASSEMBLERS/M_Dassemble_rho_McWEDA_Harris.f90:96-710 and                */
/* Dassemble_vxc_3c of k.DASSEMBLERS/M_Dassemble_vxc_3c_McWEDA_Harris.f90).  */
/* Inputs: the density matrix, the overlap S and its Dblocks dS, and the     */
/* value pass's rho_in, rho_bond and weighted densities.  Outputs: the pair  */
/* forces vxc_off_site(3, p) and vxc_on_site(3, p) and the three-center     */
/* forces f3xca/b/c (3 N, overwritten).                                      */
/* ------------------------------------------------------------------------ */

/* derivative of a 2c density interaction summed over the shells of the
 * atom isp_q with Qneutral weights, rotated as (in1, in3): out(3, nmu, nnu) */
static int d_rho_sum(or_fdata *fd, int in1, int in2, int in3, int iint, int qsp, double z, const double *eps,
                     const double *deps, const double *eta, int nmu, int nnu, int rotate_it, double *out) {
  double mm[MAXORB * MAXORB], dm[MAXORB * MAXORB], vdm[3 * MAXORB * MAXORB], vdx[3 * MAXORB * MAXORB];
  for (int k = 0; k < 3 * nmu * nnu; k++) out[k] = 0.0, vdm[k] = 0.0;
  for (int isorp = 1; isorp <= fd->sp[qsp].nssh; isorp++) {
    double Q = fd->sp[qsp].qn[isorp - 1];
    int st = or_getDMEs_2c(fd, in1, in2, iint, isorp, z, nmu, nnu, mm, dm);
    if (st) return st;
    for (int inu = 0; inu < nnu; inu++)
      for (int imu = 0; imu < nmu; imu++)
        if (z > 1.0e-3)
          for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
    if (rotate_it) {
      drotate(fd, in1, in3, eps, deps, nmu, nnu, mm, vdm, vdx);
      for (int k = 0; k < 3 * nmu * nnu; k++) out[k] = out[k] + vdx[k] * Q;
    } else {
      for (int k = 0; k < 3 * nmu * nnu; k++) out[k] = out[k] + vdm[k] * Q;
    }
  }
  return OK;
}

int or_dassemble_vxc(or_sys *s, const double *rho, const double *S, const double *dS, const double *rho_in,
                     const double *rho_bond, const double *wrho_in, const double *wrho_bond, double *off_site,
                     double *on_site, double *f3xca, double *f3xcb, double *f3xcc) {
  or_fdata *fd = s->fd;
  int N = s->natoms, P = s->npairs, err = OK;
  int mo = 1;
  for (int k = 1; k <= fd->nspecies; k++) if (fd->sp[k].norb_max > mo) mo = fd->sp[k].norb_max;
  size_t sa = (size_t)3 * mo * mo;
  /* Dassemble_rho_2c: ontop Dblocko (blk layout, 3 per element; rho_in and
   * rho_bond share it) and the atom case Dblock of each pair (3 nmu nmu) */
  double *drho_o = (double *)calloc((size_t)3 * s->nblock + 1, sizeof(double));
  double *drho_a = (double *)calloc(sa * P + 1, sizeof(double));
  /* Dassemble_rho_weighted_2c: ontop Dblocko and atom Dblock, 3 x 9 per pair */
  double *dw_o = (double *)calloc((size_t)27 * P + 1, sizeof(double));
  double *dw_a = (double *)calloc((size_t)27 * P + 1, sizeof(double));
  for (int i = 0; i < N && !err; i++) {
    double r1[3], r2[3], z, eps[9], deps[27], eta[3], tmp[3 * MAXORB * MAXORB];
    int in1 = s->imass[i], nmu = fd->sp[in1].norb_max, ni = fd->sp[in1].nssh, st;
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
      int nnu = fd->sp[in2].norb_max, nj = fd->sp[in2].nssh;
      if (i == j && s->neigh_b[p] == 0) continue;
      pair_frame(s, i, p, r1, r2, &z, eps);
      or_depsilon_2c(r1, r2, z, eps, deps);
      for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
      long long o = s->blk_off[p];
      /* :141-196 ontop left + right */
      if ((st = d_rho_sum(fd, in1, in2, in2, P_rho_ontopL, in1, z, eps, deps, eta, nmu, nnu, 1, tmp))) { err = st; break; }
      for (int k = 0; k < 3 * nmu * nnu; k++) drho_o[3 * o + k] = drho_o[3 * o + k] + tmp[k];
      if ((st = d_rho_sum(fd, in1, in2, in2, P_rho_ontopR, in2, z, eps, deps, eta, nmu, nnu, 1, tmp))) { err = st; break; }
      for (int k = 0; k < 3 * nmu * nnu; k++) drho_o[3 * o + k] = drho_o[3 * o + k] + tmp[k];
      /* :245-281 atom case of this neighbor */
      if ((st = d_rho_sum(fd, in1, in2, in1, P_rho_atom, in2, z, eps, deps, eta, nmu, nmu, 1, tmp))) { err = st; break; }
      memcpy(drho_a + sa * p, tmp, sizeof(double) * 3 * nmu * nmu);
      /* weighted :505-551 and :610-636, no rotations */
      if ((st = d_rho_sum(fd, in1, in2, in2, P_rhoS_ontopL, in1, z, eps, deps, eta, ni, nj, 0, tmp))) { err = st; break; }
      for (int k = 0; k < 3 * ni * nj; k++) dw_o[27 * p + k] = dw_o[27 * p + k] + tmp[k];
      if ((st = d_rho_sum(fd, in1, in2, in2, P_rhoS_ontopR, in2, z, eps, deps, eta, ni, nj, 0, tmp))) { err = st; break; }
      for (int k = 0; k < 3 * ni * nj; k++) dw_o[27 * p + k] = dw_o[27 * p + k] + tmp[k];
      if ((st = d_rho_sum(fd, in1, in2, in1, P_rhoS_atom, in2, z, eps, deps, eta, ni, ni, 0, tmp))) { err = st; break; }
      memcpy(dw_a + 27 * p, tmp, sizeof(double) * 3 * ni * ni);
    }
  }
  for (int k = 0; k < 3 * P; k++) off_site[k] = 0.0, on_site[k] = 0.0;
  /* Dassemble_vxc_SN (:203-616) and Dassemble_vxc_bond (:638-810) */
  for (int i = 0; i < N && !err; i++) {
    const species_t *A = &fd->sp[s->imass[i]];
    int in1 = s->imass[i], nmu = A->norb_max, ni = A->nssh, st;
    int ps = s->pair_off[i] + s->neigh_self[i];
    long long os = s->blk_off[ps];
    double lin[6], lbo[6];
    for (int in = 0; in < s->neighn[i]; in++) {
      int p = s->pair_off[i] + in, j = s->neigh_j[p], in2 = s->imass[j];
      const species_t *B = &fd->sp[in2];
      int nnu = B->norb_max;
      long long o = s->blk_off[p];
      double *fo = off_site + 3 * (size_t)p, *fn = on_site + 3 * (size_t)p;
      if (i == j && s->neigh_b[p] == 0) continue;
      /* off-site SN (:289-356) */
      int n1 = 0;
      for (int a = 0; a < ni; a++) {
        int l1 = A->lssh[a];
        n1 = n1 + l1 + 1;
        int n2 = 0;
        for (int b = 0; b < B->nssh; b++) {
          int l2 = B->lssh[b];
          n2 = n2 + l2 + 1;
          double wi = wrho_in[WSH * p + a + ni * b], wb = wrho_bond[WSH * p + a + ni * b];
          const double *dwi = dw_o + 27 * (size_t)p + 3 * (a + ni * b), *dwb = dwi;
          or_lda_ceperley_alder(wi, lin);
          or_lda_ceperley_alder(wb, lbo);
          for (int m1 = -l1; m1 <= l1; m1++)
            for (int m2 = -l2; m2 <= l2; m2++) {
              int imu = n1 + m1 - 1, inu = n2 + m2 - 1, q = imu + nmu * inu;
              double ov = S[o + q], ri = rho_in[o + q], rb = rho_bond[o + q], r = rho[o + q];
              const double *dov = dS + 3 * (o + q), *dri = drho_o + 3 * (o + q), *drb = dri;
              for (int c = 0; c < 3; c++) {
                fo[c] = fo[c] - r * (dov[c] * (lin[1] - lin[4] * wi) + dwi[c] * lin[5] * (ri - wi * ov) + lin[4] * dri[c]);
                fo[c] = fo[c] + r * (dov[c] * (lbo[1] - lbo[4] * wb) + dwb[c] * lbo[5] * (rb - wb * ov) + lbo[4] * drb[c]);
              }
            }
          n2 = n2 + l2;
        }
        n1 = n1 + l1;
      }
      /* on-site SN for this neighbor (:360-606) */
      n1 = 0;
      for (int a = 0; a < ni; a++) {
        int l1 = A->lssh[a];
        n1 = n1 + l1 + 1;
        {
          double wi = wrho_in[WSH * ps + a + ni * a], wb = wrho_bond[WSH * ps + a + ni * a];
          /* Dblocko of the self pair: never assembled, zero */
          const double *dwi = dw_o + 27 * (size_t)ps + 3 * (a + ni * a), *dwb = dwi;
          or_lda_ceperley_alder(wi, lin);
          or_lda_ceperley_alder(wb, lbo);
          for (int m1 = -l1; m1 <= l1; m1++) {
            int imu = n1 + m1 - 1, q = imu + nmu * imu;
            double pri = rho_in[os + q], prb = rho_bond[os + q], r = rho[os + q];
            const double *dri = drho_a + sa * p + 3 * q;
            for (int c = 0; c < 3; c++) {
              fn[c] = fn[c] - r * (lin[4] * dri[c] + dwi[c] * lin[5] * (pri - wi));
              fn[c] = fn[c] + r * (lbo[4] * dwb[c] + dwb[c] * lbo[5] * (prb - wb));
            }
          }
        }
        int n2 = 0;
        for (int b = 0; b < ni; b++) {
          int l2 = A->lssh[b];
          n2 = n2 + l2 + 1;
          double wi = wrho_in[WSH * ps + a + ni * b], wb = wrho_bond[WSH * ps + a + ni * b];
          const double *dwi = dw_a + 27 * (size_t)p + 3 * (a + ni * b), *dwb = dwi;
          or_lda_ceperley_alder(wi, lin);
          or_lda_ceperley_alder(wb, lbo);
          for (int m1 = -l1; m1 <= l1; m1++)
            for (int m2 = -l2; m2 <= l2; m2++) {
              int imu = n1 + m1 - 1, inu = n2 + m2 - 1, q = imu + nmu * inu;
              if (imu == inu) continue;
              double pri = rho_in[os + q], prb = rho_bond[os + q], r = rho[os + q];
              const double *dri = drho_a + sa * p + 3 * q, *drb = dri;
              for (int c = 0; c < 3; c++) {
                fn[c] = fn[c] - r * (dwi[c] * lin[5] * pri + lin[4] * dri[c]);
                fn[c] = fn[c] + r * (dwb[c] * lbo[5] * prb + lbo[4] * drb[c]);
              }
            }
          n2 = n2 + l2;
        }
        n1 = n1 + l1;
      }
      /* Dassemble_vxc_bond (:735-790) */
      {
        double r1[3], r2[3], z, eps[9], deps[27], eta[3], mm[MAXORB * MAXORB], dm[MAXORB * MAXORB];
        double vdm[3 * MAXORB * MAXORB], vdx[3 * MAXORB * MAXORB];
        pair_frame(s, i, p, r1, r2, &z, eps);
        or_depsilon_2c(r1, r2, z, eps, deps);
        for (int k = 0; k < 3; k++) eta[k] = E2(eps, k, 2);
        for (int k = 0; k < 3 * nmu * nnu; k++) vdm[k] = 0.0;
        if ((st = or_getDMEs_2c(fd, in1, in2, P_vxc_ontop, 0, z, nmu, nnu, mm, dm))) { err = st; break; }
        for (int inu = 0; inu < nnu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            if (z > 1.0e-3)
              for (int c = 0; c < 3; c++) vdm[c + 3 * (imu + nmu * inu)] = -eta[c] * dm[imu + nmu * inu];
        drotate(fd, in1, in2, eps, deps, nmu, nnu, mm, vdm, vdx);
        for (int inu = 0; inu < nnu; inu++)
          for (int imu = 0; imu < nmu; imu++)
            for (int c = 0; c < 3; c++)
              fo[c] = fo[c] - rho[o + imu + nmu * inu] * vdx[c + 3 * (imu + nmu * inu)];
      }
    }
  }
  /* Dassemble_vxc_3c (M_Dassemble_vxc_3c_McWEDA_Harris.f90:97-514) */
  for (int k = 0; k < 3 * N; k++) f3xca[k] = f3xcb[k] = f3xcc[k] = 0.0;
  for (int ia = 0; ia < N && !err; ia++) {
    double mm[MAXORB * MAXORB], dpm[MAXORB * MAXORB], dxm[MAXORB * MAXORB], dym[MAXORB * MAXORB];
    double Ma[3 * MAXORB * MAXORB], Mb[3 * MAXORB * MAXORB], Xa[3 * MAXORB * MAXORB], Xb[3 * MAXORB * MAXORB];
    double rxa[3 * MAXORB * MAXORB], rxb[3 * MAXORB * MAXORB], rsa[27], rsb[27];
    double depsA[27], depsB[27], amt[3], bmt[3], lin[6];
    for (int t = s->trip_off[ia]; t < s->trip_off[ia + 1] && !err; t++) {
      trip_t g;
      trip_frame(s, ia, t, &g);
      int nmu = fd->sp[g.in1].norb_max, nnu = fd->sp[g.in2].norb_max;
      int ni = fd->sp[g.in1].nssh, nj = fd->sp[g.in2].nssh, nk = fd->sp[g.indna].nssh;
      int p = s->pair_off[g.iatom] + g.mneigh;
      long long o = s->blk_off[p];
      or_depsilon_3c(g.r1, g.r2, g.r21, g.z, g.rna, g.rnabc, g.eps, depsA, depsB);
      for (int k = 0; k < 3 * nmu * nnu; k++) rxa[k] = rxb[k] = 0.0;
      for (int k = 0; k < 27; k++) rsa[k] = rsb[k] = 0.0;
      for (int isorp = 1; isorp <= nk; isorp++) { /* :262-310 */
        double Q = fd->sp[g.indna].qn[isorp - 1];
        int st = or_getDMEs_3c(fd, g.in1, g.in2, g.indna, P_rho_3c, isorp, g.x, g.z, nmu, nnu, g.cost, mm, dpm, dxm,
                               dym);
        if (st) { err = st; break; }
        if (g.x > 1.0e-5)
          for (int k = 0; k < 3; k++) amt[k] = (g.sighat[k] - g.cost * g.rhat[k]) / g.x;
        else
          amt[0] = amt[1] = amt[2] = 0.0;
        for (int k = 0; k < 3; k++) bmt[k] = (g.cost * g.sighat[k] - g.rhat[k]) / g.z;
        for (int k = 0; k < 3 * nmu * nnu; k++) Ma[k] = Mb[k] = 0.0;
        cell3c *c = get_cell3c(fd, g.in1, g.in2, g.indna, P_rho_3c, isorp, 1);
        for (int m = 0; m < c->nME; m++) {
          int k = (c->mu[m] - 1) + nmu * (c->nu[m] - 1);
          for (int q = 0; q < 3; q++) Ma[q + 3 * k] = g.rhat[q] * dxm[k] + amt[q] * dpm[k];
          for (int q = 0; q < 3; q++) Mb[q + 3 * k] = -g.sighat[q] * dym[k] + bmt[q] * dpm[k] - Ma[q + 3 * k] / 2.0;
        }
        drotate(fd, g.in1, g.in2, g.eps, depsA, nmu, nnu, mm, Ma, Xa);
        drotate(fd, g.in1, g.in2, g.eps, depsB, nmu, nnu, mm, Mb, Xb);
        for (int k = 0; k < 3 * nmu * nnu; k++) rxa[k] = rxa[k] + Xa[k] * Q, rxb[k] = rxb[k] + Xb[k] * Q;
      }
      if (err) break;
      for (int isorp = 1; isorp <= nk; isorp++) { /* :330-368 */
        double Q = fd->sp[g.indna].qn[isorp - 1];
        int st = or_getDMEs_3c(fd, g.in1, g.in2, g.indna, P_rhoS_3c, isorp, g.x, g.z, ni, nj, g.cost, mm, dpm, dxm,
                               dym);
        if (st) { err = st; break; }
        for (int a = 0; a < ni; a++)
          for (int b = 0; b < nj; b++) {
            int k = a + ni * b;
            for (int q = 0; q < 3; q++) {
              double va = g.rhat[q] * dxm[k] + amt[q] * dpm[k];
              double bq = (g.cost * g.sighat[q] - g.rhat[q]) / g.z;
              double vb = -g.sighat[q] * dym[k] + bq * dpm[k] - va / 2.0;
              rsa[q + 3 * k] = rsa[q + 3 * k] + va * Q;
              rsb[q + 3 * k] = rsb[q + 3 * k] + vb * Q;
            }
          }
      }
      if (err) break;
      const species_t *A = &fd->sp[g.in1], *B = &fd->sp[g.in2];
      int n1 = 0;
      for (int a = 0; a < ni; a++) { /* :371-402 */
        int l1 = A->lssh[a];
        n1 = n1 + l1 + 1;
        int n2 = 0;
        for (int b = 0; b < nj; b++) {
          int l2 = B->lssh[b];
          n2 = n2 + l2 + 1;
          double w = wrho_in[WSH * p + a + ni * b];
          or_lda_ceperley_alder(w, lin);
          const double *pa_ = rsa + 3 * (a + ni * b), *pb_ = rsb + 3 * (a + ni * b);
          for (int m1 = -l1; m1 <= l1; m1++)
            for (int m2 = -l2; m2 <= l2; m2++) {
              int imu = n1 + m1 - 1, inu = n2 + m2 - 1, q = imu + nmu * inu;
              double dev = rho_in[o + q] - w * S[o + q], r = rho[o + q];
              for (int c = 0; c < 3; c++) {
                double mxa = lin[4] * rxa[c + 3 * q] + pa_[c] * lin[5] * dev;
                double mxb = lin[4] * rxb[c + 3 * q] + pb_[c] * lin[5] * dev;
                double mxc = -mxa - mxb;
                f3xca[3 * ia + c] = f3xca[3 * ia + c] - r * mxa;
                f3xcb[3 * g.iatom + c] = f3xcb[3 * g.iatom + c] - r * mxb;
                f3xcc[3 * g.jatom + c] = f3xcc[3 * g.jatom + c] - r * mxc;
              }
            }
          n2 = n2 + l2;
        }
        n1 = n1 + l1;
      }
    }
  }
  free(drho_o); free(drho_a); free(dw_o); free(dw_a);
  return err;
}
