/*
 * fb_oracle.h -- CPU oracle for the FIREBALL Harris matrix-element assembly.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran routines on the assembly path.  Only the test suite, the smoke check
 * and the CPU-baseline leg of the benchmark load it, and only as the checker
 * or the timed CPU baseline; the GPU library never links or calls it.
 *
 * Parity status: UNPINNED.  The reference ships no tests, golden vectors or
 * Fdata, and its Fortran cannot be compiled where this project is built (no
 * Fortran compiler), so this restatement is checked by property tests
 * (polynomial exactness of the interpolators, Hermiticity through neigh_back,
 * rotation invariance, finite differences of the derivative paths) rather
 * than against outputs of the reference itself.
 *
 * Layout conventions (shared with the GPU library):
 *   pairs   p = pair_off[i] + ineigh, CSR by atom i, reference order
 *   blocks  block p at blk_off[p], column-major norb_i x norb_j (Fortran
 *           block(mu,nu) of T_assemble_block, a.GLOBAL/M_assemble_blocks.f90:44)
 *   Dblocks 3 * blk_off[p], layout Dblock(3,mu,nu) column-major
 *   per-pair 3-vectors (vna_ontop, vna_atom) at 3*p
 *   per-atom 3-vectors at 3*i
 */
#ifndef FB_ORACLE_H
#define FB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_fdata or_fdata;
typedef struct or_sys or_sys;

/* read_info + read_Fdata_2c + read_Fdata_3c.  Returns NULL on failure and
 * writes a message into err. */
or_fdata *or_load_fdata(const char *dir, int nspecies, const int *nZ,
                        char *err, int errlen);
void or_free_fdata(or_fdata *fd);
int or_species_norb(const or_fdata *fd, int ispecies /* 1-based */);

/* structure + make_cells; positions (natoms,3) row-major Angstrom,
 * imass 1-based species, lattice rows a1,a2,a3 */
or_sys *or_create_system(or_fdata *fd, int natoms, const double *ratom,
                         const int *imass, const double *lattice, int icluster);
void or_free_system(or_sys *s);

/* driver_neighbors: find_neigh_max/find_neighbors/find_common_* */
int or_neighbors(or_sys *s);
int or_npairs(const or_sys *s);
int or_ntriplets(const or_sys *s);
long long or_nblock(const or_sys *s);        /* total doubles of one block set */
/* copy out neighbor maps (caller allocates) */
void or_get_pairs(const or_sys *s, int *pair_off, int *neigh_j, int *neigh_b,
                  int *neigh_back, int *neigh_self, long long *blk_off);
void or_get_triplets(const or_sys *s, int *trip_off, int *iatom_j,
                     int *iatom_b, int *jatom_j, int *jatom_b,
                     int *neigh_common);

/* assemblers (j.ASSEMBLERS Harris): outputs are full block sets */
int or_assemble_2c(or_sys *s, double *S, double *T, double *vna_block,
                   double *vna_blocko);
int or_assemble_3c(or_sys *s, double *vna_block);   /* accumulates */

/* derivative assemblers (k.DASSEMBLERS Harris); rho = denmat block set */
int or_dassemble_2c(or_sys *s, const double *rho, double *dS, double *dT,
                    double *vna_ontop, double *vna_atom);
int or_dassemble_3c(or_sys *s, const double *rho, double *f3naa,
                    double *f3nab, double *f3nac);
/* build_forces, assembly terms only: kinetic, vna, f3na, pulay, ftot */
int or_build_forces(or_sys *s, const double *rho, const double *cape,
                    const double *dS, const double *dT,
                    const double *vna_ontop, const double *vna_atom,
                    const double *f3naa, const double *f3nab,
                    const double *f3nac, double *kinetic, double *vna,
                    double *pulay, double *ftot);

/* Bloch sum of one block set into nk dense n x n complex matrices
 * (column-major, re/im interleaved) -- h.SOLVESH/M_kspace_Lowdin.f90 */
int or_bloch(or_sys *s, int nk, const double *kpts, const double *blocks,
             double *out);

/* DOGS (j.ASSEMBLERS/M_assemble_2c_DOGS.f90, M_assemble_3c_DOGS.f90):
 * shell charges dq[i * nssh_max + isorp - 1] = Qin - Qneutral; z-dipole
 * blocks; the charge-weighted vna 2c (fills vb, vbo from the overlap S) and
 * vna 3c (accumulates onto vb from S and dip) */
int or_set_charges(or_sys *s, const double *dq, int nssh_max);
int or_assemble_dipole_z(or_sys *s, double *dip);
int or_assemble_vna_2c_dogs(or_sys *s, const double *S, double *vb,
                            double *vbo);
int or_assemble_vna_3c_dogs(or_sys *s, const double *S, const double *dip,
                            double *vb);
/* Ewald (j.ASSEMBLERS/M_assemble_ewald_DOGS.f90): the N x N long-range
 * Coulomb matrix (row-major), and the ewaldsr / ewaldlr block sets over the
 * neighbor map from the overlap and z-dipole blocks and the atoms' total
 * charges (the sum of the shell charges of or_set_charges) */
int or_assemble_ewald(or_sys *s, double *ewald);
int or_assemble_ewaldsr(or_sys *s, const double *S, const double *dip,
                        double *sr);
int or_assemble_ewaldlr(or_sys *s, const double *ewald, const double *S,
                        const double *dip, double *lr);
/* Ewald force pass (k.DASSEMBLERS/M_Dassemble_ewald_DOGS.f90): dewald
 * ([(i * N + j) * 3 + c], derivative of ewald(i, j) in r_i) and the Ewald
 * energy force; the ewaldsr pair forces (3 per pair) with the three-center
 * terms added into f3naa/b/c; the ewaldlr atom forces.  rho is the density
 * matrix, dS / ddip the overlap and dipole Dblocks */
int or_dassemble_ewald(or_sys *s, double *dewald, double *fewald);
int or_dassemble_ewaldsr(or_sys *s, const double *rho, const double *S,
                         const double *dS, const double *dip,
                         const double *ddip, double *fsr, double *f3naa,
                         double *f3nab, double *f3nac);
int or_dassemble_ewaldlr(or_sys *s, const double *rho, const double *ewald,
                         const double *dewald, const double *S,
                         const double *dS, const double *dip,
                         const double *ddip, double *flr);
/* DOGS force derivatives (k.DASSEMBLERS/M_Dassemble_2c_DOGS.f90,
 * M_Dassemble_3c_DOGS.f90): z-dipole Dblocks; vna ontop / atom pair terms;
 * f3na{a,b,c} (neutral + charged; overwrites) from S, dS, dip, ddip */
int or_dassemble_dipole_z(or_sys *s, double *ddip);
int or_dassemble_vna_2c_dogs(or_sys *s, const double *rho, const double *S,
                             double *vna_ontop, double *vna_atom);
int or_dassemble_vna_3c_dogs(or_sys *s, const double *rho, const double *S,
                             const double *dS, const double *dip,
                             const double *ddip, double *f3naa,
                             double *f3nab, double *f3nac);

/* non-local pseudopotential (vnl): driver_neighbors_PP; sizes (pairs of the
 * PP, PPx, PPp maps, PP common triplets, svnl and vnl block doubles); the
 * maps (0-based; which 0 PP, 1 PPx, 2 PPp); assemble_svnl / vnl_2c /
 * vnl_3c (vnl_3c accumulates); the derivatives and the build_forces vnl
 * terms.  rho_pp: the density over PPp (s%denmat_PP). */
int or_neighbors_pp(or_sys *s);
void or_pp_sizes(const or_sys *s, int *npp, int *nppx, int *nppp, int *ntrip,
                 long long *nsvnl, long long *nvnl);
void or_get_pp(const or_sys *s, int which, int *off, int *jj, int *bb,
               int *self, int *map, int *point);
void or_get_pp_common(const or_sys *s, int *off, int *ci, int *cib, int *cj,
                      int *cjb, int *m, int *m31, int *m32);
int or_assemble_svnl(or_sys *s, double *svnl);
int or_assemble_vnl_2c(or_sys *s, const double *svnl, double *vnl);
int or_assemble_vnl_3c(or_sys *s, const double *svnl, double *vnl);
int or_dassemble_svnl(or_sys *s, double *dsvnl);
int or_dassemble_vnl_2c(or_sys *s, const double *rho_pp, const double *svnl,
                        const double *dsvnl, double *vnl_atom,
                        double *vnl_ontop);
int or_dassemble_vnl_3c(or_sys *s, const double *rho_pp, const double *svnl,
                        const double *dsvnl, double *f3nla, double *f3nlb,
                        double *f3nlc);
int or_build_forces_vnl(or_sys *s, const double *vnl_atom,
                        const double *vnl_ontop, const double *f3nla,
                        const double *f3nlb, const double *f3nlc, double *vnl,
                        double *ftot_add);

/* McWEDA exchange-correlation, Harris (M_assemble_rho_McWEDA_Harris.f90,
 * M_assemble_vxc_McWEDA_Harris.f90): the Ceperley-Alder LDA (out = exc,
 * muxc, dexc, d2exc, dmuxc, d2muxc); the input densities rho_in / rho_bond
 * (orbital blocks) and their shell-level weighted forms (9 doubles per pair,
 * (issh, jssh) at [9 p + issh + nssh_i jssh]), 2c part (overwrites) and 3c
 * part (accumulates onto rho_in and wrho_in); the vxc blocks from the
 * overlap S and those densities (sn, snb, bond optional: vxc_SN,
 * vxc_SN_bond, vxc_bond). */
void or_lda_ceperley_alder(double rh, double *out);
int or_assemble_rho_2c(or_sys *s, double *rho_in, double *rho_bond,
                       double *wrho_in, double *wrho_bond);
int or_assemble_rho_3c(or_sys *s, double *rho_in, double *wrho_in);
int or_assemble_vxc(or_sys *s, const double *S, const double *rho_in,
                    const double *rho_bond, const double *wrho_in,
                    const double *wrho_bond, double *vxc, double *sn,
                    double *snb, double *bond);
/* McWEDA force pass (Dassemble_vxc, k.DASSEMBLERS/M_Dassemble_vxc_McWEDA_Harris.f90,
 * with Dassemble_rho_2c / _weighted_2c and Dassemble_vxc_3c): from the density
 * matrix, S and its Dblocks dS (3 per element) and the value pass's
 * densities; vxc_off_site and vxc_on_site (3 per pair) and f3xca/b/c (3 N) */
int or_dassemble_vxc(or_sys *s, const double *rho, const double *S,
                     const double *dS, const double *rho_in,
                     const double *rho_bond, const double *wrho_in,
                     const double *wrho_bond, double *off_site,
                     double *on_site, double *f3xca, double *f3xcb,
                     double *f3xcc);

/* pointwise interpolators (module M_Fdata_2c / M_Fdata_3c); hmbox etc are
 * norb_mu x norb_nu column-major */
int or_getMEs_2c(or_fdata *fd, int isp, int jsp, int iint, int isub, double x,
                 int norb_mu, int norb_nu, double *hmbox);
int or_getDMEs_2c(or_fdata *fd, int isp, int jsp, int iint, int isub,
                  double x, int norb_mu, int norb_nu, double *hmbox,
                  double *dhmbox);
int or_getMEs_3c(or_fdata *fd, int isp, int jsp, int ksp, int iint, int isub,
                 double x, double y, int norb_mu, int norb_nu, double cost,
                 double *hmbox);
int or_getDMEs_3c(or_fdata *fd, int isp, int jsp, int ksp, int iint, int isub,
                  double x, double y, int norb_mu, int norb_nu, double cost,
                  double *hmbox, double *dphmbox, double *dxhmbox,
                  double *dyhmbox);
void or_epsilon(const double *r1, const double *r2, double *spe);
void or_depsilon_2c(const double *r1, const double *r2, double z,
                    const double *eps, double *deps);
void or_depsilon_3c(const double *r1, const double *r2, const double *r21,
                    double z, const double *ratm, const double *rnabc,
                    const double *eps3, double *dera3, double *der13);
void or_rotate(or_fdata *fd, int in1, int in3, const double *eps, int norb_mu,
               int norb_nu, const double *mmatrix, double *xmatrix);

/* Test switch, off by default: 1 replaces the reference's two forms that are
 * not the derivative of its values -- the (dden*3) of d2dec in
 * lda_ceperley_alder (g.XC_FUNCTIONALS/lda_ceperley_alder.f90:142) and the
 * three-point linear branch of getMEs/getDMEs_Fdata_3c
 * (e.FDATA/M_Fdata_3c.f90:406-410, :684-691), whose x / y derivatives use
 * one scalar gradient for every matrix element -- by exact ones (dden**3,
 * the bicubic everywhere), so finite differences can check the rest of a
 * force restatement. */
void or_set_exact_derivatives(int on);

/* OpenMP thread count for the assemblers (1 = serial reference order) */
void or_set_threads(int n);
const char *or_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
