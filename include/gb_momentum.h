/*
 * gb_momentum.h -- C-ABI of the device-resident GOLDSTEIN momentum step.
 *
 * Replaces the momentum part of step_goldstein (src/goldstein/goldstein.f90:198-233): wind
 * (:3685-3714), jbar (:3217-3315), ubarsolv (:3500-3565), the island path integrals
 * (goldstein_lib.f90:186-241) with matmult (:3470-3492) and the island corrections of ub and
 * psi (:209-229), and velc (:3568-3679).  It reads the density of a gb_go handle and writes
 * that handle's velocities, so the ocean step (momentum, then tstepo) runs without host copies
 * of rho or u.  With the split-precision form the density is first formed from the current
 * state, and the transfer coefficients are rebuilt on the device from the new velocities (the
 * handle's first velocity field must come from gb_go_set_velocity).
 *
 * The initialisation of the reference (invert :3138-3204, the unit-source solves and island
 * integrals and matinv_gold of :1788-1814) runs on the host at gb_mo_create.  The banded
 * streamfunction solve of ubarsolv is a serial chain (each back-substitution row is a
 * left-to-right sum ending in the row just solved), so on the device the streamfunction is
 * the product of the explicit inverse of the reference's matrix (built at create from the
 * reference's LU factors, one unit column at a time) and the right-hand side.  psi, ub and u
 * then agree with the reference's to a relative 1e-9 (the tests' tolerance), not bit for bit;
 * everything else follows the reference's operation order.  Grids up to GB_MO_MAX_PSI
 * streamfunction points (maxi*(maxj+1)) use the inverse (8*(maxi*(maxj+1))^2 bytes).  Larger
 * grids (up to GB_MO_MAX_PSI_BT points, rows of at most GB_MO_MAX_ROW) solve the same matrix in
 * its block-tridiagonal form -- one block per row j of psi points, coupled to rows j-1 and j+1
 * through diagonal blocks -- with the inverse Schur complements of its block LU factored at
 * create (8*maxi^2*(maxj+1) bytes on the device, e.g. 188 MB for 360x180) and, per step, one
 * matrix-vector product per block row forward and one backward; the same 1e-9 tolerance.
 *
 * Layouts are the reference's, column-major, with their Fortran lower bounds: e.g.
 * rh(3, 0:maxi+1, 0:maxj+1) at (l-1) + 3*(i + (maxi+2)*j); u(3, 0:maxi, 0:maxj, 1:maxk);
 * ub(2, 0:maxi+1, 0:maxj); psi(0:maxi, 0:maxj); arrays of j with bounds (0:maxj) start at j = 0,
 * (1:maxj-1) at j = 1, rds2 (2:maxj-1) at j = 2.  Return codes are those of gb_goldstein.h.
 */
#ifndef GB_MOMENTUM_H
#define GB_MOMENTUM_H

#include "gb_goldstein.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_mo gb_mo;

#define GB_MO_MAX_PSI 8192
#define GB_MO_MAX_PSI_BT 1048576
#define GB_MO_MAX_ROW 2048

/* isles: islands (landmasses - 1, goldstein.f90:1505-1518), mpi: path array length (2*(maxi+maxj));
 * solver: 0 = by size (the inverse up to GB_MO_MAX_PSI points, else block-tridiagonal),
 * 1 = block-tridiagonal at any size */
typedef struct {
    int32_t maxi, maxj, maxk, isles, mpi, solver;
} gb_mo_dims;

typedef struct {
    double dphi, rdphi;
    double rel;          /* velocity relaxation (ini_gold_nml) */
} gb_mo_params;

typedef struct {
    const double *s, *c, *sv, *cv, *rc;   /* (0:maxj) */
    const double *rcv, *dsv, *rdsv;       /* (1:maxj-1) */
    const double *ds, *rds;               /* (1:maxj) */
    const double *rds2;                   /* (2:maxj-1) */
    const double *dz, *dza;               /* (1:maxk) */
    const int32_t *k1;                    /* (0:maxi+1, 0:maxj+1) */
    const int32_t *ku;                    /* (2, maxi, maxj) */
    const int32_t *mk;                    /* (maxi+1, maxj) */
    const int32_t *getj;                  /* (maxi, maxj): 0 or 1 */
    const double *rh;                     /* (3, 0:maxi+1, 0:maxj+1) */
    const double *drag;                   /* (2, maxi+1, maxj) */
    const double *rtv, *rtv3;             /* (maxi, maxj) */
    const double *psiles;                 /* landmass labels at the psi points, as gbold after
                                             the .psiles read: (maxi*(maxj+1)), index i+j*maxi-1 */
    const int32_t *npi;                   /* (isles) */
    const int32_t *lpisl, *ipisl, *jpisl; /* (mpi, isles) */
} gb_mo_grid;

int gb_mo_create(const gb_mo_dims *dims, const gb_mo_params *params, const gb_mo_grid *grid, int device, gb_mo **out);
void gb_mo_destroy(gb_mo *h);
/* the wind stress of the step: tau, dztau, dztav, each (2, maxi, maxj) (goldstein.f90:102-107) */
int gb_mo_set_wind(gb_mo *h, const double *tau, const double *dztau, const double *dztav);
/* u and u1 (3, 0:maxi, 0:maxj, maxk), e.g. from a restart; both start at 0 otherwise */
int gb_mo_upload_velocity(gb_mo *h, const double *u, const double *u1);
/* One momentum step on `ocean`'s density (a gb_go handle of the same grid, either form); the new
   velocities become `ocean`'s velocities for its next gb_go_tstepo. */
int gb_mo_step(gb_mo *h, gb_go_handle *ocean);
/* u, u1 (3, 0:maxi, 0:maxj, maxk), ub (2, 0:maxi+1, 0:maxj), psi (0:maxi, 0:maxj); any may be NULL */
int gb_mo_download(gb_mo *h, double *u, double *u1, double *ub, double *psi);
const char *gb_mo_last_error(const gb_mo *h);

#ifdef __cplusplus
}
#endif

#endif
