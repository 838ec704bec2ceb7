// Host-side declarations shared by the C-ABI layer and the mesh preparation.
#pragma once
#include "bem_common.h"
#include "../../include/mfbem.h"

#include <string>
#include <vector>

namespace mfb {

const GLTables& host_gauss_tables();
QsCurves qs_curves(double relative_error);
// fbem_qs_phijac_ngp_2d of a quad8 element (host_prep.cpp)
int host_phijac_ngp_q8(const double* x, double error_height);

// thread-local error string behind mfbem_last_error()
void set_error(const std::string& s);
int fail(int code, const std::string& s);

}  // namespace mfb

// ---------------------------------------------------------------------------
// Caller-side mesh preparation (the role of MultiFEBE's Fortran host: build_data*,
// assign_default_bem_formulation, build_auxiliary_variables_*). It turns an input
// deck into the arrays of an mfbem_mesh_desc. Exported for the Python harness.
// ---------------------------------------------------------------------------
extern "C" {
typedef struct mfbem_prep mfbem_prep;
/* deck: coordinates [nn][3], connectivity [ne][8] (0-based), ctype [nn][3],
   cvalue [nn][3][2]; settings as in mfbem_mesh_desc. */
mfbem_prep* mfbem_prep_create(int32_t nn, const double* X, int32_t ne, const int32_t* conn, const int32_t* ctype,
                              const double* cvalue, double qsi_relative_error, int32_t qsi_ns_max,
                              int32_t n_precalsets, const int32_t* precalset_gln, double geometric_tolerance);
const mfbem_mesh_desc* mfbem_prep_desc(const mfbem_prep* p);
void mfbem_prep_free(mfbem_prep* p);
/* diagnostic copies: dof [nn][3] 0-based (row-1); node order [nn] */
void mfbem_prep_dof(const mfbem_prep* p, int32_t* dof, int32_t* order);
/* BEM formulation per node (0 SBIE, 1 'hbie', 2 'dual_bm_same', 3 'dual_bm_mixed'), Burton &
   Miller alpha and HBIE point offset delta per node (NULL: 1 and 0.22540333);
   mfbem_prep_dual then returns the descriptor for mfbem_mesh_upload_dual
   (NULL before). */
int mfbem_prep_set_formulation(mfbem_prep* p, const int32_t* form, const double* alpha, const double* delta);
/* crack-like boundary: crack_el [ne] 0/1, face 2 conditions ctype2 [nn][3],
   cvalue2 [nn][3][2]; renumbers the DOF (mfbem_prep_desc's n_dof, row, col)
   and makes the dual descriptor. -1: a crack node in an ordinary element,
   -2: ctype2 out of range. */
int mfbem_prep_set_crack(mfbem_prep* p, const int32_t* crack_el, const int32_t* ctype2, const double* cvalue2);
/* face 2's DOF [nn][3] (0-based, -1 off crack-like boundaries) */
void mfbem_prep_dof2(const mfbem_prep* p, int32_t* dof2);
const mfbem_dual_desc* mfbem_prep_dual(const mfbem_prep* p);
}
