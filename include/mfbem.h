/*
 * mfbem.h - C-ABI of the GB300 collocation-BEM library (drop-in for the
 * element integration + dense solve path of MultiFEBE 2.0.1).
 *
 * The entry points replace, one to one, the reference routines that fill and
 * solve the dense BEM system:
 *
 *   mfbem_assemble_staela  <- subroutine build_lse_mechanics_bem_staela(kr)
 *                             src/build_lse_mechanics_bem_staela.f90:22 (called from
 *                             src/build_lse_mechanics_static.f90:62)
 *   mfbem_assemble_harela  <- subroutine build_lse_mechanics_bem_harela(kf,kr)
 *                             src/build_lse_mechanics_bem_harela.f90:22 (called from
 *                             src/build_lse_mechanics_harmonic.f90:88)
 *   mfbem_solve_r          <- subroutine solve_lse_r(n_dof,A,ipiv,Aodim,Ao,equed,r,c,n_rhs,b,
 *                             factorize,scaling,condition,refine), src/solve_lse_r.f90:25
 *   mfbem_solve_c          <- subroutine solve_lse_c(...), src/solve_lse_c.f90:25
 *   mfbem_mesh_upload      <- the module state those builders read (problem_variables:
 *                             element(:), node(:), qsi_parameters, precalset_gln,
 *                             src/problem_variables.f90:73-109), snapshotted once per mesh
 *   mfbem_sweep_harela     <- the frequency loop of src/multifebe.f90:107-119
 *                             (build_lse_mechanics_harmonic + solve_lse_c per frequency),
 *                             batched on the device; no reference counterpart as one call
 *
 * Conventions (those of the reference's Fortran globals):
 *   - all indices that name nodes, elements, rows or columns are 1-based;
 *   - matrices are column-major with leading dimension lda >= n_dof;
 *   - complex numbers are interleaved (re, im) doubles, i.e. complex(real64);
 *   - the builders ADD into A and b (the caller zeroes them, as
 *     src/build_lse_mechanics_static.f90:52-53 does), unless MFBEM_OVERWRITE;
 *   - return value 0 on success, > 0 LAPACK-style info (index of the first
 *     zero pivot), < 0 an MFBEM_E* error; mfbem_last_error() describes it.
 *
 * Threading: calls are synchronous, made from one host thread, not re-entrant
 * per handle. A handle owns device memory for one mesh and its work buffers.
 */
#ifndef MFBEM_H
#define MFBEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFBEM_OK 0
#define MFBEM_EARG (-1)        /* invalid argument */
#define MFBEM_ECUDA (-2)       /* CUDA runtime failure / no device */
#define MFBEM_ENOMEM (-3)      /* device allocation failed */
#define MFBEM_ETIMEOUT (-4)    /* a bounded device wait gave up */
#define MFBEM_EGEOMETRY (-5)   /* invalid normals/tangents at a free-term node
                                  (the reference stops: bem_staela3d.f90:296-303) */
#define MFBEM_ENOCONV (-6)     /* iterative refinement did not reach the tolerance */
#define MFBEM_EUNSUPPORTED (-7)

/* flags */
#define MFBEM_DEVICE_PTRS 0x1  /* A, b (and x) are device pointers */
#define MFBEM_OVERWRITE 0x2    /* overwrite A and b instead of adding into them */

/* Mesh snapshot of one BE region with ordinary boundaries of continuous quad8
 * elements, in the layout of the reference's derived types. */
typedef struct mfbem_mesh_desc {
  int32_t n_nodes;
  int32_t n_elements;
  int32_t n_dof;                 /* row-1 after build_auxiliary_variables_* */
  /* element(se): x_gn(3,8), node(8) (1-based), csize, n_phi, bball_centre(3),
     bball_radius, and the reversion flag of its boundary in the region */
  const double* x_gn;            /* [n_elements][8][3] */
  const int32_t* element_node;   /* [n_elements][8] */
  const double* csize;           /* [n_elements] */
  const int32_t* n_phi;          /* [n_elements] */
  const double* bball;           /* [n_elements][4]: centre x,y,z, radius */
  const int32_t* reversion;      /* [n_elements] 0/1, may be NULL (all 0) */
  /* element(se)%n_gn(3,8) and %tbp_gn(3,8): unit normal and forward element
     boundary tangent at each node (free-term inputs) */
  const double* n_gn;            /* [n_elements][8][3] */
  const double* tbp_gn;          /* [n_elements][8][3] */
  /* node(sn): row(3,1), col(6,1) (0 where unused), ctype(3,1), cvalue(3,1,1)
     (complex, the real part is used by the static path), and the SBIE
     formulation (0 nodal SBIE, 1 SBIE with MCA) */
  const int32_t* row;            /* [n_nodes][3] */
  const int32_t* col;            /* [n_nodes][6] */
  const int32_t* ctype;          /* [n_nodes][3]: 0 u known, 1 t known */
  const double* cvalue;          /* [n_nodes][3][2] */
  const int32_t* sbie;           /* [n_nodes] */
  /* element(se)%xi_i_sbie_mca(2,8) and %x_i_sbie_mca(3,8) (read for MCA nodes) */
  const double* xi_i_sbie_mca;   /* [n_elements][8][2] */
  const double* x_i_sbie_mca;    /* [n_elements][8][3] */
  /* settings (src/read_settings.f90): qsi_relative_error, qsi_ns_max,
     precalset_gln(1:n_precalsets), geometric_tolerance */
  double qsi_relative_error;
  int32_t qsi_ns_max;
  int32_t n_precalsets;
  const int32_t* precalset_gln;
  double geometric_tolerance;
} mfbem_mesh_desc;

typedef struct mfbem_handle mfbem_handle;

/* Per-call accounting written by the assemble / sweep entry points. */
typedef struct mfbem_stats {
  int64_t pairs_regular, pairs_adaptive, pairs_singular;
  int64_t points_regular, points_adaptive, points_singular;
  int32_t adaptive_leaves;
  int32_t refinement_iterations; /* sweep: total over frequencies */
  double max_backward_error;     /* sweep: max over frequencies of ||b-Ax||/(||A|| ||x||) */
  double ms_assemble, ms_factor, ms_solve;
  /* device time of the assembly kernels of the last call (CUDA events on the
     library's stream): regular, adaptive, singular pairs and free terms */
  double ms_regular, ms_adaptive, ms_singular, ms_free;
  int64_t kernel_launches;       /* this library's kernels launched by the call */
  int32_t gmres_iterations;      /* mixed: inner GMRES steps of GMRES-based refinement (0: classical only) */
  int32_t refactorizations;      /* mixed: FP32 refactorisations after TF32 factors stalled the refinement */
} mfbem_stats;

/* mesh lifetime */
int mfbem_mesh_upload(const mfbem_mesh_desc* desc, mfbem_handle** out);
int mfbem_mesh_release(mfbem_handle* h);

/* HBIE collocation on the boundary: the node(sn)%hbie / %dual /
   %dual_is_common / %alpha and element(se)%xi_i_hbie / %x_i_hbie / %n_i_hbie
   members the reference sets from the [bem formulation over boundaries]
   section (src/read_bem_formulation_selected_nodes.f90:70-260) and
   src/build_data_at_collocation_points.f90:148-160,368-376, for ordinary
   boundaries of continuous elements. Per node, (hbie, dual, dual_is_common):
     (0, 0, 0)  the SBIE of the mesh descriptor: nodal, or MCA by its sbie flag;
     (1, 0, 0)  'hbie': the HBIE alone, collocated at x_i_hbie in every
                element of the node (h = m, g = l);
     (1, 1, 1)  'dual_bm_same': SBIE and HBIE at the same points x_i_hbie,
                Burton & Miller: h + beta m, g + beta l with beta = alpha in
                the static builder (build_lse_mechanics_bem_staela.f90:835-841)
                and alpha i / c2 in the harmonic one, c2 = sqrt(mu / rho) the
                complex S-wave speed (build_lse_mechanics_bem_harela.f90:1174-1181).
     (1, 1, 0)  'dual_bm_mixed': the node's SBIE at its own point (nodal, or
                MCA by its sbie flag at x_i_sbie_mca) plus beta times the
                HBIE at the points x_i_hbie of its elements, integrated on
                their own (sbie_auto and hbie_auto in both builders,
                src/read_bem_formulation_selected_nodes.f90:243-295). The
                reference's non-common branch keeps a nodal SBIE's h of the
                node's first element for its later ones (the rows it
                assembles are not this weighted sum); the library assembles
                the weighted sum;
     (1, 2, 1)  a node of a crack-like boundary (fbem_dual_boundary,
                src/assign_default_bem_formulation.f90:94-128): the SBIE and
                the HBIE at the same points x_i_hbie, each its own equation.
   Other combinations return MFBEM_EUNSUPPORTED.
   Crack-like boundaries (boundary class cracklike, src/read_boundaries.f90:
   105; dual BEM): crack_el marks their elements (NULL: none), whose nodes
   belong to no ordinary element and carry two faces, face 1 with the
   element normal and face 2 with the reversed one; ctype2 / cvalue2 are
   node(sn)%ctype(k,2) / %cvalue(k,1,2) of face 2. A crack node takes six
   rows r..r+5 in the reference's order: row(k,1) = r + 2(k-1) its SBIE,
   row(k,2) = row(k,1) + 1 its HBIE, face 1's unknown of direction k in
   column row(k,1) (the mesh descriptor's row / col) and face 2's in
   row(k,1) + 1 (src/build_auxiliary_variables_mechanics_static.f90:146-207);
   n_dof = 3 n_nodes + 3 (crack nodes). Face 2 takes -h, g, -m, l of the
   element (src/build_lse_mechanics_bem_staela.f90:883-887); the SBIE
   equation takes 1/2 phi(xi_i) on both faces' u, the HBIE -1/2 phi(xi_i) on
   face 1's t and +1/2 phi(xi_i) on face 2's (staela.f90:195-204,
   build_lse_mechanics_bem_harela.f90:344-360). Internal points of such a
   region: mfbem_internal_points_faces_staela / _harela.
   The HBIE points are classified as hbie_auto does
   (lib/fbem/src/bem_staela3d.f90:4307-4373, 1/r^7 estimate); the element
   holding a point takes the interior (hypersingular) integration
   (bem_staela3d.f90:4918-5353, bem_harela3d.f90:3169-3630); the SBIE part of
   a Burton & Miller point is classified like sbie_auto by the static builder
   and like shbie_auto (bem_harela3d.f90:4888-4957) by the harmonic one. The
   n_i_hbie of an element whose reversion flag is set is reversed on upload.
   A half-space region with HBIE points is MFBEM_EUNSUPPORTED. */
typedef struct mfbem_dual_desc {
  const int32_t* hbie;           /* [n_nodes] */
  const int32_t* dual;           /* [n_nodes] */
  const int32_t* dual_is_common; /* [n_nodes] */
  const double* alpha;           /* [n_nodes] */
  const double* xi_i_hbie;       /* [n_elements][8][2] */
  const double* x_i_hbie;        /* [n_elements][8][3] */
  const double* n_i_hbie;        /* [n_elements][8][3] */
  const int32_t* crack_el;       /* [n_elements] 0/1, may be NULL (no crack-like boundary) */
  const int32_t* ctype2;         /* [n_nodes][3] face 2 (read for crack nodes) */
  const double* cvalue2;         /* [n_nodes][3][2] face 2 */
} mfbem_dual_desc;
int mfbem_mesh_upload_dual(const mfbem_mesh_desc* desc, const mfbem_dual_desc* dual, mfbem_handle** out);

/* Region space (region(kr)%space, %halfspace_n, %halfspace_x, %halfspace_bc
   of src/read_regions.f90:130-200): n = 0 full space (the default), else a
   half-space whose hyperplane x(|n|) = x has the unit normal sign(n) e_|n|,
   with bc = 1 (traction-free surface; bc = 0 is MFBEM_EUNSUPPORTED, as the
   reference stops on it). Both builders then double the free term of
   collocation points on the hyperplane (build_lse_mechanics_bem_staela.f90:502-513,
   build_lse_mechanics_bem_harela.f90:688-697); the static builder adds, for
   n = -3 only (half-space x3 >= x), the complementary kernel of Mindlin's
   solution to every pair (fbem_bem_staela3d_hsc_sbie_auto,
   lib/fbem/src/bem_staela3d.f90:9047-9118), so that the free surface needs no
   elements. The complementary pair lists are built at the next static
   assembly; a node or collocation point outside the half-space, or an element
   holding a collocation point of the surface without lying on it, returns
   MFBEM_EGEOMETRY there (the reference stops). Static internal points of a
   half-space region (n = -3) add the complementary kernels from each point's
   image (fbem_bem_staela3d_hsc_sbie_auto / _hsc_hbie_auto,
   src/calculate_internal_points_mechanics_static.f90:288-310,401-418); a
   point outside the half-space returns MFBEM_EGEOMETRY, one on the free
   surface on an element MFBEM_EUNSUPPORTED (the reference stops). */
int mfbem_set_halfspace(mfbem_handle* h, int32_t n, double x, int32_t bc);

/* build_lse_mechanics_bem_staela: A (n_dof x n_dof, real) and b (n_dof). */
int mfbem_assemble_staela(mfbem_handle* h, double mu, double nu, double* A, int32_t lda, double* b,
                          int32_t flags);

/* build_lse_mechanics_bem_harela for one frequency omega (rad/s): lambda, mu
   and nu complex (region property_c(6), property_c(2), property_c(3)), rho
   real. A and b complex(real64). */
int mfbem_assemble_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                          const double nu[2], double omega, double* A, int32_t lda, double* b, int32_t flags);

/* solve_lse_r / solve_lse_c with LAPACK semantics, on the GPU in FP64, every
   option of the reference:
     scaling    (factorize) ?geequ + ?laqge: A equilibrated in place, r and c
                receive the row / column factors and *equed 'N', 'R', 'C' or
                'B'; (no factorize) equed, r and c from an earlier call are used.
                b is scaled by r before the solve (equed R/B), x by c after
                it (equed C/B). A zero row i / column j of A returns i / n + j.
     factorize  getrf: on return A holds the LU factors and ipiv the 1-based
                pivots, exactly as LAPACK leaves them; 0 reuses them.
     condition  (factorize) ?gecon: reciprocal one-norm condition estimate of
                the (scaled) matrix, read with mfbem_solve_report.
     refine     ?gerfs: at most five refinement steps with the residual of
                the unfactorised matrix; ferr / berr read with
                mfbem_solve_report.
   With condition or refine, aodim must be n and Ao (n x n) receives the
   unfactorised (scaled) matrix when factorize is set; a later call with
   factorize = 0 and refine reads it back, as src/solve_lse_r.f90:70-78,
   199-206 do. A singular matrix returns info > 0 (zero pivot U(info,info)). */
int mfbem_solve_r(int32_t n, double* A, int32_t* ipiv, int32_t aodim, double* Ao, char* equed, double* r,
                  double* c, int32_t n_rhs, double* b, int32_t factorize, int32_t scaling, int32_t condition,
                  int32_t refine);
int mfbem_solve_c(int32_t n, double* A, int32_t* ipiv, int32_t aodim, double* Ao, char* equed, double* r,
                  double* c, int32_t n_rhs, double* b, int32_t factorize, int32_t scaling, int32_t condition,
                  int32_t refine);
/* Internal points: calculate_internal_points_mechanics_bem_staela /
   _harela (src/calculate_internal_points_mechanics_static.f90:188-502,
   src/calculate_internal_points_mechanics_bem_harela.f90:22-505), after the
   solve. From the nodal solution u_nodes, t_nodes [n_nodes][3] (node%value
   (1:3) and (4:6): real for staela, complex for harela), for n_ip points
   x_ip [n_ip][3] inside the region:
     u_ip     [n_ip][3]      displacement (value(1:3, 0))
     sigma_ip [n_ip][3][3]   sigma_ip[ip][kc][il] = stress sigma(il, kc),
                             the traction on the plane of normal e_kc
                             (value(1:3, kc), column-major like the reference)
   with the SBIE kernels for u and the HBIE kernels (d*, s*) for sigma, the
   same classification (precalculated / adaptive rules, 1/r^7 estimate for
   the HBIE). A point at a boundary node (distance < 1e-12 csize of the node's
   first element) returns the node's displacement and zero stress, as the
   reference does; a point on an element away from its nodes returns
   MFBEM_EUNSUPPORTED. Ordinary boundaries; no symmetry planes, body loads or
   incident field. FP64 on the device. */
int mfbem_internal_points_staela(mfbem_handle* h, double mu, double nu, int32_t n_ip, const double* x_ip,
                                 const double* u_nodes, const double* t_nodes, double* u_ip, double* sigma_ip);
int mfbem_internal_points_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                                 double omega, int32_t n_ip, const double* x_ip, const double* u_nodes,
                                 const double* t_nodes, double* u_ip, double* sigma_ip);
/* The same for a region with crack-like boundaries: u2_nodes, t2_nodes
   [n_nodes][3] hold face 2's solution (node%value(:, 2); read for the crack
   nodes), which the reference integrates with the reversed element
   (calculate_internal_points_mechanics_static.f90:320-354,431-465,
   calculate_internal_points_mechanics_bem_harela.f90:343-470). The two
   functions above return MFBEM_EUNSUPPORTED on such a region; a point at a
   crack node (where the faces' values differ) returns MFBEM_EUNSUPPORTED. */
int mfbem_internal_points_faces_staela(mfbem_handle* h, double mu, double nu, int32_t n_ip, const double* x_ip,
                                       const double* u_nodes, const double* t_nodes, const double* u2_nodes,
                                       const double* t2_nodes, double* u_ip, double* sigma_ip);
int mfbem_internal_points_faces_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho,
                                       double omega, int32_t n_ip, const double* x_ip, const double* u_nodes,
                                       const double* t_nodes, const double* u2_nodes, const double* t2_nodes,
                                       double* u_ip, double* sigma_ip);

/* Gmsh *.msh 2.2 ASCII reader, host only: the gmsh branch of
   fbem_mesh%read_from_file (lib/fbem/src/mesh.f90:104-494) with its checks
   ($MeshFormat 2.2, $PhysicalNames as the parts, element parts = first tag,
   known element types, unique positive ids). Entities keep the file's order
   and ids; element nodes are node ids in gmsh order. Returns 0, or -1 with
   the reason in mfbem_msh_error(). counts = parts, nodes, elements,
   element-node entries; names: n_parts x name_len bytes, NUL-padded;
   offsets: [n_elements + 1] into nodes. */
int mfbem_msh_read(const char* path, void** msh);
const char* mfbem_msh_error(void);
int mfbem_msh_sizes(void* msh, int32_t* counts);
int mfbem_msh_parts(void* msh, int32_t* id, int32_t* dim, char* names, int32_t name_len);
int mfbem_msh_nodes(void* msh, int32_t* id, double* x);
int mfbem_msh_elements(void* msh, int32_t* id, int32_t* type, int32_t* part, int32_t* offsets, int32_t* nodes);
void mfbem_msh_free(void* msh);

/* Nodal-solution export (*.nso), host only: the boundary-node records that
   export_solution_mechanics_{harmonic,static}_nso write for an ordinary
   boundary of a BE region (src/export_solution_mechanics_harmonic_nso.f90,
   src/export_solution_mechanics_static_nso.f90), with the Fortran edit
   descriptors of the export settings (src/read_export.f90:61-70,163-171):
   integer columns I<int_w>, real columns kind 'E' (Ew.dEe, sci_*) or 'N'
   (ENw.dEe, eng_*). One record per node in export order: C1 frequency index
   (0 static), C2 frequency (0 static), C3-C5 region id / 1 / 2, C6-C8
   boundary id / 1 / 1, C9 node id, C10-C12 coordinates, then u1..u3, t1..t3
   (harmonic: complex_notation 2 re/im, 1 |z|/arg z, then the zero incident
   field). values: [n][6] real (static) or [n][6] complex as re/im pairs.
   header: text written first (NULL: none); append: add to the file.
   Returns 0, or -1 with the reason in mfbem_nso_error(). */
int mfbem_nso_write(const char* path, int32_t append, const char* header, int32_t harmonic, int32_t kf, double omega,
                    int32_t region_id, int32_t n, const int32_t* node_id, const int32_t* boundary_id, const double* x,
                    const double* values, int32_t int_w, char kind, int32_t w, int32_t d, int32_t e,
                    int32_t complex_notation);
const char* mfbem_nso_error(void);
/* One value under a Fortran edit descriptor ('I' w, 'E' Ew.dEe, 'N'
   ENw.dEe), right-justified in w characters, NUL-terminated into out. */
int mfbem_fortran_format(char kind, int32_t w, int32_t d, int32_t e, double v, char* out);

/* Device memory released with a mesh handle (mfbem_mesh_release) is kept by
   the library for later handles: buffers of at least 1 MB, up to a quarter of
   the device memory (environment MFBEM_DEVICE_CACHE_MB overrides the cap; 0
   disables the cache), with the handles' streams. This
   returns every cached buffer to the driver. No counterpart in the reference. */
int mfbem_trim_device_cache(void);

/* Diagnostics of the last mfbem_solve_r / mfbem_solve_c on the calling
   thread, which the reference prints at verbose level 2: rcond (NaN unless
   condition was set with factorize) and per right-hand side the forward-error
   bound ferr and the componentwise backward error berr (NaN unless refine). */
int mfbem_solve_report(double* rcond, int32_t n_rhs, double* ferr, double* berr);

/* Harmonic sweep on the device: for each of n_freq frequencies, assemble the
   FP64 system (same integration as mfbem_assemble_harela), factorise and solve.
   precision 0: plain FP64 LU (the drop-in method).
   precision 1: complex64 LU with FP64 iterative refinement to rel_tol in the
                backward error (the FP64 residual r = b - A x is evaluated with
                the FP64 matrix) and until the last correction is below 1e-10
                of x. The LU's trailing updates run on the tensor cores
                (tcgen05, 3xTF32: FP32-accurate factors); classical refinement
                x += LU^-1 r follows, GMRES-based refinement (FP64 GMRES
                preconditioned by the LU factors) when it stalls. With
                MFBEM_FP32_GEMM=tf32 (single-pass TF32 updates) a stall first
                redoes the LU with SIMT FP32 updates.
   precision 2: GMRES-based refinement from the start.
   x_out receives n_dof complex values per frequency (column f at f*n_dof).
   The right-hand side is the one assembled from the prescribed values. */
int mfbem_sweep_harela(mfbem_handle* h, const double lambda[2], const double mu[2], double rho, const double nu[2],
                       int32_t n_freq, const double* omega, int32_t precision, double rel_tol, double* x_out,
                       int32_t flags, mfbem_stats* stats);

/* Same for a static problem (one solve). */
int mfbem_solve_staela(mfbem_handle* h, double mu, double nu, int32_t precision, double rel_tol, double* x_out,
                       int32_t flags, mfbem_stats* stats);

/* No-allocation variant of mfbem_solve_c. No counterpart in the reference.
   For callers that cannot allocate device memory: hosts whose device memory
   is owned by another runtime's pool allocator, or that run under a hard cap
   on device allocations. Same arguments and results as mfbem_solve_c with
   scaling = condition = refine = 0 (host arrays; A receives the LU factors,
   ipiv the 1-based pivots, b the solutions; factorize = 0 reuses A/ipiv).
   The device working set is a fixed file-scope array of about 16 MiB that
   every GPU loading the library holds until the process exits; the call
   makes no cudaMalloc/cudaFree and uses no allocating library. Limits:
   n <= MFBEM_STATIC_MAX_N, n_rhs <= MFBEM_STATIC_MAX_RHS, else MFBEM_EARG.
   The first call on a device resolves the array's device address with that
   device current: make it before any stream capture. Every call shares the
   array; calls that overlap on the GPU (several host threads) race. */
#define MFBEM_STATIC_MAX_N 1024
#define MFBEM_STATIC_MAX_RHS 4
int mfbem_solve_c_static(int32_t n, double* A, int32_t* ipiv, int32_t n_rhs, double* b, int32_t factorize);

/* Statistics of the last assemble / sweep on this handle. */
int mfbem_last_stats(mfbem_handle* h, mfbem_stats* stats);

/* Error message of the last failing call on this thread ("" if none). */
const char* mfbem_last_error(void);

/* Library build identification: "<version> sm_103a". */
const char* mfbem_version(void);

/* Batch of harmonic sweeps over meshes of uneven size (no counterpart in the
   reference; the reference solves one problem at a time). Mesh i has its own
   material (lambda[2i], mu[2i], nu[2i] complex, rho[i]), n_freq[i]
   frequencies omega[i][...] and solution array x_out[i] (as
   mfbem_sweep_harela); the sweeps run concurrently on the GPU (one host
   thread and stream per mesh). stats: [n_mesh] or NULL. */
int mfbem_sweep_harela_batch(int32_t n_mesh, mfbem_handle* const* hs, const double* lambda, const double* mu,
                             const double* rho, const double* nu, const int32_t* n_freq, const double* const* omega,
                             int32_t precision, double rel_tol, double* const* x_out, int32_t flags,
                             mfbem_stats* stats);

/* ---------------------------------------------------------------------------
 * Learned quadrature of quasi-singular pairs. No counterpart in the reference:
 * an extension that replaces sbie_ext_adp's adaptive subdivision
 * (lib/fbem/src/bem_staela3d.f90:973-1096) by a rule an MLP predicts to be
 * accurate enough, keeping the reference rule where no candidate qualifies.
 * Candidates (index c): c < 7, the reference adaptive rule at
 * qsi_relative_error 10^-(3+c); c >= 7, graded subdivision of depth
 * D = (c-7)/9 toward the nearest point (3D + 1 leaves) with a Telles-mapped
 * g x g Gauss rule per leaf, g = {3,4,6,8,10,12,16,20,30}[(c-7)%9]. Network:
 * 8 features -> 3 x 64 tanh -> 52 predicted log10 relative errors, FP32
 * weights (mfbem_mlp_size() floats).
 * ------------------------------------------------------------------------- */

/* Labels of n (element, point) pairs generated by the caller: elem [n][8][3]
   quad8 node coordinates, pts [n][3]; kernel 0 static (nu = 0.3), 1 harmonic
   (E = 1, nu = 0.3, rho = 1, xi = 0.02, omega set by kcl[n] = |k2| x size).
   Outputs: feat [n][8] network inputs, logerr [n][52] log10 relative error of
   every candidate against the converged rule (D = 9, g = 30; errors below
   1e-10 are reported as 1e-10), cost [n][52] its quadrature points (-1 and
   error 10 for a reference-rule candidate beyond 128 leaves), valid [n]
   (converged rule checked to 1e-10 against D = 9, g = 24). */
int mfbem_qlearn_label(int32_t n, const double* elem, const double* pts, int32_t kernel, const double* kcl,
                       float* feat, float* logerr, int32_t* cost, int32_t* valid);
int32_t mfbem_mlp_size(void);
/* network outputs [n][52] for features [n][8] */
int mfbem_mlp_forward(const float* w, int32_t n, const float* feat, float* out);
/* mean squared error over valid samples and outputs, and its gradient [mfbem_mlp_size()] */
int mfbem_mlp_loss_grad(const float* w, int32_t n, const float* feat, const float* y, const int32_t* valid,
                        float* loss, float* grad);
/* Adam training in place on device-drawn mini-batches; loss_hist [steps] may be NULL */
int mfbem_mlp_train(float* w, int32_t n, const float* feat, const float* y, const int32_t* valid, int32_t steps,
                    int32_t batch, float lr, uint64_t seed, float* loss_hist);
/* Rebuild a mesh's quasi-singular pair rules from the network w (NULL: the
   reference rule everywhere): per pair the cheapest candidate whose predicted
   log10 error is <= log10_tol, else the reference rule. kernel / kcl are the
   network inputs for the wavenumber (0 / 0 for the static kernel). */
int mfbem_set_learned_quadrature(mfbem_handle* h, const float* w, double log10_tol, int32_t kernel, double kcl,
                                 int32_t* n_learned);

#ifdef __cplusplus
}
#endif
#endif /* MFBEM_H */
