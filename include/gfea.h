/*
 * gfea.h -- C ABI of libgb300fea.so, the GB300 (sm_103a) finite-element hot
 * path behind easyfea_gb300's Simulations.Elastic / Simulations.PhaseField.
 *
 * Conventions
 *  - extern "C", plain pointers and sizes, no C++ types across the boundary.
 *  - Every array argument is a DEVICE pointer (caller-owned, e.g. a torch
 *    tensor's data_ptr()) unless its name ends in _host.
 *  - Every entry point returns an int status (GFEA_OK == 0); nothing throws.
 *  - The library allocates no device memory: scratch comes from caller
 *    buffers sized by the matching *_workspace_size query.
 *  - All work is enqueued on the given stream; calls that return values to
 *    the host (counts, PCG results) synchronise that stream.
 *
 * Data layout (DOF numbering node*dof_n + component, EasyFEA/FEM/_group_elem.py:346-380):
 *  - coord   double[Nn*3]           node coordinates (x, y, z)
 *  - connect int32[Ne*nPe]          element connectivity, reference node order
 *  - node graph: node_ptr int32[Nn+1], nbr int32[node_ptr[Nn]] -- sorted
 *    neighbour nodes of every node (nodes sharing an element, itself included)
 *  - rank    uint8[Ne*nPe*nPe]      position of connect[e,q] in the neighbour
 *    list of connect[e,p]; the CSR slot of element entry (p,i,q,j) is
 *    indptr[dof_n*a+i] + dof_n*rank + j with a = connect[e,p]
 *  - CSR values are laid out exactly as scipy's canonical CSR of the
 *    reference (sorted column indices, one slot per coupled DOF pair):
 *    row (a,i) starts at dof_n^2*node_ptr[a] + i*dof_n*nnb(a).
 */
#ifndef GFEA_H
#define GFEA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GFEA_ABI_VERSION 1

/* status codes */
#define GFEA_OK 0
#define GFEA_ERR_ARG 1          /* invalid argument / size                       */
#define GFEA_ERR_CUDA 2         /* a CUDA runtime call failed                    */
#define GFEA_ERR_CAPACITY 3     /* a node has more neighbours than supported     */
#define GFEA_ERR_SINGULAR 4     /* zero / singular diagonal block                */
#define GFEA_ERR_NOT_CONVERGED 5/* PCG reached max_iters                         */
#define GFEA_ERR_BREAKDOWN 6    /* PCG p.Ap <= 0 (matrix not SPD on unknowns)    */
#define GFEA_ERR_NAN 7          /* non-finite value met                          */
#define GFEA_ERR_WORKSPACE 8    /* workspace too small                           */
#define GFEA_ERR_TIMEOUT 9      /* a bounded device wait gave up (staged copies)  */

/* element codes; each element's local node order is the reference's
   (EasyFEA/FEM/Elems/_seg.py, _tri.py, _quad.py, _tetra.py, _hexa.py,
   _prism.py Get_Local_Coords) */
#define GFEA_SEG2 0
#define GFEA_TRI3 1
#define GFEA_QUAD4 2
#define GFEA_QUAD9 3
#define GFEA_HEXA8 4
#define GFEA_TETRA4 5
#define GFEA_TRI6 6
#define GFEA_QUAD8 7
#define GFEA_TETRA10 8
#define GFEA_SEG3 9
#define GFEA_HEXA20 10
#define GFEA_HEXA27 11
#define GFEA_PRISM6 12
#define GFEA_PRISM15 13
#define GFEA_PRISM18 14
#define GFEA_TRI10 15
#define GFEA_TRI15 16
#define GFEA_SEG4 17
#define GFEA_SEG5 18

/* value types */
#define GFEA_F64 0
#define GFEA_F32 1

/* phase-field splits and regularisations (EasyFEA/Models/_phasefield.py:41-70) */
#define GFEA_SPLIT_BOURDIN 0
#define GFEA_SPLIT_AMOR 1
#define GFEA_SPLIT_MIEHE 2
#define GFEA_SPLIT_ZHANG 3
#define GFEA_SPLIT_STRESS 4
#define GFEA_SPLIT_HE 5
#define GFEA_SPLIT_ANISOT_STRAIN 6
#define GFEA_SPLIT_ANISOT_STRAIN_PM 7
#define GFEA_SPLIT_ANISOT_STRAIN_MP 8
#define GFEA_SPLIT_ANISOT_STRAIN_NOCROSS 9
#define GFEA_SPLIT_ANISOT_STRESS 10
#define GFEA_SPLIT_ANISOT_STRESS_PM 11
#define GFEA_SPLIT_ANISOT_STRESS_MP 12
#define GFEA_SPLIT_ANISOT_STRESS_NOCROSS 13
#define GFEA_AT1 0
#define GFEA_AT2 1

const char* gfea_version(void);
const char* gfea_status_string(int status);

/* ------------------------------------------------------------------------
 * Sparsity pattern.  Replaces _Simu.__Get_csr_map (EasyFEA/Simulations/
 * _simu.py:1062-1102) and _GroupElem.Get_rows_e/Get_columns_e
 * (EasyFEA/FEM/_group_elem.py:382-402): the node graph and the element slot
 * ranks are built on the device; indptr/indices equal scipy's canonical
 * pattern bit for bit.
 * ---------------------------------------------------------------------- */
int gfea_graph_workspace_size(int64_t n_nodes, int64_t n_elems, int nPe, size_t* bytes_host);
/* pass 1: node_ptr[Nn+1] (exclusive scan of neighbour counts); also copies
 * node_ptr[Nn] (number of node pairs) to *n_pairs_host. */
int gfea_graph_count(const int32_t* connect, int64_t n_elems, int nPe, int64_t n_nodes,
                     int32_t* node_ptr, int64_t* n_pairs_host, void* work, size_t work_bytes,
                     void* stream);
/* pass 2 (same workspace, untouched since pass 1): nbr[n_pairs], rank[Ne*nPe*nPe] */
int gfea_graph_fill(const int32_t* connect, int64_t n_elems, int nPe, int64_t n_nodes,
                    const int32_t* node_ptr, int32_t* nbr, uint8_t* rank, void* work,
                    size_t work_bytes, void* stream);
/* DOF-level CSR pattern for dof_n components per node: indptr[Nn*dof_n+1] (int64),
 * indices[dof_n^2 * n_pairs] (int32). */
int gfea_csr_pattern(const int32_t* node_ptr, const int32_t* nbr, int64_t n_nodes, int dof_n,
                     int64_t* indptr, int32_t* indices, void* stream);

/* ------------------------------------------------------------------------
 * Element operators fused with the CSR scatter.
 * ---------------------------------------------------------------------- */
/* K = sum_e sum_pg wJ B^T C B * factor into CSR values (rigi Gauss points).
 * Replaces Bilinear.LinearizedElasticity (EasyFEA/FEM/Operators/Bilinear.py:62-79)
 * with _GroupElem.Get_F_e_pg .. Get_leftDispPart_e_pg (EasyFEA/FEM/
 * _group_elem.py:833-1333), Elastic.Construct_local_matrix_system's K part
 * (EasyFEA/Simulations/_elastic.py:123-152) and _Simu.__Assemble_csr's
 * bincount (EasyFEA/Simulations/_simu.py:989-1060).
 * C: Kelvin-Mandel (3x3 in 2D, 6x6 in 3D), c_per_elem = 0 homogeneous,
 * 1 per element (Ne x n x n, Models/_utils.py:69-108), 2 a reference n x n
 * matrix followed by Ne per-element factors (C_e = f_e C_ref, e.g. a
 * per-element Young's modulus with a constant Poisson ratio); for an
 * isotropic law C = lambda 1 (x) 1 + 2 mu I (Kelvin-Mandel; plane stress with
 * its reduced lambda), c_per_elem = 3 passes C = {lambda, mu} and 4 passes
 * {lambda, mu} followed by Ne per-element factors: the same matrix from
 * K_pq = sum wJ (lambda a b^T + mu b a^T + mu (a.b) I), a = grad N_p,
 * b = grad N_q, with about a third of the floating-point work.
 * C must be symmetric (as every elastic law's Kelvin-Mandel matrix is): each
 * element computes K_pq for one of each pair of nodes and scatters K_qp =
 * K_pq^T.  values (value_type GFEA_F64/F32, n_values = dof_n^2 * n_pairs
 * entries) are zeroed first unless accumulate != 0. */
int gfea_assemble_elastic(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                          const int32_t* node_ptr, const uint8_t* rank, const double* C,
                          int c_per_elem, double factor, int value_type, void* values,
                          int64_t n_values, int accumulate, void* stream);

/* Row-owned assembly: the same K as gfea_assemble_elastic (accumulate = 0)
 * without global atomics.  The nodes are cut into parts whose CSR rows fit in
 * shared memory (max_part_values values each, nodes in Morton order of their
 * coordinates); one thread block per part adds the element blocks of its own
 * rows in shared memory and writes them once.  The plan is built on the host
 * once per mesh (and dof_n, and max_part_values):
 *   node_off[Nn]          offset of the node's rows within its part
 *   part_node_ptr[P+1], part_nodes[Nn]   the nodes of each part
 *   part_nvals[P]         values of each part
 *   visit_ptr[P+1], visit_elem[V], visit_mask[V]   the elements touching each
 *                         part, with the bitmask of their local nodes it owns
 * The host arrays must hold Nn, Nn + 1, Nn, Nn, Nn + 1, Ne*nPe and Ne*nPe
 * entries (upper bounds of P and V); *n_parts_host and *n_visits_host get
 * the sizes.  gfea_part_smem_bytes gives the dynamic shared memory a block
 * takes for parts of max_part_values values (at most 200 KiB is accepted). */
typedef struct gfea_part_plan {
  int32_t version;          /* GFEA_ABI_VERSION */
  int32_t n_parts;
  int32_t max_part_values;  /* the value the plan was built with */
  int32_t threads;          /* threads per block: a multiple of 32 up to 256; 0: 256 (FP32), 128 (FP64) */
  const int32_t* node_off;
  const int32_t* part_node_ptr;
  const int32_t* part_nodes;
  const int32_t* part_nvals;
  const int32_t* visit_ptr;
  const int32_t* visit_elem;
  const uint32_t* visit_mask;
} gfea_part_plan;
int gfea_part_plan_host(const double* coord_host, const int32_t* connect_host, int64_t n_elems, int nPe,
                        int64_t n_nodes, const int32_t* node_ptr_host, int dof_n, int32_t max_part_values,
                        int32_t* node_off_host, int32_t* part_node_ptr_host, int32_t* part_nodes_host,
                        int32_t* part_nvals_host, int32_t* visit_ptr_host, int32_t* visit_elem_host,
                        uint32_t* visit_mask_host, int32_t* n_parts_host, int64_t* n_visits_host);
size_t gfea_part_smem_bytes(int elem, int value_type, int32_t max_part_values, int threads);
int gfea_assemble_elastic_parts(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                                const int32_t* node_ptr, const uint8_t* rank, const double* C,
                                int c_per_elem, double factor, int value_type, void* values,
                                const gfea_part_plan* plan, void* stream);

/* M = sum_e sum_pg rho wJ N^T N * factor (mass Gauss points, dof_n components).
 * Replaces Bilinear.UV (EasyFEA/FEM/Operators/Bilinear.py:42-59) as used by
 * EasyFEA/Simulations/_elastic.py:137. */
int gfea_assemble_mass(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                       const int32_t* node_ptr, const uint8_t* rank, int dof_n, double rho,
                       double factor, int value_type, void* values, int64_t n_values,
                       int accumulate, void* stream);

/* Neumann surface / line loads: b[dof] += factor * value_u * sum_pg wJ N
 * over boundary elements whose every node has node_mask set (mass Gauss
 * points).  Replaces _Simu.__Bc_Integration_Dim (EasyFEA/Simulations/
 * _simu.py:2770-2842) for constant values (gfea_surface_load_field below
 * takes values that vary over the boundary), and the COO summation of
 * _Solver_Apply_Neumann (:1750-1756). */
int gfea_surface_load(int belem, const double* coord, const int32_t* bconnect, int64_t n_belems,
                      const uint8_t* node_mask, int dof_n, int n_unknowns,
                      const int32_t* unknown_idx_host, const double* values_host, double factor,
                      double* b, void* stream);

/* Coordinates of the mass Gauss points of boundary elements,
 * xyz[(e * nPg + g) * 3 + k] (n_belems * nPg * 3 doubles); *npg_host = nPg
 * (with n_belems = 0 only *npg_host is set: size xyz from it).
 * The points where _Simu.__Bc_evaluate evaluates a load given as a function
 * of position (EasyFEA/Simulations/_simu.py:2353-2385 with
 * Get_GaussCoordinates_e_pg, :2803-2811). */
int gfea_boundary_gauss_points(int belem, const double* coord, const int32_t* bconnect, int64_t n_belems,
                               double* xyz, int32_t* npg_host, void* stream);

/* Neumann load of one unknown with values varying over the boundary, on the
 * elements whose every node has node_mask set: mode 0, values at the mass
 * Gauss points (values[e * nPg + g], a function evaluated at the points of
 * gfea_boundary_gauss_points): b += factor * sum_g wJ f_g N(g); mode 1,
 * values per node (values[node]): b_p += factor * f_p * sum_g wJ N_p(g).
 * Replaces the callable and array branches of _Simu.__Bc_Integration_Dim
 * (EasyFEA/Simulations/_simu.py:2811-2832). */
int gfea_surface_load_field(int belem, const double* coord, const int32_t* bconnect, int64_t n_belems,
                            const uint8_t* node_mask, int dof_n, int unknown_idx, int mode,
                            const double* values, double factor, double* b, void* stream);

/* ------------------------------------------------------------------------
 * Phase field.
 * ---------------------------------------------------------------------- */
typedef struct gfea_pf_params {
  int32_t version;       /* GFEA_ABI_VERSION */
  int32_t split;         /* GFEA_SPLIT_* */
  int32_t regularization;/* GFEA_AT1 / GFEA_AT2 */
  int32_t dim;           /* 2 or 3 */
  double lambda_, mu;    /* Lame constants (plane-stress lambda in 2D plane stress) */
  double Gc, l0;
  double thickness;      /* factor applied to Kd, Fd, Ku (1 in 3D) */
  double A[9];           /* diffusion tensor, row-major dim x dim (identity by default) */
  double C[36];          /* Kelvin-Mandel C, row-major n x n (Bourdin, Zhang, Stress, He splits) */
  double k_res;          /* residual stiffness of g(d), 1e-12 in the reference */
  int32_t plane_stress;  /* 2D: 1 plane stress, 0 plane strain (the Stress split's compliance) */
  int32_t pad;
  double S[36];          /* Kelvin-Mandel compliance C^-1 (AnisotStress splits) */
} gfea_pf_params;

/* Damage system at the current displacement: strain at mass Gauss points,
 * split, psi+ with the History max against H_old (NULL = none), r/f/k,
 * Kd = int r N^T N + int k grad N . A grad N, Fd = int f N (x thickness).
 * Replaces PhaseField.__Construct_Damage_Matrix and __Calc_psiPlus_e_pg
 * (EasyFEA/Simulations/_phasefield.py:494-573) with Models.PhaseField
 * Calc_psi_e_pg / Calc_C / Get_r_e_pg / Get_f_e_pg / k
 * (EasyFEA/Models/_phasefield.py:237-571, :751-1243).
 * H_new (Ne x nPg_mass) receives psi+ after the max; Kd values (dof_n 1
 * pattern) and Fd (Nn) are zeroed first. */
int gfea_pf_damage(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                   const int32_t* node_ptr, const uint8_t* rank, const double* u,
                   const gfea_pf_params* params_host, const double* H_old, double* H_new,
                   double* Kd_values, double* Fd, void* stream);

/* Degraded displacement stiffness: strain at rigi Gauss points, split,
 * g = (1 - N.d)^2 + k_res, c = g cP + cM, K = int B^T c B (x thickness).
 * Replaces PhaseField.__Construct_Elastic_Matrix (EasyFEA/Simulations/
 * _phasefield.py:444-482) and Get_g_e_pg (EasyFEA/Models/_phasefield.py:295-317). */
int gfea_pf_elastic(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                    const int32_t* node_ptr, const uint8_t* rank, const double* u, const double* d,
                    const gfea_pf_params* params_host, int value_type, void* values, void* stream);

/* psi+ / psi- and cP / cM of given strains (Ne*nPg rows of n KM components):
 * Models.PhaseField.Calc_C + Calc_psi_e_pg (EasyFEA/Models/_phasefield.py:335-571).
 * Any of cP, cM, psiP, psiM may be NULL. */
int gfea_pf_split(const double* eps, int64_t n_points, const gfea_pf_params* params_host,
                  double* cP, double* cM, double* psiP, double* psiM, void* stream);

/* ------------------------------------------------------------------------
 * Post-processing: element results of a displacement field and their node
 * averages, computed where the field lives.
 * ---------------------------------------------------------------------- */
typedef struct gfea_fields {
  int32_t version;          /* GFEA_ABI_VERSION */
  int32_t gauss;            /* 0: rigi Gauss points, 1: mass Gauss points */
  double coef;              /* strain_e / stress_e shear components are the Kelvin-Mandel
                               ones times 1/coef (sqrt(2): tensor components, as the
                               reference's results; 1: Kelvin-Mandel) */
  double thickness;         /* factor of energy_e (2D thickness, 1 in 3D) */
  const double* C;          /* elastic law, as gfea_assemble_elastic's C / c_per_elem */
  int32_t c_per_elem;
  int32_t pad;
  const gfea_pf_params* pf; /* non-NULL: phase-field stress g(d) cP eps + cM eps, and psiP_e */
  const double* d;          /* nodal damage (pf) */
  const double* H_old;      /* pf: History field at this Gauss family (Ne x nPg), max'ed into psiP_e; may be NULL */
  const double* sigma_n;    /* non-NULL: energy_e integrates 1/2 (N sigma_n) . eps, sigma_n the nodal
                               Kelvin-Mandel stress (Nn x n) -- the ZZ1 smoothed energy */
  double* strain_e;         /* Ne x n: mean over the Gauss points of eps (scaled shear) */
  double* stress_e;         /* Ne x n: same for sigma */
  double* vm_e;             /* Ne x 2: mean of the von Mises equivalent of eps, of sigma */
  double* energy_e;         /* Ne: thickness * sum_pg wJ 1/2 sigma . eps */
  double* psiP_e;           /* Ne: mean of psi+ (pf) */
} gfea_fields;
/* Replaces Elastic.Result's strain and stress results (EasyFEA/Simulations/
 * _elastic.py:296-320) through Result_strain_or_stress_field_e and
 * __Result_in_Strain_or_Stress_field (EasyFEA/Models/_utils.py:302-430),
 * Elastic._Calc_Psi_Elas with and without smoothing (_elastic.py:322-395),
 * PhaseField._Calc_Sigma_e_pg (EasyFEA/Simulations/_phasefield.py:868-915)
 * and its psiP result (:494-530, :706-714).  Any output may be NULL. */
int gfea_element_fields(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                        const double* u, const gfea_fields* fields_host, void* stream);
/* Node -> incident elements, each list ascending: inc_ptr[Nn+1], inc_list[Ne*nPe]
 * (the rows of _GroupElem.Get_connect_n_e, EasyFEA/FEM/_group_elem.py:322-345).
 * Workspace: gfea_graph_workspace_size. */
int gfea_node_incidence(const int32_t* connect, int64_t n_elems, int nPe, int64_t n_nodes,
                        int32_t* inc_ptr, int32_t* inc_list, void* work, size_t work_bytes,
                        void* stream);
/* values_n[a, c] = (sum over the elements e of node a of values_e[e, c]) / (their
 * number), summed in ascending e:
 * Mesh.Get_Node_Values (EasyFEA/FEM/_mesh.py:822-873). */
int gfea_node_average(const int32_t* inc_ptr, const int32_t* inc_list, int64_t n_nodes,
                      const double* values_e, int n_cols, double* values_n, void* stream);

/* ------------------------------------------------------------------------
 * Sparse SPD solve.  Replaces Solvers.__Solver_1 (EasyFEA/Simulations/
 * Solvers.py:502-553: Dirichlet elimination) and _Solve_Axb's spsolve
 * (Solvers.py:361-362) by block-Jacobi PCG on the masked operator
 * P A P + (I - P), P = diag(unknown), which equals the reference's reduced
 * system A_ii x_i = b_i - A_ic x_c.
 * ---------------------------------------------------------------------- */
typedef struct gfea_system {
  int32_t version;          /* GFEA_ABI_VERSION */
  int32_t dof_n;            /* components per node (1, 2, 3) */
  int64_t n_nodes;
  int64_t n_pairs;          /* node_ptr[n_nodes] */
  const int32_t* node_ptr;  /* node graph */
  const int32_t* nbr;
  const double* vals64;     /* CSR values, FP64 (may be NULL for FP32-only use) */
  const float* vals32;      /* CSR values, FP32 (may be NULL for FP64-only use) */
  const uint8_t* known;     /* per-DOF Dirichlet mask (1 = known) */
  int32_t translation_invariant; /* 1: node block rows sum to zero (elastic stiffness);
                               the FP32 products then use y_a = sum_b K_ab (x_b - x_a) */
  int32_t pad;
  const double* coord;      /* node coordinates (Nn x 3) for the coarse level; may be NULL */
} gfea_system;

typedef struct gfea_pcg_opts {
  int32_t version;          /* GFEA_ABI_VERSION */
  int32_t precision;        /* GFEA_F64: FP64 PCG; GFEA_F32: FP32 inner PCG + FP64 refinement */
  int32_t max_iters;        /* total PCG iteration cap */
  int32_t check_every;      /* host convergence check period (iterations); <= 0: adaptive
                               (first check after about as many iterations as the
                               previous reliable-update cycle took, then doubling) */
  double rtol;              /* target ||P(b - A x)|| / ||P(b - A x_c)||; the solve
                               stops at max(rtol, rounding floor), see gfea_pcg_result */
  double inner_rtol;        /* FP32: reduction of the iterated residual between FP64
                               residual replacements (reliable updates); outside (0, 1):
                               0.1 with block-Jacobi alone, 0.01 with the coarse level */
  int32_t max_refine;       /* refinement steps cap (mixed precision) */
  int32_t lanes;            /* SpMV lanes per node (0 = automatic) */
  int32_t coarse;           /* two-level preconditioner: target number of aggregates
                               (0 = block-Jacobi only, -1 = automatic); needs sys.coord */
  int32_t coarse_reuse;     /* 1: the workspace holds the aggregation of an earlier call
                               on the same mesh (same coordinates, node count and
                               'coarse'); it is kept and only the coarse matrix is rebuilt */
} gfea_pcg_opts;

typedef struct gfea_pcg_result {
  int32_t status;           /* GFEA_OK or an error code */
  int32_t iterations;       /* PCG iterations performed (all refinement steps) */
  int32_t refinements;      /* inner PCG solves (each followed by an FP64 residual) */
  int32_t pad;
  double rel_residual;      /* final FP64 ||P(b - A x)|| / ||P(b - A x_c)|| */
  double floor_rel;         /* rounding floor of that residual: 32 eps ||P(|A||x|+|b|)|| / ||P(b - A x_c)|| */
} gfea_pcg_result;

/* ------------------------------------------------------------------------
 * Batched solves: many independent Dirichlet-reduced systems (different
 * sizes, dof_n 1-3) solved in one persistent launch.  Each thread-block
 * cluster takes one system at a time and runs its whole PCG (FP32 iteration
 * with FP64 reliable updates, or FP64) with cluster-wide reductions, so a
 * system's result does not depend on the other systems in the batch.  This
 * is the batched driver behind the reference's per-instance loop of
 * Simulations.*.Solve calls (one SuperLU solve each, Solvers.py:361).
 * ---------------------------------------------------------------------- */
/* Coarse level of the two-level preconditioner for one system of a batch
 * (gfea_coarse_setup): pointers into the workspace it was built in. */
typedef struct gfea_coarse_level {
  int32_t n_agg;            /* aggregates (0: no coarse level, block-Jacobi only) */
  int32_t nr;               /* rigid-body modes per aggregate (1, 3 or 6) */
  int32_t nc;               /* coarse dimension nr * n_agg (<= 512) */
  int32_t pad;
  const int32_t* agg;       /* node -> aggregate */
  const float* off;         /* 4 floats per node: offset from its cell centre, scaled */
  const int32_t* agg_ptr;   /* n_agg + 1: ranges of agg_nodes */
  const int32_t* agg_nodes; /* the nodes of each aggregate, ascending */
  const double* inv;        /* nc x nc inverse of the coarse matrix R^T A R */
  const float* inv32;       /* its FP32 copy */
  double* rc;               /* nc: restriction scratch of the batched solve */
  double* ec;               /* nc: coarse correction scratch */
} gfea_coarse_level;

typedef struct gfea_batch_instance {
  int32_t version;          /* GFEA_ABI_VERSION */
  int32_t dof_n;
  int64_t n_nodes;
  int64_t n_pairs;
  const int32_t* node_ptr;
  const int32_t* nbr;
  const double* vals64;     /* FP64 CSR values (residuals) */
  const float* vals32;      /* FP32 copy (FP32 iteration); may be NULL for FP64 batches */
  const uint8_t* known;
  int32_t translation_invariant;
  int32_t max_iters;
  double rtol;
  const double* b;          /* right-hand side */
  double* x;                /* in: known values + initial guess; out: solution */
  void* work;               /* gfea_batch_workspace_size() bytes, 256-byte aligned */
  gfea_pcg_result* result;  /* device pointer, written when the system's solve ends */
  gfea_coarse_level coarse; /* two-level preconditioner (n_agg = 0: block-Jacobi only) */
} gfea_batch_instance;

size_t gfea_batch_workspace_size(int64_t n_nodes, int dof_n, int precision);
/* Coarse level of one batch system: the aggregation, coarse matrix and
 * inverse of gfea_pcg_solve's two-level preconditioner (aggregate count from
 * opts.coarse, automatic when -1, capped at nc = 512), built into 'work'
 * (gfea_coarse_workspace_size bytes, 256-byte aligned; FP32 coarse matrix for
 * opts.precision GFEA_F32, FP64 otherwise).  keep_aggregation != 0 keeps the
 * aggregation a previous call left in the same workspace for the same mesh
 * ('level' as that call returned it) and rebuilds only the coarse matrix and
 * its inverse, with device work only (capturable in a CUDA graph); without it
 * the aggregation reads the mesh's bounding box back to the host once.  No
 * reference counterpart (the reference solves each instance with SuperLU). */
int gfea_coarse_workspace_size(const gfea_system* sys_host, const gfea_pcg_opts* opts_host, size_t* bytes_host);
int gfea_coarse_setup(const gfea_system* sys_host, const gfea_pcg_opts* opts_host, int keep_aggregation,
                      void* work, size_t work_bytes, gfea_coarse_level* level_host, void* stream);
/* The coarse matrices and inverses of a whole batch rebuilt from the current
 * values with one launch per stage (instead of ~60 per system): prepare
 * uploads one descriptor per system into scratch
 * (gfea_coarse_batch_scratch_size(n) bytes) from systems[i], works[i] and
 * levels[i] as gfea_coarse_setup returned them (its aggregation is kept;
 * systems ordered by dof_n); build enqueues device work only (capturable):
 * dof_n_first[d - 1] = index of the first system with dof_n = d (d = 1..3,
 * n when there is none), dof_n_first[3] = n; max_nc = the largest level's nc. */
size_t gfea_coarse_batch_scratch_size(int n);
int gfea_coarse_batch_prepare(const gfea_system* systems_host, const gfea_pcg_opts* opts_host, int n,
                              void* const* works_host, const gfea_coarse_level* levels_host, void* scratch,
                              size_t scratch_bytes, void* stream);
int gfea_coarse_batch_build(const void* scratch, int n, const int32_t* dof_n_first_host, int max_nc,
                            int precision, void* stream);
size_t gfea_batch_scratch_size(int n_instances);
/* Enqueues the batch on the stream and returns; results are valid once the
 * stream has completed.  scratch: gfea_batch_scratch_size(n) device bytes
 * (work counter + descriptors).  opts: precision (GFEA_F32 / GFEA_F64) and
 * inner_rtol (FP32 reliable-update trigger); rtol and max_iters are per system. */
int gfea_batch_pcg(const gfea_batch_instance* instances_host, int n, void* scratch, size_t scratch_bytes,
                   const gfea_pcg_opts* opts_host, void* stream);
/* gfea_batch_pcg in two parts, for CUDA-graph capture of the solve:
 * gfea_batch_prepare validates the instances and uploads their descriptors
 * (largest first) into scratch; gfea_batch_launch enqueues only device work
 * (a counter reset and the persistent kernel), so it can be captured and
 * replayed while the descriptors' buffers stay valid.  n and opts must be the
 * ones given to the prepare call. */
int gfea_batch_prepare(const gfea_batch_instance* instances_host, int n, void* scratch, size_t scratch_bytes,
                       const gfea_pcg_opts* opts_host, void* stream);
int gfea_batch_launch(void* scratch, int n, const gfea_pcg_opts* opts_host, void* stream);

/* y = A x (unmasked), value_type selects vals64/x,y double or vals32/x,y float. */
int gfea_spmv(const gfea_system* sys_host, int value_type, const void* x, void* y, void* stream);

/* The workspace holds the PCG vectors, the coarse level and, when the
 * operator can be staged, a packed copy of it in node tiles (about 1.15x the
 * iterated values plus the neighbour indices) that the staged SpMV streams
 * with one bulk copy per tile.  A smaller workspace that still holds the rest
 * is accepted: the solve then runs the unstaged SpMV. */
int gfea_pcg_workspace_size(const gfea_system* sys_host, const gfea_pcg_opts* opts_host,
                            size_t* bytes_host);

/* x: on entry known DOFs hold their Dirichlet values and unknown DOFs the
 * initial guess; on exit the solution.  b: full right-hand side. */
int gfea_pcg_solve(const gfea_system* sys_host, const double* b, double* x,
                   const gfea_pcg_opts* opts_host, void* work, size_t work_bytes,
                   gfea_pcg_result* result_host, void* stream);

/* gfea_pcg_solve without a workspace argument: allocates nothing.  It has no
 * counterpart in the reference.  It is meant for callers that cannot allocate
 * device memory -- a solver embedded in an application whose device memory is
 * owned by another allocator or a pre-reserved pool, or a latency-critical
 * loop where allocation is not allowed.  Its scratch is a static 16 MiB array
 * inside this library (held by every GPU that loads it until the process
 * exits), so the problem must fit: FP64 needs (7 + dof_n) * 8 bytes per DOF
 * plus ~40 KB (about 209,000 DOF in 3D, 232,000 in 2D); larger problems are
 * rejected with GFEA_ERR_WORKSPACE before any device work.  It launches its
 * kernels directly: it instantiates no CUDA graph and creates no stream or
 * event, and it skips the schedule tuner and the kernel timing.  Every call
 * looks the array's device address up (cudaGetSymbolAddress) in the current
 * device's context; the first call on a device may also load the library's
 * module there, so make that first call before any stream capture.
 * opts.coarse_reuse is ignored: the array keeps what the last call (on any
 * mesh) left in it, so the coarse aggregation is rebuilt every call.  All
 * calls share the array and reset what must start at zero: calls that overlap
 * on the GPU (different streams or threads) race and must be serialised. */
int gfea_pcg_solve_noalloc(const gfea_system* sys_host, const double* b, double* x,
                           const gfea_pcg_opts* opts_host, gfea_pcg_result* result_host,
                           void* stream);

/* Scratch bytes of the reductions below. */
size_t gfea_reduce_workspace_size(void);

/* Reductions for Calc_Reaction / Calc_Energy (EasyFEA/Simulations/_simu.py:177-260):
 * Ax = A x (FP64); out_host[0] = sum_{dofs} (A x)[dof]  (dofs: n_dofs device
 * indices); out_host[1] = 1/2 x.A x over all DOFs. */
int gfea_reaction_energy(const gfea_system* sys_host, const double* x, const int64_t* dofs,
                         int64_t n_dofs, double* Ax, double* out_host, void* work, void* stream);

/* max_i |a_i - b_i| (PhaseField.Solve convOption 0, EasyFEA/Simulations/_phasefield.py:379) */
int gfea_max_abs_diff(const double* a, const double* b, int64_t n, double* out_host,
                      void* work, void* stream);

/* Instrumentation: kernels launched by the library so far; optional
 * CUDA-event timing of the launches of PCG iterations (per kernel kind, from
 * every host thread); gfea_profile_read returns the SpMV kernel's total ms and
 * launches since the last read (reading resets; with GFEA_DEBUG set in the
 * environment the per-kind table is printed to stderr). */
long long gfea_launch_count(void);
/* CUDA graphs the library has instantiated in this process (the PCG captures
 * four iterations per graph for a solve running alone; the allocation-free
 * solve never does). */
long long gfea_cuda_graph_count(void);
int gfea_profile_enable(int on);
int gfea_profile_read(double* ms_host, long long* launches_host);

/* Self-test of the bounded device waits (no reference counterpart): one
 * thread waits on an mbarrier phase with a limit of limit_us microseconds
 * (1 .. 1e6), after one arrival (arrive != 0: *status_host = GFEA_OK) or none
 * (*status_host = GFEA_ERR_TIMEOUT, the status a staged SpMV reports when a
 * wait runs out); the context stays usable. */
int gfea_selftest_wait(int32_t limit_us, int32_t arrive, int32_t* status_host, void* stream);

/* FP64 -> FP32 copy of CSR values (mixed-precision operator) */
int gfea_cast_f64_f32(const double* src, float* dst, int64_t n, void* stream);

/* ------------------------------------------------------------------------
 * Autotuner (no counterpart in the reference).  Two schedules are chosen by
 * measurement and kept per problem class: the SpMV row-block schedule (lanes
 * per node of the node-row products, keyed by dof_n, value type and the log2
 * buckets of the row length and node count) and the element-kernel tile
 * schedule (blocks of 128 threads per SM, keyed by element, value type,
 * C mode and the log2 bucket of the element count).
 * mode 0: fixed rules; 1 (default): use recorded decisions; 2: also tune a
 * class on its first gfea_pcg_solve / gfea_assemble_elastic (not accumulating).
 * ---------------------------------------------------------------------- */
int gfea_tune_mode(int mode);
int gfea_tune_clear(void);
/* Times y = A x with 4, 8, 16, 32 lanes per node; records and returns the
 * fastest (lanes_host) and its time (ms_host). */
int gfea_tune_spmv(const gfea_system* sys_host, int value_type, const void* x, void* y,
                   int32_t* lanes_host, float* ms_host, void* stream);
/* gfea_assemble_elastic (accumulate = 0) timed with 4..64 blocks per SM;
 * records the fastest and leaves the values assembled. */
int gfea_tune_assemble_elastic(int elem, const double* coord, const int32_t* connect, int64_t n_elems,
                               const int32_t* node_ptr, const uint8_t* rank, const double* C,
                               int c_per_elem, double factor, int value_type, void* values,
                               int64_t n_values, int32_t* blocks_per_sm_host, float* ms_host,
                               void* stream);
/* Recorded decisions as (key, value) pairs: export writes up to max_entries
 * and sets *n_host to the total; import adds or replaces entries. */
int gfea_tune_export(int64_t* keys_host, int32_t* values_host, int max_entries, int* n_host);
int gfea_tune_import(const int64_t* keys_host, const int32_t* values_host, int n);

#ifdef __cplusplus
}
#endif

#endif /* GFEA_H */
