/*
 * svl_gb300.h -- C ABI of the GB300-native SeismoVLAB time-stepping hot path.
 *
 * Everything here is plain C: pointers, sizes and status codes, no C++ or torch
 * types.  One opaque handle per integrator; each handle owns its device
 * buffers and one CUDA stream and is not thread-safe (independent handles may
 * be driven from different host threads).  Host arrays passed to *_create are
 * copied; the caller keeps ownership.
 *
 * Error convention.  Every entry point returns an int status: SVL_OK (0) on
 * success, a positive SVL_ERR_* code otherwise, with a message available from
 * svl_last_error().  The reference returns `bool stop` (true = failure) from
 * LinearSystem::SolveSystem (RP/11-Solvers/01-Direct/EigenSolver.cpp:52-58),
 * Integrator::ComputeNewStep (RP/10-Integrators/02-CentralDifference/
 * CentralDifference.cpp:132-135) and Analysis::Analyze
 * (RP/08-Analysis/02-Dynamic/DynamicAnalysis.cpp:41-44); the C++ adapters in
 * svl_gb300/host map status != 0 to stop == true.
 *
 * Paths in citations are relative to the SeismoVLAB/SVL tree: RP/ is
 * 02-Run_Process/, PP/ is 01-Pre_Process/.
 */
#ifndef SVL_GB300_H
#define SVL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SVL_OK               0
#define SVL_ERR_INVALID      1  /* bad argument / inconsistent model           */
#define SVL_ERR_CUDA         2  /* CUDA runtime error                          */
#define SVL_ERR_NONFINITE    3  /* NaN/Inf detected in the state               */
#define SVL_ERR_MAXITER      4  /* iterative solve hit its iteration cap       */
#define SVL_ERR_BREAKDOWN    5  /* PCG breakdown (p.Ap <= 0)                   */
#define SVL_ERR_UNSUPPORTED  6  /* valid model the GPU path does not cover     */
#define SVL_ERR_NOMEM        7  /* device allocation failed                    */
#define SVL_ERR_NODEVICE     8  /* no CUDA device / extension not usable       */

/* ---- element and material kinds --------------------------------------- */
/* Element classes (RP/04-Elements/06-Quadrilateral/lin2DQuad4.cpp,
 * RP/04-Elements/10-Hexahedron/lin3DHexa8.cpp). */
#define SVL_ELEM_LIN2DQUAD4   1
#define SVL_ELEM_LIN3DHEXA8   2

/* Material classes and the layout of their 8-double parameter rows.
 *   ELASTIC2DPLANESTRAIN (RP/02-Materials/01-Linear/Elastic2DPlaneStrain.cpp:5-27)
 *   ELASTIC3DLINEAR      (RP/02-Materials/01-Linear/Elastic3DLinear.cpp:5-29)
 *       param = {E, nu, rho, 0, 0, 0, 0, 0}
 *   PLASTICPLANESTRAINJ2 (RP/02-Materials/02-NonLinear/PlasticPlaneStrainJ2.cpp:6-52)
 *   PLASTIC3DJ2          (RP/02-Materials/02-NonLinear/Plastic3DJ2.cpp:6-52)
 *       param = {K, G, rho, H, beta, SigmaY, 0, 0}                         */
#define SVL_MAT_ELASTIC2DPLANESTRAIN  1
#define SVL_MAT_ELASTIC3DLINEAR       2
#define SVL_MAT_PLASTICPLANESTRAINJ2  3
#define SVL_MAT_PLASTIC3DJ2           4
#define SVL_MAT_NPARAM                8

/* ---- pre-processed model ---------------------------------------------- */
/* The content of one SVL partition file (PP/Core/SeismoVLAB.py:79-103, parsed
 * by RP/12-Utilities/Driver.hpp:1981-2045), already converted to arrays.
 * Nodes are listed in ascending node-tag order and elements in ascending
 * element-tag order: that order is the reference's std::map iteration order
 * and therefore its assembly (summation) order.                           */
typedef struct svl_model_desc {
    int32_t ndim;              /* 2 or 3                                       */
    int32_t nnode;
    int32_t ndof;              /* dofs per node (2 for Q4, 3 for H8)            */
    const double*  coords;     /* [nnode][ndim]                                */
    const int32_t* totaldof;   /* [nnode][ndof] total-dof numbers               */
    const int32_t* freedof;    /* [nnode][ndof] >=0 free, -1 restrained, <-1 constrained */
    int32_t ntotal;            /* number of total dofs                          */
    int32_t nfree;             /* number of free dofs                           */
    /* Constraints (RP/01-Node/Constraint.cpp; T rows built as in
     * RP/06-Mesh/Mesh.cpp:328-383): slave total dof <- sum factor * master free dof. */
    int32_t nconstraint;
    const int32_t* con_slave;  /* [nconstraint] total dof of the slave          */
    const int32_t* con_ptr;    /* [nconstraint+1] CSR into con_master/factor    */
    const int32_t* con_master; /* free dofs of the masters                      */
    const double*  con_factor; /* combination factors                           */
    /* Elements: one class per model.                                          */
    int32_t elem_type;         /* SVL_ELEM_*                                    */
    int32_t nelem;
    const int32_t* conn;       /* [nelem][nen] node positions (0-based into node arrays) */
    const int32_t* elem_mat;   /* [nelem] index into the material table        */
    const double*  elem_thickness; /* [nelem] (Q4 only) or NULL for 1.0         */
    int32_t nmat;
    const int32_t* mat_type;   /* [nmat] SVL_MAT_*                              */
    const double*  mat_param;  /* [nmat][SVL_MAT_NPARAM]                        */
    int32_t lumped;            /* 1: row-sum lumped mass (massform LUMPED)      */
    const double*  node_mass;  /* [ntotal] extra nodal masses, or NULL          */
    /* Rayleigh damping of each element (Dampings "Rayleigh", Driver.hpp:1375-1400):
     * C_e = am M_e + ak K0_e with K0 the initial stiffness (lin2DQuad4.cpp:322-372,
     * lin3DHexa8.cpp).  [nelem][2] = {am, ak}, or NULL for undamped elements. */
    const double*  elem_rayleigh;
    /* Perfectly matched layers (PML2DQuad4 / PML3DHexa8, Driver.hpp:1203-1220,
     * 1288-1306).  The nodes of PML elements carry 5 (2D: ux uy s11 s22 s12) or
     * 9 (3D: ux uy uz s11 s22 s33 s12 s23 s13) dofs; `ndof` is then the row
     * stride of totaldof/freedof and node_ndof gives each node's count.  Solid
     * elements use the first ndim dofs of their nodes (lin2DQuad4.cpp:130-147),
     * PML elements all of them (PML2DQuad4.cpp:130-147).  Served by svl_xnm_*. */
    const int32_t* node_ndof;       /* [nnode], or NULL: every node has ndof dofs   */
    const int32_t* elem_pml;        /* [nelem] 1 for a PML element, or NULL         */
    const double*  elem_pml_param;  /* [nelem][3 + 2 ndim]: n, L, R, x0[ndim], npml[ndim] */
    /* Lysmer dashpots: ZeroLength1D elements with a Viscous1DLinear material
     * (RP/04-Elements/01-Zero/ZeroLength1D.cpp:210-228, Driver.hpp:602-607,
     * 1072-1078): C_e = eta a a^T with a = (-1, +1) on the direction `dir` of
     * the element's two nodes; no mass, no stiffness and no internal force (the
     * material's elastic stress is 0).  Listed in element-tag order.         */
    int32_t ndashpot;
    const int32_t* dashpot_dof;     /* [ndashpot][2] total dofs (node 1, node 2) */
    const double*  dashpot_eta;     /* [ndashpot] damping coefficients          */
} svl_model_desc;

/* ---- loads -------------------------------------------------------------- */
/* Time series are the reference's "TimeSeries" functions (Driver.hpp:1514-1527).
 * A force entry adds coef * series[s][k] to total dof `force_dof` at step k
 * (series[s][k] = 0 past the end; the reference indexes without a check,
 * RP/05-Loads/Load.cpp:69-71).  Point loads (Assembler.cpp:334-350) become one
 * entry per loaded dof with coef = combination factor * direction; element body
 * loads (Assembler.cpp:439-459) become one entry per element dof with coef =
 * factor * (rho * integral of H^T dir), see svl_element_body_force.
 * Support motions (Assembler.cpp:493-532, Node.cpp:228-247): dof `sm_dof`
 * follows factor * series[s][k] (series[s][0] past the end).                */
typedef struct svl_load_desc {
    int32_t nseries;
    const int32_t* series_ptr;  /* [nseries+1] offsets into series_val          */
    const double*  series_val;
    int32_t nforce;
    const int32_t* force_dof;
    const int32_t* force_series;
    const double*  force_coef;
    int32_t nsupport;
    const int32_t* sm_dof;
    const int32_t* sm_series;
    const double*  sm_factor;
    /* Domain-reduction loads (ELEMENTLOAD "GENERALWAVE", Driver.hpp:1669-1722;
     * Assembler.cpp:460-478).  Every entry adds, at step k, factor times
     * M~ A_o + C~ V_o + K~ U_o of its element (lin2DQuad4.cpp:564-614,
     * lin3DHexa8.cpp:661-718): the element matrices with the blocks between two
     * boundary dofs and between two exterior dofs set to zero, and U_o, V_o, A_o
     * the free-field motion of the element's nodes at row k, negated at
     * exterior nodes as the run-process does when it reads the files.        */
    int32_t ndrm;
    const int32_t* drm_elem;        /* [ndrm] element positions, in load-list order        */
    const double*  drm_factor;      /* [ndrm] combination factor of the entry's load       */
    int32_t drm_nt;                 /* rows of every node's motion                         */
    const int32_t* drm_node_row;    /* [nnode] block of the node in drm_motion, -1 if none */
    const int32_t* drm_node_ext;    /* [nnode] 1 exterior node, 0 boundary node            */
    const double*  drm_motion;      /* [blocks][drm_nt][3 ndim] u[ndim] v[ndim] a[ndim]   */
} svl_load_desc;

/* ---- page-locked host memory ---------------------------------------------- */
/* History buffers handed to the *_run calls are copied into with DMA; when
 * they are page-locked the copies run at full link speed and overlap the
 * stepping.  Returns NULL on failure.  No counterpart in the reference. */
void* svl_host_alloc(size_t bytes);
void  svl_host_free(void* p);

/* ---- library info ------------------------------------------------------- */
const char* svl_version(void);
const char* svl_last_error(void);
int svl_device_info(int* device_count, int* sm_count, int* cc_major, int* cc_minor);
/* Selects the CUDA device for handles created afterwards on this host thread
 * (one process per GPU: pass the local rank).  No counterpart in the
 * reference, whose ranks are MPI processes without a device. */
int svl_set_device(int device);

/* ---- structured mesh generator + PlainScheme numbering ------------------ */
/* Mirrors PP/Method/Builder.py makeDomainArea (244-418) / makeDomainVolume
 * (57-242): nodes numbered x-fastest, Q4 conn (i,j),(i+1,j),(i+1,j+1),(i,j+1),
 * H8 conn as Builder.py:167-183, then PP/Core/Numberer.py PlainScheme
 * (185-233) for total/free dof numbers.
 * fix_mask[f] restrains dof bits on face f (0:xmin 1:xmax 2:ymin 3:ymax
 * 4:zmin 5:zmax; bit d = dof d).  Faces are applied in that order.  With
 * periodic_x != 0 every unrestrained dof of a node on xmax is tied by an
 * EQUAL constraint (factor 1) to the node on xmin at the same y(,z); the
 * constraints are numbered in ascending slave-node order, dof-minor.      */
typedef struct svl_grid_spec {
    int32_t ndim;
    int32_t ne[3];
    double  h[3];
    double  origin[3];
    int32_t fix_mask[6];
    int32_t periodic_x;
} svl_grid_spec;

int svl_grid_sizes(const svl_grid_spec* spec, int32_t* nnode, int32_t* nelem,
                   int32_t* ntotal, int32_t* nfree, int32_t* nconstraint);
/* Output arrays sized from svl_grid_sizes (nen = 4 for 2D, 8 for 3D; each
 * constraint has exactly one master, so con_master/con_factor have
 * nconstraint entries and con_ptr nconstraint+1). */
int svl_grid_build(const svl_grid_spec* spec, double* coords, int32_t* totaldof,
                   int32_t* freedof, int32_t* conn, int32_t* con_slave,
                   int32_t* con_ptr, int32_t* con_master, double* con_factor);

/* Nodal load vector of a unit-amplitude element body load, rho * int(H^T q)
 * over the element (lin2DQuad4.cpp:528-560 / lin3DHexa8 ComputeBodyForces).
 * fe has nen*ndim entries. */
int svl_element_body_force(const svl_model_desc* model, int32_t elem,
                           const double* q, double* fe);

/* Row-sum lumped mass on total dofs, assembled in element-tag order with the
 * mass tolerance filter (Assembler.cpp:48-67, 623-697). */
int svl_lumped_mass(const svl_model_desc* model, double mtol, double* mass_total);

/* ---- explicit central difference (CentralDifference + Linear) ---------- */
/* Replaces, for lumped mass without damping:
 *   CentralDifference::Initialize / ComputeEffectiveForce /
 *   ComputeEffectiveStiffness / ComputeSupportMotionVector / ComputeNewStep
 *     (RP/10-Integrators/02-CentralDifference/CentralDifference.cpp:36-71,
 *      124-151, 190-231),
 *   Linear::ComputeNewIncrement (RP/09-Algorithms/01-Linear/Linear.cpp:22-56),
 *   EigenSolver::SolveSystem on the diagonal K = M/dt^2 (EigenSolver.cpp:19-59),
 *   Algorithm::UpdateStatesIncrements (RP/09-Algorithms/Algorithm.cpp:18-56),
 *   Assembler::ComputeInternalForceVector / ComputeExternalForceVector /
 *     ComputeSupportMotionIncrement (RP/07-Assembler/Assembler.cpp:240-269,
 *     291-532),
 *   and the element/material calls under them.                              */
#define SVL_PREC_FP64   0   /* everything in FP64 (the plain form)             */
#define SVL_PREC_MIXED  1   /* TF32 hi/lo element forces with FP32 accumulation;
                               displacement state as a compensated FP32 pair */

typedef struct svl_cd_opts {
    double  dt;
    double  ftol;        /* force assembly tolerance (JSON integrator ftol, 1e-12) */
    double  mtol;        /* mass assembly tolerance  (JSON integrator mtol, 1e-12) */
    int32_t precision;   /* SVL_PREC_*                                          */
    int32_t check_every; /* NaN/Inf scan every n steps (0 = never)               */
} svl_cd_opts;

typedef struct svl_cd svl_cd;

int  svl_cd_create(const svl_model_desc* model, const svl_load_desc* loads,
                   const svl_cd_opts* opts, svl_cd** out);
/* Initial conditions on total dofs (host arrays, NULL = zero); sets
 * Up = U - dt V + dt^2/2 A (CentralDifference.cpp:61). */
int  svl_cd_set_initial(svl_cd* cd, const double* U0, const double* V0, const double* A0);
/* Advances steps k_first .. k_first+nsteps-1 (the reference's loop index k,
 * DynamicAnalysis.cpp:36).  If U_hist is not NULL it receives the total
 * displacement after every step, [nsteps][ntotal], copied to the host. */
int  svl_cd_run(svl_cd* cd, int32_t k_first, int32_t nsteps, double* U_hist);
/* which: 0 = U, 1 = V, 2 = A (total dofs, host copy). */
int  svl_cd_get(svl_cd* cd, int32_t which, double* out);
/* Reaction forces after step k (the step just run), as DynamicAnalysis::
 * UpdateDomain stores them (DynamicAnalysis.cpp:128-150) through
 * CentralDifference::ComputeReactionForce (CentralDifference.cpp:156-171):
 * R = m A + sum over the elements with a fixed node (a node with a free-dof
 * entry of -1) of Fint_e + C_e V_e + M_e A_e, minus Fext(k), on the dofs of
 * fixed nodes; zeros elsewhere (Node::GetReaction).  R: [ntotal] host array. */
int  svl_cd_reaction(svl_cd* cd, int32_t k, double* R);
/* Element responses after the last step for the ELEMENT recorders
 * (Recorder.cpp:272-323) of the listed element positions: response 0 =
 * material strain at each Gauss point (Element::GetStrain: elastic the
 * engineering strain, J2 the material's strain with tensor shears), 1 =
 * material total stress at each Gauss point (GetStress), 2 = internal force
 * (ComputeInternalForces, NC values), 3 = strain rate (GetStrainRate: zeros for
 * these materials).  out: [nlist][ngp][3 (2D) or 6 (3D)] or [nlist][NC]. */
int  svl_cd_element_response(svl_cd* cd, int32_t response, int32_t nlist, const int32_t* elems, double* out);
/* Device pointer of U / V / A (valid until the next svl_cd_run). */
int  svl_cd_device_ptr(svl_cd* cd, int32_t which, const double** dptr);
/* Number of kernel launches the last svl_cd_run issued. */
int  svl_cd_launch_count(svl_cd* cd, int64_t* launches);
/* svl_cd_run without history, bracketed by CUDA events recorded on the
 * handle's own stream; *ms = elapsed device time of the nsteps.  No
 * counterpart in the reference (measurement hook). */
int  svl_cd_run_timed(svl_cd* cd, int32_t k_first, int32_t nsteps, float* ms);
/* Runs nsteps launching every kernel individually with CUDA events between
 * them; ms_kernel[i] receives the summed device time of kernel kind i
 * (0 = element forces, 1 = node gather/update, 2 = residual, 3 = free-dof
 * solve, 4 = update; unused kinds stay 0).  No counterpart in the reference. */
int  svl_cd_profile(svl_cd* cd, int32_t k_first, int32_t nsteps, double* ms_kernel);
int  svl_cd_sync(svl_cd* cd);
void svl_cd_destroy(svl_cd* cd);

/* ---- structured grids: mixed-precision batched central difference ------ */
/* The same step as svl_cd_run for `ninst` instances of one uniform
 * lin3DHexa8 grid (svl_grid_build layout, Elastic3DLinear materials, lumped
 * mass, point/body loads, restraints; no constraints or support motion),
 * advanced together by one fused kernel per step.  The element force is the
 * tensor-core contraction F_e = lambda_e (K_lambda u_e) + mu_e (K_mu u_e):
 * the 48 x 24 stacked reference matrix times the 24 x elements displacement
 * block, the displacements split into TF32 hi + lo parts and the reference
 * matrix exact in TF32 for cubes (integers times h/72; other shapes: also
 * split, three products) with FP32 accumulation in TMEM.  The displacement state is a compensated pair of FP32 numbers per
 * dof (hi + lo, about 48 significant bits, updated with error-free TwoSum
 * transformations), not FP64; results state their error against the FP64
 * path (<= 1e-5 relative L2 over the history in the tests).  Reference summation order
 * at every node is kept; the assembler's force tolerance filter is not
 * applied on this path.  `models` and `loads` are arrays of ninst
 * descriptors (one per instance, same grid).  precision must be
 * SVL_PREC_MIXED.  Replaces the same reference functions as svl_cd_create /
 * svl_cd_run for models of that shape. */
typedef struct svl_cdx svl_cdx;
int  svl_cdx_create(const svl_grid_spec* grid, int32_t ninst, const svl_model_desc* models,
                    const svl_load_desc* loads, const svl_cd_opts* opts, svl_cdx** out);
/* Ensembles of uneven grids: instance b lives on grids[b] (every grid with
 * the element size of grids[0]; models and loads as for svl_cdx_create on
 * their own grids; no PML layers, support motion or domain reduction).  The
 * instances are embedded in the grid that bounds them all (restrained nodes
 * and elements without stiffness or mass fill the rest, so the instances'
 * results do not change) and the fused kernel schedules only the tiles that
 * meet an instance's own nodes.  set_initial / get take each instance's own
 * total dofs; run's history is [nsteps][sum of the instances' ntotal], the
 * instances one after the other.  No counterpart in the reference (an
 * ensemble there is one process per model). */
int  svl_cdx_create_ensemble(const svl_grid_spec* grids, int32_t ninst, const svl_model_desc* models,
                             const svl_load_desc* loads, const svl_cd_opts* opts, svl_cdx** out);
/* Initial conditions of instance `inst` (total dofs, NULL = zero). */
int  svl_cdx_set_initial(svl_cdx* cdx, int32_t inst, const double* U0, const double* V0, const double* A0);
/* Steps k_first .. k_first+nsteps-1 of every instance; U_hist (host, or
 * NULL) receives [nsteps][ninst][ntotal] displacements (ensembles: the
 * instances' own ntotal one after the other). */
int  svl_cdx_run(svl_cdx* cdx, int32_t k_first, int32_t nsteps, double* U_hist);
/* svl_cdx_run without history bracketed by CUDA events on the handle's
 * stream (measurement hook, no counterpart in the reference). */
int  svl_cdx_run_timed(svl_cdx* cdx, int32_t k_first, int32_t nsteps, float* ms);
/* which: 0 = U, 1 = V, 2 = A of instance `inst` after the last step. */
int  svl_cdx_get(svl_cdx* cdx, int32_t inst, int32_t which, double* out);
int  svl_cdx_launch_count(svl_cdx* cdx, int64_t* launches);
/* Persistent-grid size of the fused step kernel: `ctas` CTAs (one per SM at
 * most; 0 = one per SM, the default), each looping over the node tiles
 * blockIdx.x, blockIdx.x + ctas, ...  Fewer CTAs give each one more tiles
 * (a test and tuning hook: the results do not depend on it).  No
 * counterpart in the reference. */
int  svl_cdx_set_ctas(svl_cdx* cdx, int32_t ctas);
/* Runs nsteps (no history) with CUDA events between the kernels of each
 * step; ms_kernel[i] receives the summed device time of kernel i: 0 = the
 * fused tensor-core step, then the PML band's 1 = element forces on the
 * displacement rows, 2 = displacement-row update, 3 = element forces on the
 * stress rows, 4 = stress-row update (0 without a band).  No counterpart in
 * the reference (measurement hook). */
int  svl_cdx_profile(svl_cdx* cdx, int32_t k_first, int32_t nsteps, double* ms_kernel);
int  svl_cdx_get_ctas(svl_cdx* cdx, int32_t* ctas);
/* Schedule of a step: choice[0] persistent CTAs of the fused kernel (0 = one
 * per SM), choice[1] the order in which the CTAs walk the node tiles (0
 * natural: x fastest, then y, z, instance; 1 instances interleaved; 2 y
 * fastest; 3 blocks of 2 x 2 x 2 tiles), choice[2] threads per block of the
 * PML band's element kernels (128 or 256), choice[3] 1 = the band's stream
 * has the higher priority.  Results do not depend on it.  No counterpart in
 * the reference. */
int  svl_cdx_set_schedule(svl_cdx* cdx, const int32_t* choice);
int  svl_cdx_get_schedule(svl_cdx* cdx, int32_t* choice);
/* Autotuner: times nsteps steps (from k_first on, after two warm-up steps) of
 * every schedule in a small grid (eight CTA counts from one per SM down to
 * half of the SMs, the four tile orders and, with a PML band, both block
 * sizes and priorities), times the four fastest again over 4 * nsteps steps,
 * keeps the fastest of those and returns it in choice[4] (*ms_best: its time
 * per step in the second timing).  The steps advance the state: set the
 * initial conditions again before the run that counts. */
int  svl_cdx_tune(svl_cdx* cdx, int32_t k_first, int32_t nsteps, int32_t* choice, float* ms_best);
void svl_cdx_destroy(svl_cdx* cdx);

/* ---- implicit Newmark (average acceleration), Linear algorithm --------- */
/* NewmarkBeta with beta = 1/4, gamma = 1/2 (ExtendedNewmarkBeta with G = 0)
 * and the Linear algorithm: one solve of the effective stiffness per step.
 * Replaces
 *   NewmarkBeta::Initialize / ComputeNewStep / ComputeEffectiveForce /
 *     ComputeEffectiveStiffness (RP/10-Integrators/03-Newmark/
 *     NewmarkBeta.cpp:35-66, 117-141, 198-235),
 *   Linear::ComputeNewIncrement (RP/09-Algorithms/01-Linear/Linear.cpp:22-56),
 *   and the effective-stiffness solve of EigenSolver::SolveSystem /
 *     PetscSolver KSP CG (RP/11-Solvers/01-Direct/EigenSolver.cpp:19-59,
 *     RP/11-Solvers/02-Iterative/PetscSolver.cc:53-150).
 * The effective stiffness T^T (K + 4/dt^2 M) T is never assembled: the
 * Jacobi-preconditioned conjugate gradient applies it element by element
 * (the stiffness action of every element, summed per node in ascending
 * element order, plus the lumped mass), in FP64, and stops on the TRUE
 * relative residual |Feff - Keff du| / |Feff| <= pcg_tol.  Dot products are
 * reduced in a fixed order: runs are bitwise reproducible.
 * With SVL_ALGO_NEWTON the step iterates NewtonRaphson::ComputeNewIncrement:
 * effective force from the current element states, a PCG solve with the
 * consistent tangent (J2 elements: the tangent of their last return mapping,
 * as Material::GetTangentStiffness returns it), the states updated from
 * U + dU, until the chosen convergence test passes or `maxit` iterations.
 * Covered: elastic materials (both algorithms), J2 materials (Newton),
 * lumped or consistent mass (massform CONSISTENT: the element mass action in
 * the operator and the effective force), Rayleigh damping (am with the
 * element's mass, ak with its initial stiffness), ZeroLength1D dashpots,
 * EQUAL constraints (T^T Keff T) and support motion (T^T Keff SM of step
 * k - 1, NewmarkBeta.cpp:180-194), domain-reduction loads with a lumped
 * elastic layer; other models return SVL_ERR_UNSUPPORTED. */
#define SVL_ALGO_LINEAR     0   /* Linear.cpp:22-56: one solve per step           */
#define SVL_ALGO_NEWTON     1   /* NewtonRaphson.cpp:24-75: tangent iterations    */
#define SVL_PRECOND_JACOBI  0
#define SVL_PRECOND_LEARNED 1   /* see svl_nm_train_preconditioner                */
/* svl_nm_opts.integrator.  SVL_NM_CENTRAL_DIFFERENCE: CentralDifference with
 * an effective stiffness K = M/dt^2 + C/2dt that is not diagonal -- a
 * consistent mass (massform CONSISTENT) and/or stiffness-proportional
 * Rayleigh damping (ak != 0) -- which the reference factorises once and
 * solves every step (CentralDifference.cpp:64-70, 122-152, 204-231).  Here the
 * same Jacobi-PCG applies K element by element: sum_e (1/dt^2 + am_e/2dt)
 * M_e p_e + (ak_e/2dt) K0_e p_e plus the nodal masses / dt^2, stopping on
 * the true relative residual <= pcg_tol.  Step: Feff = Fext - Fint +
 * (M/dt^2 - C/2dt)(U - Up), solve, V = (U + dU - Up)/2dt, A = (dU - U +
 * Up)/dt^2, Up = U, U += dU.  Covered: elastic and J2 materials (the
 * element update from U + T du once per step, as the diagonal path), EQUAL
 * constraints (T^T K T, Feff = T^T R), support motion (dU = T du + SM(k),
 * Feff -= T^T K SM(k)), ZeroLength1D dashpots (their C in K); not
 * domain-reduction loads (SVL_ERR_UNSUPPORTED); algorithm must be
 * SVL_ALGO_LINEAR and precond Jacobi.  A lumped mass without ak is the
 * diagonal path of svl_cd_create. */
#define SVL_NM_NEWMARK            0
#define SVL_NM_CENTRAL_DIFFERENCE 1
typedef struct svl_nm_opts {
    double  dt;
    double  ftol;        /* force assembly tolerance (as svl_cd_opts)             */
    double  mtol;        /* mass assembly tolerance                               */
    double  pcg_tol;     /* relative true-residual tolerance of each solve        */
    int32_t pcg_maxit;   /* iteration cap per solve (SVL_ERR_MAXITER past it)     */
    int32_t precond;     /* SVL_PRECOND_JACOBI or SVL_PRECOND_LEARNED             */
    int32_t algorithm;   /* SVL_ALGO_LINEAR or SVL_ALGO_NEWTON                    */
    int32_t maxit;       /* Newton: iterations per step (the algorithm's nstep)   */
    double  cnvgtol;     /* Newton: convergence tolerance (cnvgtol; 0 = always
                            `maxit` iterations)                                   */
    int32_t cnvgtest;    /* Newton: 4 relative unbalanced force (the reference's
                            default), 5 relative displacement increment
                            (Algorithm.cpp:122-188)                               */
    int32_t single_inner;/* 1: the inner iterations of each solve apply the
                            effective stiffness in single precision (elastic
                            models without damping or constraints; others
                            ignore it); every answer is confirmed with the FP64
                            operator -- the true residual -- and the solve
                            restarts from it until pcg_tol holds, so the result
                            keeps the FP64 tolerance.  0: FP64 throughout.      */
    int32_t integrator;  /* SVL_NM_NEWMARK (0) or SVL_NM_CENTRAL_DIFFERENCE     */
} svl_nm_opts;

typedef struct svl_nm svl_nm;
int  svl_nm_create(const svl_model_desc* model, const svl_load_desc* loads,
                   const svl_nm_opts* opts, svl_nm** out);
/* Initial conditions on total dofs (host arrays, NULL = zero). */
int  svl_nm_set_initial(svl_nm* nm, const double* U0, const double* V0, const double* A0);
/* Steps k_first .. k_first+nsteps-1; U_hist as in svl_cd_run. */
int  svl_nm_run(svl_nm* nm, int32_t k_first, int32_t nsteps, double* U_hist);
/* svl_nm_run without history bracketed by CUDA events on the handle's
 * stream; *ms = elapsed time (measurement hook, no counterpart). */
int  svl_nm_run_timed(svl_nm* nm, int32_t k_first, int32_t nsteps, float* ms);
int  svl_nm_get(svl_nm* nm, int32_t which, double* out);
/* NewmarkBeta::ComputeReactionForce after step k (as svl_cd_reaction). */
int  svl_nm_reaction(svl_nm* nm, int32_t k, double* R);
/* Element responses after the last step (as svl_cd_element_response). */
int  svl_nm_element_response(svl_nm* nm, int32_t response, int32_t nlist, const int32_t* elems, double* out);
/* Conjugate-gradient iterations summed over all solves, of the last solve,
 * and the last solve's true relative residual. */
int  svl_nm_stats(svl_nm* nm, int64_t* iters_total, int64_t* iters_last, double* rel_residual_last);
/* Newton iterations over all steps, of the last step, and the last step's
 * final convergence-test value. */
int  svl_nm_newton_stats(svl_nm* nm, int64_t* iters_total, int64_t* iters_last, double* residual_last);
int  svl_nm_launch_count(svl_nm* nm, int64_t* launches);
int  svl_nm_sync(svl_nm* nm);
void svl_nm_destroy(svl_nm* nm);

/* ---- ExtendedNewmarkBeta with PML (svl_xnm_*) ---------------------------- */
/* ExtendedNewmarkBeta (RP/10-Integrators/03-Newmark/ExtendedNewmarkBeta.cpp)
 * with the Linear or NewtonRaphson algorithm on a mesh of elastic or J2
 * lin2DQuad4/lin3DHexa8 solid elements (lumped mass, optional Rayleigh
 * damping with the initial stiffness) and elastic PML2DQuad4/PML3DHexa8
 * elements (5 / 9 dofs per node, consistent mass):
 *   Feff = Fext - Fint - G (Ubar + dt U + dt^2/6 V) + C V + M (4/dt V + A)  (:208-229)
 *   Keff = K + 4/dt^2 M + 2/dt C + dt/3 G                                   (:233-245)
 *   Feff -= T^T Keff SM(k)  (the increment of step k, :190-204)
 *   Ubar += dt U + dt/3 (dU + SM) + dt^2/6 V; U += dU + SM;
 *   A = 4/dt^2 dU - 4/dt V - A; V = 2/dt dU - V                             (:123-153)
 * Fint of a solid element from its state after the last solve (strain of
 * U + T dU), of a PML element K_e U_e (PML3DHexa8.cpp:716-742).  Newton
 * iterations (NewtonRaphson.cpp:24-75) repeat force, tangent solve and state
 * update with the accumulated dU; the effective force has no increment terms
 * (ExtendedNewmarkBeta.cpp:208-229), so only Fint follows the iterate.  With PML the effective
 * matrix is symmetric indefinite, so the solve is MINRES with the
 * D = |diag(Keff)| preconditioner, matrix-free on the GPU, stopped on the true
 * residual in the norm MINRES minimises, ||b - Keff du||_{D^-1} <= tol ||b||_{D^-1}
 * (displacement and stress rows differ by ~13 orders of magnitude).  The
 * reference solves the same system with SimplicialLDLT / MUMPS / PETSc
 * (EigenSolver.cpp:19-59). */
#define SVL_XNM_EXTENDED_NEWMARK 0  /* ExtendedNewmarkBeta.cpp (the formulas above)  */
#define SVL_XNM_NEWMARK          1  /* NewmarkBeta.cpp:117-235 on the same elements:
                                       Feff = Fext - Fint + M (4/dt V + A - 4/dt^2 dU)
                                              + C (V - 2/dt dU) - T^T Keff SM(k-1),
                                       Keff = K + 4/dt^2 M + 2/dt C (G is not used;
                                       the NEWMARK integrator of a PML model)     */
/* SVL_XNM_CENTRAL_DIFFERENCE: explicit central difference on a model with PML
 * layers -- a scheme of this library, for the CENTRALDIFFERENCE integrator of
 * a PML model.  The reference's CentralDifference applies no PML history
 * (CentralDifference.cpp:114-120) and keeps the PML mass consistent with a
 * negative stress block (PML3DHexa8.cpp:214-284), so its M/dt^2 + C/2dt is
 * sparse and indefinite.  Here the same element matrices M, C, K, G are
 * advanced explicitly: displacements at the integer steps, the PML stress
 * dofs S at the half steps (leapfrog); the N N blocks of the PML matrices are
 * row-sum lumped per node (diagonal on displacement dofs, one ns x ns block
 * per node on its stress dofs), the displacement-stress couplings act
 * through the element action, and ubar / Sbar integrate by the trapezoid /
 * midpoint rules:
 *   (Mu/dt^2 + Cu/2dt) du = Fext(k) - Fint_solid(u^k)
 *       - (C_uS sdot + K_uS smid + G_uS Sbar^k) - Ku u^k - Gu ubar^k
 *       + (Mu/dt^2 - Cu/2dt)(u^k - u^(k-1)),
 *   sdot = (S^(k+1/2) - S^(k-1/2))/dt, smid = (S^(k+1/2) + S^(k-1/2))/2;
 *   (Ms/dt^2 + Cs/2dt) dS = -(C_Su udot + K_Su umid + G_Su ubar^(k+1/2))
 *       - Ks S^(k+1/2) - Gs Sbar^(k+1/2) + (Ms/dt^2 - Cs/2dt)(S^(k+1/2) - S^(k-1/2)),
 *   udot = (u^(k+1) - u^k)/dt, umid = (u^(k+1) + u^k)/2.
 * Without PML elements it is the plain central difference.  Element forces
 * on displacement rows carry the force filter.  U on a PML node's stress
 * dofs holds S at the half step after U's time; V and A follow
 * CentralDifference.cpp:141-144 on every dof.  The Linear algorithm only;
 * constraints with one master per constrained displacement dof (the EQUAL
 * ties mergeDomain writes; the solve is T^T d T, diagonal), none on stress
 * dofs; no dashpots or domain-reduction loads; support motion on
 * displacement dofs; mass-proportional Rayleigh damping on solid elements;
 * tol and maxit are not used.  Stable below the lumped-mass step limit of
 * the solid region (measured: 0.9 h/Vp on 2D boxes). */
#define SVL_XNM_CENTRAL_DIFFERENCE 2
typedef struct svl_xnm svl_xnm;
typedef struct svl_xnm_opts {
    double  dt;
    double  ftol;        /* force assembly tolerance (1e-12)                       */
    double  mtol;        /* mass assembly tolerance (1e-12)                        */
    double  tol;         /* relative true-residual tolerance (D^-1 norm) of each solve */
    int32_t maxit;       /* MINRES iteration cap per solve (SVL_ERR_MAXITER past it) */
    int32_t algorithm;   /* SVL_ALGO_LINEAR or SVL_ALGO_NEWTON                    */
    int32_t newton_maxit;/* Newton: iterations per step (the algorithm's nstep)   */
    int32_t cnvgtest;    /* Newton: 4 relative unbalanced force, 5 relative
                            displacement increment (Algorithm.cpp:122-188)        */
    double  cnvgtol;     /* Newton: convergence tolerance (0 = always newton_maxit) */
    int32_t integrator;  /* SVL_XNM_EXTENDED_NEWMARK, SVL_XNM_NEWMARK or
                            SVL_XNM_CENTRAL_DIFFERENCE                          */
    int32_t single_inner;/* 1: the inner MINRES iterations apply the element
                            operators in single precision; every restart forms
                            the true residual with the double operator and the
                            stopping test is on it (iterative refinement)      */
} svl_xnm_opts;
int  svl_xnm_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_xnm_opts* opts,
                    svl_xnm** out);
/* U0, V0, A0, Ubar0: [ntotal] host arrays or NULL for zero. */
int  svl_xnm_set_initial(svl_xnm* x, const double* U0, const double* V0, const double* A0, const double* Ubar0);
/* Steps k_first .. k_first+nsteps-1; U_hist [nsteps][ntotal] host array or NULL. */
int  svl_xnm_run(svl_xnm* x, int32_t k_first, int32_t nsteps, double* U_hist);
/* which: 0 U, 1 V, 2 A, 3 Ubar (GetPMLHistoryVector); out [ntotal]. */
int  svl_xnm_get(svl_xnm* x, int32_t which, double* out);
/* Reaction forces after step k (as svl_cd_reaction) through ExtendedNewmarkBeta
 * / NewmarkBeta::ComputeReactionForce (ExtendedNewmarkBeta.cpp:158-172,
 * NewmarkBeta.cpp:148-162): PML elements with a fixed node add K_e u_e +
 * C_e v_e + M_e a_e over all their dofs (PML3DHexa8.cpp:746-767, no history
 * term), so the stress dofs of fixed PML nodes get reactions too.  Not for
 * the explicit PML scheme (SVL_ERR_UNSUPPORTED).  R: [ntotal] host array. */
int  svl_xnm_reaction(svl_xnm* x, int32_t k, double* R);
int  svl_xnm_stats(svl_xnm* x, int64_t* iters_total, int64_t* iters_last, double* res_last);
/* Newton iterations over all steps, of the last step, and the last step's
 * final convergence-test value (1 iteration per step with Linear). */
int  svl_xnm_newton_stats(svl_xnm* x, int64_t* iters_total, int64_t* iters_last, double* residual_last);
void svl_xnm_destroy(svl_xnm* x);

/* ---- learned preconditioner (no counterpart in the reference) ----------- */
/* For hexahedral models whose nodes form a lattice (svl_grid_build meshes and
 * any other mesh with one node per point of an nx x ny x nz lattice), the
 * solve can be preconditioned by a small 3D convolutional network on that
 * lattice: z = D^-1/2 (r_hat + net(r_hat, rho r_hat)), r_hat = D^-1/2 r,
 * D = diag(K_eff), rho = (4/dt^2 m) / D; four 3x3x3 convolutions
 * 6 -> 16 -> 16 -> 16 -> 3 with ReLU between them, FP32.  The solve is then a
 * flexible conjugate gradient (each direction K_eff-orthogonalised against
 * the previous one).  Jacobi-PCG is both the fallback and the yardstick: a solve
 * that has used as many iterations as the last plain Jacobi-PCG solve without
 * reaching pcg_tol continues with Jacobi-PCG from where it stands, and every
 * solve ends on the true FP64 residual.  The network is trained on the GPU
 * by the library's own forward and backward kernels (Adam, fixed-order
 * reductions). */
typedef struct svl_nn_train_opts {
    int32_t  solve_steps;  /* Newmark steps advanced with Jacobi-PCG whose CG
                              iterates give (r_k, e_k = x* - x_k) pairs        */
    int32_t  record_every; /* record every n-th CG iterate (at most 12 a solve) */
    int32_t  n_synthetic;  /* pairs (e, r = K_eff e), e random with 0..5
                              smoothing sweeps of the scaled operator          */
    int32_t  iters;        /* Adam iterations                                  */
    int32_t  batch;        /* pairs per iteration                              */
    float    lr;           /* Adam step (decays to 1/4 at 60 %, 1/20 at 85 %) */
    uint64_t seed;
    int32_t  max_sweeps;   /* synthetic pair i gets i % (max_sweeps + 1)
                              smoothing sweeps (0 = the default, 5)           */
    int32_t  crop;         /* > 0: every sample is a random crop x crop x crop
                              window of a pair, the loss masked 4 nodes inside
                              window faces that lie inside the lattice (the
                              network's reach); 0: the whole lattice          */
} svl_nn_train_opts;
/* Runs the solve_steps steps k_first.. (they advance the state), generates
 * the synthetic pairs, trains, and switches the handle to
 * SVL_PRECOND_LEARNED.  *loss = mean relative squared error of the trained
 * preconditioner on its pairs over the last tenth of the iterations. */
int  svl_nm_train_preconditioner(svl_nm* nm, int32_t k_first, const svl_nn_train_opts* opts, float* loss);
int  svl_nm_set_preconditioner(svl_nm* nm, int32_t precond);
/* Number of network weights; get (w_out) and/or set (w_in) them.  Layout:
 * layer by layer, [cout][cin][27] with tap t = 9 (dz+1) + 3 (dy+1) + (dx+1). */
int  svl_nn_num_weights(void);
int  svl_nm_preconditioner_weights(svl_nm* nm, float* w_out, const float* w_in);
/* Solves that used the learned preconditioner, how many of them fell back to
 * Jacobi-PCG, and the iteration count of the last plain Jacobi-PCG solve. */
int  svl_nm_precond_stats(svl_nm* nm, int64_t* learned_solves, int64_t* fallbacks, int64_t* jacobi_ref_iters);
/* Node lattice dims (nx, ny, nz), zeros if the model is not a lattice. */
int  svl_nm_lattice(svl_nm* nm, int32_t* dims);
/* Test hook: loss sum and weight gradient of one sample on the device.  x, t:
 * host grids [3][nz][ny][nx] of r_hat and e_hat; grad: svl_nn_num_weights(). */
int  svl_nm_nn_loss_grad(svl_nm* nm, const float* x, const float* t, float* loss, float* grad);
/* Network output y for a host r_hat grid x (both [3][nz][ny][nx]) through the
 * FP32 CUDA-core kernels (path 0) or the BF16 tensor-core kernels (path 1).
 * Test hook. */
int  svl_nm_nn_forward(svl_nm* nm, const float* x, float* y, int32_t path);
/* Inference path of the learned preconditioner inside the solve: 1 = BF16
 * tensor cores (tcgen05, the default), 0 = FP32 CUDA cores (the training
 * kernels). */
int  svl_nm_nn_set_path(svl_nm* nm, int32_t path);
/* Test hook: the rho feature grid and the free-dof mask grid, [3][nz][ny][nx]. */
int  svl_nm_nn_grids(svl_nm* nm, float* rho, float* mask);

/* ---- PML elements ---------------------------------------------------------- */
/* Element action of PML2DQuad4 (5 dofs per node: ux uy s11 s22 s12) and
 * PML3DHexa8 (9 dofs per node: ux uy uz s11 s22 s33 s12 s23 s13) for a batch
 * of elements, on the GPU:
 *   y_e = coef[0] M_e u0_e + coef[1] C_e u1_e + coef[2] K_e u2_e + coef[3] G_e u3_e
 * with M, C, K, G the element mass, damping, stiffness and PML-history
 * matrices of PML2DQuad4.cpp:233-470 / PML3DHexa8.cpp:214-712 (G is empty
 * in 2D), applied at the Gauss points without forming them.  coef[2] = 1,
 * others 0 gives ComputeInternalForces (K u, :474-494 / :716-742).
 *   X      [nelem][nen][ndim] node coordinates in the element's node order
 *   mat    [nelem][3] E, nu, rho (Elastic2DPlaneStrain / Elastic3DLinear)
 *   thick  [nelem] thickness (2D) or NULL for 1
 *   par    [nelem][3 + 2 ndim] m, L, R, x0[ndim], n[ndim] (the element's
 *          PML parameters in the order of the reference constructors)
 *   u      [4][nelem][nc] input vectors (a block may hold anything when its
 *          coefficient is 0), y [nelem][nc] output; host arrays.
 * No counterpart in the reference beyond the element functions named. */
int  svl_pml_element_action(int32_t ndim, int32_t nelem, const double* X, const double* mat,
                            const double* thick, const double* par, const double* coef,
                            const double* u, double* y);

/* ---- stepping without device allocation -------------------------------- */
/* No counterpart in the reference: SVL allocates all of its (host) memory
 * freely.  Some callers of this library cannot let it call cudaMalloc or
 * cudaFree once their time loop runs: applications that hand out all device
 * memory from their own pool (a framework's caching allocator, or a solver
 * that reserved the remaining HBM for itself) and forbid third-party code
 * from allocating, because those calls synchronise the whole device and can
 * fail or fragment the pool in the middle of a simulation.  svl_cd_run may
 * allocate on first use (it instantiates a CUDA graph, and a device history
 * buffer when a history is requested); svl_cd_run_noalloc never allocates.
 *
 * It advances the handle's state exactly like svl_cd_run(cd, k_first,
 * nsteps, NULL) -- the same launch sequence per step (element forces,
 * domain-reduction forces when the loads have them, then the node kernels),
 * the same results -- but the per-step element force block lives in one
 * library-wide static device array of SVL_NOALLOC_SCRATCH_BYTES instead of
 * the handle's own buffer, and the kernels are launched directly (no graph).
 * Every GPU that loads the library holds that array until the process exits.
 * svl_cd_launch_count then reports this call's kernels (one step-index
 * set-up kernel plus the per-step kernels).
 *
 * Limit: nelem * nen * ndof * 8 bytes must fit in SVL_NOALLOC_SCRATCH_BYTES
 * (8 MiB: at most 43690 lin3DHexa8 or 131072 lin2DQuad4 elements); larger
 * models are rejected with SVL_ERR_UNSUPPORTED.
 * Output: if d_U_out is not NULL it must be a device buffer of ntotal
 * doubles owned by the caller; it receives U after the last step.
 * The call is asynchronous on the handle's stream (svl_cd_sync waits) and
 * does not scan for NaN/Inf.
 * Set-up: the first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device made current for the lookup);
 * make that first call before any stream capture.
 * Sharing: all calls in the process share the one array and it keeps the
 * last call's contents.  Each step overwrites every entry it later reads,
 * so nothing has to start at zero, but calls that overlap on the GPU
 * (different streams, handles or host threads) race on the array and must
 * be serialised by the caller. */
#define SVL_NOALLOC_SCRATCH_BYTES (8u << 20)
int  svl_cd_run_noalloc(svl_cd* cd, int32_t k_first, int32_t nsteps, double* d_U_out);

#ifdef __cplusplus
}
#endif
#endif /* SVL_GB300_H */
