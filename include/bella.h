/*
 * bella.h -- C ABI of libbella_gb300.so, the GB300 (sm_103a) implicit nodal
 * pressure projection of pyBELLA.
 *
 * Plain C: device pointers, sizes, doubles and an opaque workspace.  No
 * framework types cross this boundary.  Every call returns an int status
 * (BELLA_OK == 0); no exceptions cross the ABI.  `stream` is a cudaStream_t
 * passed as void* (NULL = legacy default stream).
 *
 * Ownership: the caller allocates and owns every input/output buffer (device
 * memory).  The library owns only what hangs off a bella_ws workspace
 * (prepared operator planes, Krylov vectors, reduction partials), created
 * with bella_ws_create and freed with bella_ws_destroy.  One workspace must
 * not be used from two host threads at the same time.
 *
 * Vector layout (identical to the reference's solver vectors):
 *   2D: inner nodes, y-major, idx = j*nx + i  (second_projection.py:174,214,245)
 *   3D: inner nodes, C order over (x,y,z), idx = (i*ny + j)*nz + k
 *       (second_projection.py:224,268)
 */
#ifndef BELLA_H
#define BELLA_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BELLA_OK          0   /* converged / done                              */
#define BELLA_MAXITER     1   /* iteration limit reached without convergence    */
#define BELLA_BREAKDOWN   2   /* rho or omega (or <r^,v>) below breakdown limit */
#define BELLA_NONFINITE   3   /* NaN/Inf met in a residual norm                 */
#define BELLA_TIMEOUT     4   /* wall-clock limit of the host loop exceeded     */
#define BELLA_EINVAL    (-1)  /* invalid argument                               */
#define BELLA_ECUDA     (-2)  /* CUDA runtime error (see bella_last_error)      */
#define BELLA_ENOOP     (-3)  /* workspace has no operator set                  */

typedef struct bella_ws bella_ws;   /* opaque workspace */

/*
 * 2D 9-point nodal operator, operands exactly as packed by the reference's
 * stencil_9pt_numba_test (laplacian.py:496-528) and consumed by
 * lap2D_gather_new (laplacian.py:546-746):
 *   hplusx, hplusy, cxx, cyy, cxy, cyx : (ny+1)*(nx+1) cell values, row stride nx+1
 *   hcenter, diag_inv                  : ny*nx node values
 * All FP64 device pointers.  hcenter, cxy, cyx may be NULL (== all zero).
 * x_wall / y_wall: 1 zeroes the hplus of the outer cell column / row
 * (the reference's wall handling, laplacian.py:691-713); periodic wrap with
 * the duplicated seam (wrap distance n-1, laplacian.py:595-638) is always on.
 * y_wall = BELLA_Y_MIRROR (x_wall = 0) is the operator of the reference's
 * LAMB_BDRY branch (lap2D_numba_test, laplacian.py:511-512, 531-543, 749-868):
 * the same operands, x periodic, y padded by mirroring (node -1 <- node 1,
 * node ny <- node ny-2), no cell zeroed.  Only bella_apply_* and bella_bicgstab
 * take it (no null-space projection); the ensemble, background solve and
 * allocation-free entry points reject it.
 */
#define BELLA_Y_MIRROR 2
typedef struct bella_op2d {
    int nx, ny;
    int x_wall, y_wall;
    double dx, dy;
    const double *hplusx, *hplusy, *hcenter;
    const double *cxx, *cyy, *cxy, *cyx;
    const double *diag_inv;
} bella_op2d;

/*
 * 3D 27-point nodal operator: the arithmetic of the reference's lap3D
 * (laplacian.py:898-1026) with the 2D path's boundary conventions (the
 * reference's own 3D glue, second_projection.py:183-203, cannot run):
 *   hplusx, hplusy, hplusz : (nx+1)*(ny+1)*(nz+1) cells, C order (z fastest)
 *   hcenter, diag_inv      : nx*ny*nz inner nodes, C order (z fastest)
 * corrf = dt * coriolis_strength[0] (laplacian.py:894); 0 drops the cross
 * terms.  hcenter may be NULL (== 0).  A wall axis zeroes the outer cell
 * planes; a periodic axis wraps with the duplicated seam.
 */
typedef struct bella_op3d {
    int nx, ny, nz;
    int x_wall, y_wall, z_wall;
    double dx, dy, dz;
    double corrf;
    const double *hplusx, *hplusy, *hplusz, *hcenter;
    const double *diag_inv;
} bella_op3d;

/* Solver options.  tol/atol follow the reference's scipy call
 * (second_projection.py:230, scipy 1.7 legacy `tol`): converged when
 * ||b - A x|| <= max(atol, tol*||b||); ||b|| <= tol returns x = 0 at once. */
typedef struct bella_solve_opts {
    double tol;              /* relative tolerance on ||b - A x||            */
    double atol;             /* absolute floor (0 = none)                    */
    int    maxiter;          /* inner BiCGStab iteration limit (total)       */
    int    precision;        /* 0: FP64 BiCGStab;  1: FP32 inner solves in FP64
                                iterative refinement, double-float fallback
                                accepted on the FP64 true residual only;
                                2: double-float BiCGStab (FP32-pair vectors
                                and arithmetic, ~48-bit, on the FP32 pipe)   */
    int    x0_zero;          /* 1: start from x = 0 (x is output only)       */
    int    project_null;     /* 1: keep x orthogonal to the left null vector
                                (pseudo-incompressible operator)           */
    double inner_tol;        /* IR: inner relative residual reduction        */
    int    max_outer;        /* IR: outer iteration limit                    */
    int    check_every;      /* iterations per captured graph block          */
    double timeout_s;        /* host wall-clock limit (0 = none)             */
} bella_solve_opts;

typedef struct bella_solve_stats {
    int    status;           /* BELLA_OK, BELLA_MAXITER, ...                 */
    int    iterations;       /* BiCGStab iterations (all inner solves)       */
    int    outer;            /* IR outer iterations (0 for precision 0)      */
    int    matvecs;          /* operator applications                        */
    double relres;           /* final FP64 ||b - A x|| / ||b||               */
    double bnorm;            /* ||b||                                        */
    double seconds;          /* host wall time of the call                   */
    int    fallback;         /* 1: the FP32 (or learned) inner solves failed
                                (non-finite, breakdown or no progress) and the
                                solve was finished by the plain method from the
                                FP64 iterate                                  */
    int    detail;           /* breakdown test that fired: 1 rho, 2 omega,
                                3 <r^,A p> == 0, 4 ||A s|| == 0, 5 the
                                double-float recursion diverged (x is the best
                                iterate seen, after up to 4 restarts from it)
                                (0: none)                                     */
} bella_solve_stats;

/* ---- workspace --------------------------------------------------------- */
int  bella_ws_create(bella_ws **ws, int device);
int  bella_ws_destroy(bella_ws *ws);
const char *bella_last_error(void);
const char *bella_status_string(int status);
int  bella_version(void);
/* number of library kernel launches issued through this workspace */
long long bella_ws_launches(const bella_ws *ws);
/* per-kernel CUDA-event timing of the solver kernels (0 = off).  kind:
 * 0 = p-direction stencil (v = A p), 1 = s-direction stencil (t = A s),
 * 2 = vector update, 3 = FP64 residual stencil.  Totals since enable. */
int  bella_ws_profile(bella_ws *ws, int enable);
int  bella_ws_kernel_time(bella_ws *ws, int kind, double *total_ms, long long *count);

/* ---- 2D operator (replaces the closure returned by stencil_9pt_numba_test,
 *      laplacian.py:496-528, wrapped as LinearOperator at
 *      second_projection.py:205) ----------------------------------------- */
int bella_op2d_set(bella_ws *ws, const bella_op2d *op, void *stream);

/* ---- 3D operator (replaces the closure returned by stencil_27pt,
 *      laplacian.py:872-896) -------------------------------------------- */
int bella_op3d_set(bella_ws *ws, const bella_op3d *op, void *stream);

/* y = A x with the prepared operator (2D or 3D): FP64 (parity path) and FP32 planes.
 * Replaces one call of lap2D_gather_new (laplacian.py:546-746). */
int bella_apply_f64(bella_ws *ws, const double *x, double *y, void *stream);
int bella_apply_f32(bella_ws *ws, const float *x, float *y, void *stream);

/* ---- solver (replaces scipy.sparse.linalg.bicgstab at
 *      second_projection.py:230) ----------------------------------------
 * Returns the solver status (BELLA_OK, BELLA_MAXITER, BELLA_BREAKDOWN,
 * BELLA_NONFINITE, BELLA_TIMEOUT; also in stats->status) or a negative error. */
void bella_solve_opts_default(bella_solve_opts *o);
int  bella_bicgstab(bella_ws *ws, const double *b, double *x,
                    const bella_solve_opts *opts, bella_solve_stats *stats,
                    void *stream);

/* ---- the whole 2D projection on the device (replaces
 *      euler_backward_non_advective_impl_part, second_projection.py:97-277):
 * cell boundary data, coefficients, Coriolis factors, Jacobi diagonal, nodal
 * divergence right-hand side, the solve, ghost nodes, momentum / rhoX
 * correction and p2 update, all on device arrays in the reference's layout
 * (NumPy C order over (x, y); cells (inx+3)x(iny+3), nodes (inx+4)x(iny+4)).
 * Sol (and Sol0, whose ghost cells are refreshed) and p2 are updated in
 * place.  Returns the solver status or a negative error. */
typedef struct bella_proj2d {
    int inx, iny;                 /* grid nodes per direction (ud.inx, ud.iny)       */
    int x_wall, y_wall;           /* 0: periodic, 1: wall                              */
    double dx, dy, dt;
    double Msq, g, gamm, nonhydro, compressibility;
    double coriolis[3];           /* ud.coriolis_strength                             */
    int is_compressible;
    int precond;                  /* 0: the solve of opts->precision; 1: flexible
                                     BiCGStab preconditioned by the background solve
                                     (bella_spectral2d_create, y a wall), set up per call */
    double *rho, *rhou, *rhov, *rhow, *rhoY, *rhoX;          /* Sol                    */
    double *rho0, *rhou0, *rhov0, *rhow0, *rhoY0, *rhoX0;    /* Sol0 or all NULL       */
    double *p2;                   /* mpv.p2_nodes                                     */
    const double *hydro_rhoY0;    /* mpv.HydroState.rhoY0 (iny+3 cell rows)            */
    const double *S0n;            /* mpv.HydroState_n.S0 (iny+4 node rows)             */
    const double *strat_inv;      /* 1/ud.stratification(elem.y) (iny+3)               */
    double *rhs_out;              /* mpv.rhs (inx+2)x(iny+2) or NULL                   */
} bella_proj2d;
int bella_projection2d(bella_ws *ws, const bella_proj2d *args, const bella_solve_opts *opts,
                       bella_solve_stats *stats, void *stream);
/* The projections of an ensemble's members at one stage of their time steps
 * (time_update.py:251, 462 for each member, __main__.py:223-254 runs them one
 * after another): every member's preparation, then all members' solves in one
 * persistent launch (bella_bicgstab_batched: opts->precision 0 FP64, otherwise
 * double-float with FP64 refinement; config < 0 takes the autotuned launch
 * configuration), then every member's correction.  Each member has its own
 * workspace (ws[m] distinct); precond must be 0.  stats[nmembers]. */
int bella_projection2d_batched(bella_ws *const *ws, const bella_proj2d *const *args, int nmembers,
                               const bella_solve_opts *opts, int config, bella_solve_stats *stats,
                               void *stream);

/* ---- the whole 3D projection on the device -------------------------------
 * euler_backward_non_advective_impl_part (second_projection.py:97-277) in 3D.
 * The reference's pieces run in 3D (boundary.py:7-369; second_projection.py:
 * 280-356, 496-575, 604-646, with divergence_nodes' 3D sign on the x term, :563),
 * its step does not (:183-203 use diag_inv and p2 unassigned); this entry point
 * assembles it with the glue of the 2D branch: unknowns the inner nodes
 * (inx*iny*inz, C order over x, y, z, :224), the 27-point operator of lap3D
 * (laplacian.py:898-1026) on the cells around them with corrf = dt *
 * coriolis[0], the 3D precon_diag_prepare, rhs = divergence / dt * diag_inv.
 * Arrays: the reference's NumPy C order over (x, y, z), ghosts included: cells
 * (inx+3)(iny+3)(inz+3), p2 on nodes (inx+4)(iny+4)(inz+4), rhs_out (mpv.rhs)
 * on node.isc (inx+2)(iny+2)(inz+2).  Gravity along y.  precond 0: the solve of
 * opts->precision (bella_bicgstab); 1: flexible BiCGStab preconditioned by the
 * background solve (bella_spectral3d, y must be a wall), set up per call. */
typedef struct bella_proj3d {
    int inx, iny, inz;            /* grid nodes per direction (ud.inx, ud.iny, ud.inz) */
    int x_wall, y_wall, z_wall;   /* 0: periodic, 1: wall                              */
    double dx, dy, dz, dt;
    double Msq, g, gamm, nonhydro, compressibility;
    double coriolis[3];           /* ud.coriolis_strength                             */
    int is_compressible;
    int precond;
    double *rho, *rhou, *rhov, *rhow, *rhoY, *rhoX;          /* Sol                    */
    double *rho0, *rhou0, *rhov0, *rhow0, *rhoY0, *rhoX0;    /* Sol0 or all NULL       */
    double *p2;                   /* mpv.p2_nodes                                     */
    const double *hydro_rhoY0;    /* mpv.HydroState.rhoY0 (iny+3 cell planes)          */
    const double *S0n;            /* mpv.HydroState_n.S0 (iny+4 node planes)           */
    const double *strat_inv;      /* 1/ud.stratification(elem.y) (iny+3)               */
    double *rhs_out;              /* mpv.rhs (inx+2)(iny+2)(inz+2) or NULL             */
    int div_sign_2d;              /* 0: divergence_nodes' 3D sign on its x term (:563);
                                     1: the 2D branch's sign (the 3D time step needs it) */
} bella_proj3d;
int bella_projection3d(bella_ws *ws, const bella_proj3d *args, const bella_solve_opts *opts,
                       bella_solve_stats *stats, void *stream);

/* ---- explicit parts of the projection (2D), in place on device arrays ------
 * Arrays as in bella_proj2d (reference NumPy C order over (x, y), ghosts
 * included).  S0c: mpv.HydroState.get_S0c(elem) on cells; S0n, hydro_rhoY0,
 * strat_inv as in bella_proj2d. */
typedef struct {
    int inx, iny;                 /* node.iicx, node.iicy                              */
    int x_wall, y_wall;
    double dx, dy, dt;
    double Msq, g, gamm, nonhydro, compressibility;
    double coriolis[3];           /* ud.coriolis_strength                              */
    double wind[3];               /* ud.u_wind_speed, v_wind_speed, w_wind_speed       */
    int is_compressible, is_ArakawaKonor;
    double *rho, *rhou, *rhov, *rhow, *rhoY, *rhoX;
    double *p2;                   /* mpv.p2_nodes (forward step)                       */
    double *rhs_out;              /* mpv.rhs, (inx+2)x(iny+2) (forward step)           */
    const double *S0c, *S0n, *hydro_rhoY0, *strat_inv;
} bella_expl2d;
/* euler_forward_non_advective (second_projection.py:22-74): momenta, rhoX, p2,
 * mpv.rhs, ghost nodes and boundary data */
int bella_euler_forward2d(const bella_expl2d *args, void *stream);
/* euler_backward_non_advective_expl_part (second_projection.py:77-92) */
int bella_expl_part2d(const bella_expl2d *args, void *stream);

/* ---- advection (the reference's explicit.py, recovery.py, numerical_flux.py) --
 * Device arrays in the reference's NumPy C order: cells (inx+3)(iny+3) over (x, y);
 * fx[q]: x-face arrays (iny+3)(inx+4) (elem.sfx: row y, face x), fy[q]: y-face
 * arrays (inx+3)(iny+4), q = rho, rhou, rhov, rhow, rhoY (the face mass flux),
 * rhoX.  Face arrays are zeroed by the caller once: their outer faces are never
 * written.  Gravity along y (g = ud.gravity_strength[1]); hydro_rhoY0 and strat_inv
 * as in bella_proj2d.  The limiter is the reference's only one (NONE).  */
typedef struct bella_adv2d {
    int inx, iny;                 /* grid nodes per direction                          */
    int x_wall, y_wall;           /* 0: periodic, 1: wall                              */
    double dx, dy, g, gamm;
    int is_compressible;
    int pad_;
    double *rho, *rhou, *rhov, *rhow, *rhoY, *rhoX;          /* Sol                    */
    double *fx[6], *fy[6];        /* flux[0], flux[1] of the reference                */
    const double *hydro_rhoY0, *strat_inv;
    double *pwchi;                /* advect_rk's Sol.pwchi (cells) or NULL              */
} bella_adv2d;
/* recompute_advective_fluxes (numerical_flux.py:5-46): fx rhoY, fy rhoY on the inner faces */
int bella_advective_fluxes2d(const bella_adv2d *args, void *stream);
/* advect (explicit.py:5-74): Strang-split sweeps over dt, odd = step % 2 */
int bella_advect2d(const bella_adv2d *args, double dt, int odd, void *stream);
/* advect_rk (explicit.py:160-257): first-order update over dt from the start state's fluxes */
int bella_advect_rk2d(const bella_adv2d *args, double dt, void *stream);
/* set_explicit_boundary_data (boundary.py:7-216) of the cell state: along x, then y */
int bella_boundary2d(const bella_adv2d *args, void *stream);

/* The same in 3D: cells (inx+3)(iny+3)(inz+3) over (x, y, z); face arrays as the
 * reference's elem.sfx = (iny+3)(inz+3)(inx+4), sfy = (inz+3)(inx+3)(iny+4),
 * sfz = (inx+3)(iny+3)(inz+4); pwchi (cells) after the z sweep's flip, i.e. in
 * the (x, y, z) order of the state. */
typedef struct bella_adv3d {
    int inx, iny, inz;
    int x_wall, y_wall, z_wall;
    double dx, dy, dz, g, gamm;
    int is_compressible;
    int pad_;
    double *rho, *rhou, *rhov, *rhow, *rhoY, *rhoX;
    double *fx[6], *fy[6], *fz[6];
    const double *hydro_rhoY0, *strat_inv;
    double *pwchi;
} bella_adv3d;
int bella_advective_fluxes3d(const bella_adv3d *args, void *stream);
int bella_advect3d(const bella_adv3d *args, double dt, int odd, void *stream);
int bella_advect_rk3d(const bella_adv3d *args, double dt, void *stream);
int bella_boundary3d(const bella_adv3d *args, void *stream);

/* ---- explicit parts of the projection (3D), in place on device arrays ------
 * Arrays as in bella_proj3d; S0c: mpv.HydroState.get_S0c(elem) on cells (S0 along
 * y repeated over x and z); scratch: (inx+2)(iny+2)(inz+2) doubles for the forward
 * part's pressure increment; rhs_out (mpv.rhs, node.isc) or NULL. */
typedef struct bella_expl3d {
    int inx, iny, inz;
    int x_wall, y_wall, z_wall;
    double dx, dy, dz, dt;
    double Msq, g, gamm, nonhydro, compressibility;
    double coriolis[3];           /* ud.coriolis_strength                              */
    double wind[3];               /* ud.u_wind_speed, v_wind_speed, w_wind_speed       */
    int is_compressible, is_ArakawaKonor;
    double *rho, *rhou, *rhov, *rhow, *rhoY, *rhoX;
    double *p2, *rhs_out, *scratch;
    const double *S0c, *S0n, *hydro_rhoY0, *strat_inv;
    int div_sign_2d;              /* as in bella_proj3d */
} bella_expl3d;
/* euler_forward_non_advective (second_projection.py:22-74) in 3D, with the glue of the
 * 2D branch (the reference's 3D call cannot run: it writes divergence_nodes' node.sc
 * result into the node.isc mpv.rhs): divergence on node.isc, wall rows doubled */
int bella_euler_forward3d(const bella_expl3d *args, void *stream);
/* euler_backward_non_advective_expl_part (second_projection.py:77-92) in 3D */
int bella_expl_part3d(const bella_expl3d *args, void *stream);

/* ---- CFL time step (cfl.py:5-74): the maxima over the device state ----------
 * out[6] (host) = max |u|, |v|, |w|, |u|+c, |v|+c, |w|+c over all n cells, with
 * c = sqrt(gamm rhoY^gamm / rho) / sqrt(Msq), as numpy's .max() over the whole
 * arrays in cfl.py:25-45: a NaN in any cell makes that maximum NaN.  scratch: 48
 * bytes (6 x 8) of device memory owned by the caller, reused across calls (the
 * entry point allocates nothing).  Synchronises the stream. */
int bella_cfl_maxima(const double *rho, const double *rhou, const double *rhov, const double *rhow,
                     const double *rhoY, long long n, double gamm, double Msq, void *scratch, double *out,
                     void *stream);

/* ---- ensemble: the solves of many 2D members in one persistent launch ----
 * Each member is the reference's call (second_projection.py:205-230) on its own
 * workspace (bella_op2d_set): FP64 BiCGStab, scipy 1.7 control flow, x0 = 0.
 * One cooperative kernel iterates all members (phases separated by a bounded
 * grid barrier); tol, atol, maxiter from opts; opts->precision 0: FP64
 * arithmetic, otherwise double-float on the FP32 pipe, whose members are
 * refined in FP64 (residual, batched correction solve, update) when their FP64
 * true residual misses the tolerance; members whose batched iteration broke
 * down, or that still miss after four refinement rounds, are finished alone by
 * the FP64 bella_bicgstab from their iterate within the iteration budget left
 * (the batched iterate is kept unless that lowers its FP64 true residual).  config: index of a launch configuration
 * (tile shape, CTAs per SM), < 0 for the autotuned one.  stats[m].outer reports
 * the configuration used, stats[m].fallback the refinement rounds of member m,
 * plus 256 when it was finished alone.
 * Returns BELLA_OK when every member converged, else the first failing
 * member's status. */
int bella_bicgstab_batched(bella_ws *const *ws, int nmembers, const double *const *b, double *const *x,
                           const bella_solve_opts *opts, int config, bella_solve_stats *stats, void *stream);
/* times every launch configuration on probe_iters iterations of this batch and keeps
 * the fastest for these member sizes and precision (0 FP64, else double-float);
 * ms (optional) receives the times */
int bella_batch_autotune(bella_ws *const *ws, int nmembers, const double *const *b, double *const *x,
                         int precision, int probe_iters, int *choice, double *ms, void *stream);
int bella_batch_config_count(void);
int bella_batch_config(int index, int *tile_x, int *tile_y, int *ctas_per_sm);

/* ---- learned preconditioner: 6-layer 3x3x3 CNN, 32 channels, BF16 weights and
 *      activations, FP32 accumulation, tensor-core implicit GEMM (no counterpart
 *      in the reference, which has no learned component) -------------------
 * block = 1: the convolutions run on the node grid (1 input, 1 output channel).
 * block = 2: they run on the grid of 2x2x2 node blocks, the 8 nodes of a block
 *   being 8 channels (sub-node ((a*2+b)*2+d) for offsets (a,b,d)).
 * capacity: voxels of the grid the convolutions run on, summed over the samples
 *   of a training batch (ceil(nx/block)*ceil(ny/block)*ceil(nz/block)*nsamples). */
typedef struct bella_cnn bella_cnn;
int       bella_cnn_create(bella_cnn **net, int device, int block, long long capacity);
int       bella_cnn_destroy(bella_cnn *net);
long long bella_cnn_param_count(int block);
int       bella_cnn_block(const bella_cnn *net);
/* mode 0: ReLU network with biases; 1: linear (no ReLU, no biases); 2: ReLU without biases
 * (positively homogeneous); biases must be zero for modes 1 and 2 and stay zero in training */
int       bella_cnn_set_mode(bella_cnn *net, int mode);
/* identity path: every map (forward, gradients, training, solver) returns omega*in + CNN(in);
 * default 0 */
int       bella_cnn_set_skip(bella_cnn *net, float omega);
/* the tensor-core path (1, the default): all six forward layers and the input-gradient passes on
 * tcgen05 when the z extent of the grid the net runs on is at most 142 (staged planes fit in
 * shared memory, mma.sync otherwise), the weight gradients on tcgen05 when it is at most 151
 * (FP32 CUDA-core loops otherwise); 0: mma.sync and the CUDA-core loops throughout */
int       bella_cnn_set_tc(bella_cnn *net, int on);
/* 1 if a tensor-core completion wait gave up since the last call (synchronises) */
int       bella_cnn_tc_error(bella_cnn *net);
/* FP32 parameters, layer by layer W[27][cin][cout] (tap = (dx+1)*9+(dy+1)*3+(dz+1)) then b[cout];
 * host or device pointer; set_params resets the Adam state */
int       bella_cnn_set_params(bella_cnn *net, const float *params, void *stream);
int       bella_cnn_get_params(bella_cnn *net, float *params, void *stream);
/* out = omega*in + CNN(in * in_scale) / in_scale on the nodes of an nx x ny x nz grid (C order,
 * z fastest); device FP32 arrays */
int       bella_cnn_forward(bella_cnn *net, int nx, int ny, int nz, const float *in, float *out,
                            float in_scale, void *stream);
/* grads = d/dparams sum(gout * CNN(in)); out (optional) = CNN(in); device FP32 arrays */
int       bella_cnn_gradients(bella_cnn *net, int nx, int ny, int nz, const float *in, const float *gout,
                              float *grads, float *out, void *stream);
/* one Adam step on nsamples (in, target) pairs stacked as [nsamples][nx][ny][nz];
 * loss = mean_s ||CNN(in_s) - target_s||^2 / ||target_s||^2 (before the step, optional,
 * synchronises); nx, ny, nz multiples of block, nx/block a multiple of 4 when nsamples > 1 */
int       bella_cnn_train_step(bella_cnn *net, int nsamples, int nx, int ny, int nz, const float *in,
                               const float *target, float lr, double *loss, void *stream);
/* one Adam step on the operator residual of the predicted error over nsamples crops of
 * S^3 nodes: loss = mean_s ||core(A_s(M(in_s) - target_s))||^2 / ||core(in_s)||^2, M the map
 * with its identity path, core = nodes at least margin nodes inside the crop, A_s the
 * 27-point operator (hplusx = hplusy = hplusz = hcell, no hcenter/Coriolis term) on the
 * crop with zero values outside it; hcell [nsamples][(S+1)^3] cell coefficients,
 * dinv [nsamples][S^3]; device FP32 arrays */
int       bella_cnn_train_step_op(bella_cnn *net, int nsamples, int S, const float *in, const float *target,
                                  const float *hcell, const float *dinv, double dx, double dy, double dz,
                                  int margin, float lr, double *loss, void *stream);
/* y = A_crop u for the crop operator above, zero within margin nodes of the crop's faces;
 * flux: scratch of nsamples*(S+1)^3*3 floats */
int       bella_crop_apply(int nsamples, int S, const float *u, const float *hcell, const float *dinv,
                           double dx, double dy, double dz, int margin, float *flux, float *y, void *stream);
long long bella_cnn_launches(const bella_cnn *net);
/* Flexible BiCGStab on the 3D operator of ws, right-preconditioned by net: the
 * preconditioner slot of scipy's bicgstab (its M argument), which the reference
 * leaves empty at second_projection.py:230.  FP32 inner iterations (FP32 stencil,
 * FP64 reductions) inside FP64 iterative refinement on the true residual (the
 * residual of the FP64 iterate formed in double-float arithmetic, about 1e-14 of
 * |A||x|, when tol >= 1e-11; in FP64 below that and after a fallback); tol,
 * atol, maxiter, x0_zero, project_null, inner_tol, max_outer, check_every and
 * timeout_s as for bella_bicgstab (precision is ignored); each inner solve is
 * capped at maxiter/max_outer iterations (at least 100).  When the learned
 * iteration fails (no progress, non-finite, max_outer) the plain double-float
 * BiCGStab continues from the current iterate and stats->fallback = 1. */
int       bella_fbicgstab(bella_ws *ws, bella_cnn *net, const double *b, double *x,
                          const bella_solve_opts *opts, bella_solve_stats *stats, void *stream);

/* ---- background (spectral) solve of the 3D operator (no counterpart in the
 *      reference, whose bicgstab call at second_projection.py:230 passes no M) --
 * The exact inverse of the operator with every cell coefficient replaced by
 * its mean over x and z per y-cell (the stratified background) and hcenter by
 * its mean per y-node: Hartley (periodic axis) or DCT-I (wall axis) transforms
 * in x and z as FP32 GEMMs, one FP64 tridiagonal solve along y per mode, with
 * the pseudo-inverse on the singular modes.  The Coriolis cross terms are not
 * part of the background.  y must be a wall axis.  op holds device FP64
 * arrays as for bella_op3d_set; they are read during create only.
 * apply: out = A_bg^+ (in / diag_inv) for a residual of the Jacobi-scaled
 * system; device FP32 arrays of nx*ny*nz. */
typedef struct bella_spectral3d bella_spectral3d;
int       bella_spectral3d_create(bella_spectral3d **sp, const bella_op3d *op, int device, void *stream);
/* The same background solve for the 2D 9-point operator (the reference's
 * lap2D_gather_new, laplacian.py:546-746): cxx*hplusx and cyy*hplusy averaged
 * over x per y-cell, hcenter per node row; Hartley / DCT-I along x, tridiagonal
 * along y; the Coriolis cross terms (cxy, cyx) are not part of the background.
 * op as for bella_op2d_set (y must be a wall axis); the object is used with
 * bella_spectral3d_apply / _destroy / bella_fbicgstab_pc / bella_fgmres_pc (no
 * network in 2D). */
int       bella_spectral2d_create(bella_spectral3d **sp, const bella_op2d *op, int device, void *stream);
/* Re-derive an existing background solve from new coefficients of an operator of
 * the same shape and boundary kinds (a new time step): means, 1/diag_inv and the
 * tridiagonal factors are recomputed in place, nothing is allocated, and the
 * call waits for the device only when op has an hcenter term.  BELLA_EINVAL when
 * the shape, a boundary kind or the dimension (2D/3D) differs from create's. */
int       bella_spectral3d_update(bella_spectral3d *sp, const bella_op3d *op, void *stream);
int       bella_spectral2d_update(bella_spectral3d *sp, const bella_op2d *op, void *stream);
int       bella_spectral3d_destroy(bella_spectral3d *sp);
int       bella_spectral3d_apply(bella_spectral3d *sp, const float *in, float *out, void *stream);
long long bella_spectral3d_launches(const bella_spectral3d *sp);
/* Flexible BiCGStab as bella_fbicgstab with the preconditioner
 *   sp only:   M(r) = A_bg^+ r
 *   net only:  M(r) = net(r)                         (= bella_fbicgstab)
 *   both, each stage applied to the residual the previous stages leave
 *   (the network corrects the background solve where the coefficients
 *   depart from it):
 *     compose 0: y = A_bg^+ r;  y += net(r - A y)
 *     compose 1: y = net(r);    y += A_bg^+ (r - A y)
 *     compose 2: y = A_bg^+ r;  y += net(r - A y);  y += A_bg^+ (r - A y)
 * sp must have been created for the operator set on ws (2D or 3D; the network
 * needs a 3D operator); compose is ignored unless both are given. */
int       bella_fbicgstab_pc(bella_ws *ws, bella_spectral3d *sp, bella_cnn *net, int compose, const double *b,
                             double *x, const bella_solve_opts *opts, bella_solve_stats *stats, void *stream);
/* As bella_fbicgstab_pc with flexible GMRES (Saad's FGMRES, restart 1..64) as the
 * inner solver: one cycle of at most restart iterations per refinement step, FP32
 * Arnoldi vectors with FP64 inner products and Gram-Schmidt reorthogonalisation.
 * FGMRES keeps every preconditioned vector, so it stays exact for a preconditioner
 * that is not one fixed linear map (the BF16 network), where BiCGStab's
 * recurrences lose their footing; one preconditioner application per iteration. */
int       bella_fgmres_pc(bella_ws *ws, bella_spectral3d *sp, bella_cnn *net, int compose, int restart,
                          const double *b, double *x, const bella_solve_opts *opts, bella_solve_stats *stats,
                          void *stream);

/* ---- allocation-free variant (no counterpart in the reference) ----------
 * FP64 BiCGStab of bella_bicgstab (precision 0 only) on the reference-packed
 * 2D operands, for callers that cannot allocate device memory while they run
 * (a host model that owns the whole GPU through its own memory pool, or a
 * time loop that cannot take the device-wide stall a cudaMalloc/cudaFree can
 * cause).  Needs no workspace: all scratch lives in one fixed device array
 * inside the library (about 13 MB, held by every GPU that loads the library
 * until the process exits).  Limits: nx*ny <= 65536 nodes and
 * (nx+1)*(ny+1) <= 131072 cells; larger grids return BELLA_EINVAL.
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  Every call reuses the same array: calls that overlap on the GPU
 * (other streams, other host threads, same device) race and must not be
 * issued.  The caller passes b and x (device, FP64).  Returns the solver
 * status or a negative error. */
int bella_bicgstab2d_noalloc(const bella_op2d *op, const double *b, double *x,
                             const bella_solve_opts *opts, bella_solve_stats *stats,
                             void *stream);

#ifdef __cplusplus
}
#endif
#endif /* BELLA_H */
