/*
 * scafes_gb300.h -- C ABI of the GB300-native explicit-stencil engine.
 *
 * This library replaces the per-node update sweep of ScaFES
 * (src/ScaFES_Problem.hpp:5399-5476, evalTypeTwoAt), the known-field
 * evaluation feeding it (:3434-3485), the pointer swap (:3273-3316) and the
 * MPI ghost exchange (src/ScaFES_DataField.hpp:1912-1934) with hand-written
 * sm_103a kernels on one GPU.  Its only counterpart in the reference is the
 * never-called CUDA stub src/ScaFES_ProblemCuda.hpp:84-105
 * (updateGlobalInnerUsingCudaVect) / src/ScaFES_ProblemCuda.cu:23-37; the
 * functions below are what a ScaFES::Problem would bind in its place.
 *
 * Conventions
 *  - Host arrays hold the nodes of the global grid in Fortran order
 *    (x fastest): idx = i + nx*(j + ny*k), the order of
 *    Grid::idxNodeTuple2ScalarStyleFortran (src/ScaFES_Grid.hpp:956-968),
 *    without the ghost layer and the trailing time slot of a DataField.
 *  - Every call returns SCAFES_OK (0) or a negative status; nothing exits,
 *    aborts or throws across the ABI (the reference's stub calls exit(-1),
 *    src/ScaFES_ProblemCuda.hpp:45-55).  The message of the last failure is
 *    available from the *_last_error functions.
 *  - Calls on one handle are single-threaded and ordered on the handle's
 *    stream.  Uploads and downloads synchronise that stream.
 *  - The handle owns its device memory.
 */
#ifndef SCAFES_GB300_H
#define SCAFES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SCAFES_OK 0
#define SCAFES_ERR_ARG (-1)         /* invalid argument or size            */
#define SCAFES_ERR_CUDA (-2)        /* a CUDA runtime call failed          */
#define SCAFES_ERR_STATE (-3)       /* call out of order (e.g. no upload)  */
#define SCAFES_ERR_UNSUPPORTED (-4) /* configuration no kernel covers      */
#define SCAFES_ERR_NOMEM (-5)       /* device or host allocation failed    */
#define SCAFES_ERR_TIMEOUT (-6)     /* a bounded device wait ran out       */
#define SCAFES_ERR_IO (-7)          /* a file could not be read or written */

/* ---- arithmetic / storage of the unknown field ------------------------- */
enum scafes_precision {
    /* FP64 storage, FP64 arithmetic (the reference's CT = double). */
    SCAFES_PREC_F64 = 0,
    /* Compensated FP32: each value is an unevaluated pair hi + lo of FP32
     * numbers (8 bytes per node), updated with error-free transformations
     * (Knuth TwoSum, FMA-based TwoProd).  About 48 significant bits. */
    SCAFES_PREC_F32X2 = 1,
    /* Plain FP32 storage and arithmetic. */
    SCAFES_PREC_F32 = 2,
    /* FP64 storage, arithmetic emulated with FP32 pairs: values are split
     * into hi + lo on load and rounded back to FP64 on store. */
    SCAFES_PREC_F64E = 3
};

/* ---- field slots of a plain problem ------------------------------------ */
enum scafes_field {
    SCAFES_FIELD_U = 0,   /* the unknown data field (iterate)            */
    SCAFES_FIELD_F_A = 1, /* source F(t) = F_A + time(t) * F_B            */
    SCAFES_FIELD_F_B = 2,
    SCAFES_FIELD_G_A = 3, /* border value G(t) = G_A + s * G_B          */
    SCAFES_FIELD_G_B = 4, /*   (+ s^2 G_C + s^3 G_D + s^4 G_E), s = time(t) */
                          /*   by default (scafes_gpu_set_border_time_basis) */
    SCAFES_FIELD_E_A = 5, /* exact solution E(t) = E_A + time(t) * E_B,   */
    SCAFES_FIELD_E_B = 6, /* only read by scafes_gpu_err_linf            */
    SCAFES_FIELD_G_C = 7, /* higher time orders of G, stored in FP64;    */
    SCAFES_FIELD_G_D = 8, /* read by SCAFES_BORDER_TABLE rules only      */
    SCAFES_FIELD_G_E = 9,
    SCAFES_FIELD_C0 = 10, /* centre coefficient per node   } variable-    */
    SCAFES_FIELD_CA = 11, /* axis scale per node           } coefficient  */
                          /* update, see scafes_cfg                        */
    SCAFES_FIELD_COUNT = 12
};

/* ---- border (updateBorder) kinds --------------------------------------- */
enum scafes_border {
    /* u_new = G(time(t+1)) on every global-border node: the Dirichlet
     * updateBorder of tests/system/HeatEqnFDM/Dirichlet/Dirichlet.hpp:125-131
     * and tests/system/PennesBioheatEqnFDM/Dirichlet/Dirichlet.hpp:125-131. */
    SCAFES_BORDER_DIRICHLET = 0,
    /* u_new = u_old + u_old(opposite neighbour) - s * 2^(t) at a face node,
     * the border update of tests/system/HeatEqnFdmStencilWidthOne/
     * HeatEqnFdmStencilWidthOne.hpp:136-163 (s = +1 at min faces, -1 at max
     * faces, last face in direction order wins). */
    SCAFES_BORDER_MIRROR_POW2 = 1,
    /* A linear rule per border class (the set of faces a node lies on),
     * from a table set with scafes_gpu_set_border_forms: the Neumann and
     * Cauchy updateBorder of tests/system/HeatEqnFDM/{Neumann,Cauchy}/
     * {Neumann,Cauchy}.hpp and tests/system/PennesBioheatEqnFDM/
     * {Neumann,Cauchy}/{Neumann,Cauchy}.hpp (Dirichlet at the min faces, a
     * flux condition with the mirrored neighbour at the max faces), or any
     * other rule of the same shape. */
    SCAFES_BORDER_TABLE = 2,
    /* One linear rule per border node (scafes_gpu_set_border_node_rules):
     * borders whose rule changes from node to node, such as the Neumann and
     * Cauchy faces of the reference's tissue examples, whose coefficients
     * are fields (examples/MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:172-275,
     * examples/TumorHeatEqnFDM/TumorHeatEqnFDM.hpp:278-353).  Needs the
     * variable-coefficient update (slots C0 and CA uploaded). */
    SCAFES_BORDER_NODES = 3
};

/* The rule of one border node of a SCAFES_BORDER_NODES problem, evaluated
 * in FP64 (in FP32 for an SCAFES_PREC_F32 problem):
 *   u_new = cu*u + sum_d cn[d]*u_d + cst,  neighbours d = x-, x+, y-, y+,
 * z-, z+ (a neighbour outside the grid must have weight 0). */
typedef struct scafes_border_node_rule {
    double cu;
    double cn[6];
    double cst;
} scafes_border_node_rule;

/* One border class's rule, evaluated in FP64 on border nodes:
 *   u_new = cu*u + sum_d cn[d]*u_d + cf*F(time(t-1))
 *           + cg_old*G(time(t-1)) + cg_new*G(time(t)) + cu4*u^4
 * with neighbours d = x-, x+, y-, y+, z-, z+ (a neighbour outside the grid
 * must have weight 0).  A class is a 6-bit mask of the faces a node lies on:
 * bit 0 x == 0, bit 1 x == nx-1, bit 2 y == 0, bit 3 y == ny-1, bit 4
 * z == 0, bit 5 z == nz-1; entry 0 is the rule of border nodes on no face
 * (only with n_layers_at_border > 1, else unused).  Dirichlet is
 * cg_new = 1 with every other weight 0.  The u^4 term is the radiative
 * flux of tests/system/PennesBioheatEqnFDM/Radiation/Radiation.hpp. */
typedef struct scafes_border_form {
    double cu;
    double cn[6];
    double cf;
    double cg_old;
    double cg_new;
    double cu4;
} scafes_border_form;

#define SCAFES_BORDER_CLASSES 64

/* Flux-condition kinds of scafes_border_forms_flux. */
enum scafes_flux_kind {
    SCAFES_FLUX_NEUMANN = 0,  /* -lambda du/dn = G             (Neumann.hpp)   */
    SCAFES_FLUX_CAUCHY = 1,   /* -lambda du/dn = alpha u - G   (Cauchy.hpp)    */
    SCAFES_FLUX_RADIATION = 2 /* -lambda du/dn = alpha u^4 - G (Radiation.hpp,
                                 alpha = epsilon * sigma)                     */
};

/* Configuration of one plain (single-instance) problem.
 *
 * The inner update is the 7-point linear "star" form every constant-
 * coefficient ScaFES heat-type callback reduces to:
 *   u_new = c0*u + sum_p cp[p]*(u_{p-} + u_{p+}) + cf*F(time(t-1))
 * e.g. HeatEqnFDM (tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218):
 *   cp[p] = tau*a/h_p^2, c0 = 1 - 2*sum_p cp[p], cf = tau/(rho*c);
 * Pennes (tests/system/PennesBioheatEqnFDM/PennesBioheatEqnFDM.hpp:153-168)
 * additionally subtracts tau*(rho_b*c_b/(rho*c))*W from c0.
 * scafes_star7_heat_coeffs() fills them from the physical parameters.
 *
 * Variable coefficients: once both slots SCAFES_FIELD_C0 and
 * SCAFES_FIELD_CA are uploaded, the inner update is
 *   u_new = C0(x)*u + CA(x) * sum_p cp[p]*(u_{p-} + u_{p+}) + cf*F_A(x),
 * c0 is unused and cp[p] are the axis factors (1/h_p^2 for the Pennes
 * update with CA = tau*lambda/(rho*c)): the updateInner of the reference's
 * tissue examples, whose conductivity, heat capacity, perfusion and heat
 * source are fields over the nodes (examples/MRIDataPBHEqnFDM/
 * MRIDataPBHEqnFDM.hpp:143-169; examples/TumorHeatEqnFDM/
 * TumorHeatEqnFDM.hpp:234-270, where perfusion and source change inside
 * the tumour sphere).  C0, CA and F_A are streamed by TMA with the iterate.
 * It takes F64 or F32, one border layer, a static source (no F_B) and the
 * Dirichlet, table or per-node border. */
typedef struct scafes_cfg {
    int dim;                 /* must be 3 */
    int n_nodes[3];          /* nodes per axis, each >= 3 */
    double coord_first[3];   /* coordinates of node 0 and node n-1 */
    double coord_last[3];
    double tau;              /* time step size */
    double t_start;          /* time of iterate 0 */
    int n_layers_at_border;  /* nLayersAtBorder: nodes within this many of a
                                face are border nodes (src/ScaFES_Problem.hpp:
                                3952-3971); 1 (reference default) .. min(n)/2;
                                the mirror border takes 1 only */
    int precision;           /* enum scafes_precision */
    int border;              /* enum scafes_border */
    int tile;                /* sweep tile variant 1..4 (see
                                scafes_gpu_autotune), 0 = default: 1 for
                                FP64, else 3 on grids of at least 256 x 256
                                columns and 1 below */
    double c0;               /* centre coefficient */
    double cp[3];            /* pair coefficient per axis */
    double cf;               /* source coefficient (0 disables F) */
    void* stream;            /* cudaStream_t to run on, or NULL for an own one */
} scafes_cfg;

typedef struct scafes_handle scafes_handle;

/* Fills c0, cp[3], cf of *cfg for the heat / Pennes inner update from the
 * grid of *cfg (h_p = (last-first)/(n-1), src/ScaFES_Grid.hpp:551-553):
 * coeff_a = lambda/(rho*c), rho_c = rho*c, perf = rho_b*c_b*W/(rho*c)
 * (0 for plain heat). */
int scafes_star7_heat_coeffs(scafes_cfg* cfg, double coeff_a, double rho_c,
                             double perf);

/* Fills the 64 border rules of the reference's flux-border system tests
 * for the grid, tau and inner coefficients of *cfg (call
 * scafes_star7_heat_coeffs first): nodes on a min face (an index 0) take
 * Dirichlet u_new = G(time(t)); the others take the inner update with, in
 * each direction p where the node is on the max face, the missing
 * neighbour replaced by the inner one and the flux term
 *   - cp[p]*(2 h_p/lambda) * G(time(t-1))          (Neumann)
 *   - cp[p]*(2 h_p/lambda) * (alpha*u - G(time(t-1)))   (Cauchy)
 *   - cp[p]*(2 h_p/lambda) * (alpha*u^4 - G(time(t-1))) (Radiation)
 * (tests/system/HeatEqnFDM/Neumann/Neumann.hpp and Cauchy/Cauchy.hpp, the
 * Pennes variants add the perfusion already contained in c0).  Entry 0
 * (border nodes on no face) gets the inner update. */
int scafes_border_forms_flux(const scafes_cfg* cfg, int kind, double lambda,
                             double alpha, scafes_border_form forms[64]);

/* Allocates device memory for the problem of *cfg.  Replaces the field
 * allocation of the Problem constructor (src/ScaFES_Problem.hpp:1604-1674). */
int scafes_gpu_create(const scafes_cfg* cfg, scafes_handle** out);

/* Copies a host field (n = nx*ny*nz doubles) into slot `field` and, for the
 * unknown field, resets the step counter to 0 (the initial iterate; replaces
 * evalInitPbPhase, src/ScaFES_Problem.hpp:2755-2826, whose values come from
 * the host).  Known-field slots not uploaded read as 0. */
int scafes_gpu_upload(scafes_handle* h, int field, const double* host,
                      size_t n);

/* ---- snapshots (replaces the NetCDF writer of writeDfsToFile,
 * src/ScaFES_Problem.hpp:4254-4340, and the init-file read of :4427) ------
 *
 * scafes_gpu_step_snapshots runs n_steps like scafes_gpu_step and writes
 * the iterate to `path` (created or truncated) at the current step if
 * flags has SCAFES_SNAP_START, after every step t with t % interval == 0
 * (interval > 0; the reference's nTimesteps/nSnapshots rule for
 * LIKE_GIVEN_AT_CL), and after the last step if flags has SCAFES_SNAP_END.
 * Each snapshot is copied into a device buffer, then to pinned host memory
 * on a second stream, and written while the next steps run.  The device and
 * pinned buffers are allocated on the first call and kept by the handle.
 * Synchronises the handle's stream before it returns.
 *
 * File: a 32-byte header (8 bytes "SCAFESS1", int32 version 1, int32
 * n_nodes[3], 8 reserved bytes), then per snapshot an int64 step, an FP64
 * time and nx*ny*nz FP64 values, x fastest (little-endian). */
#define SCAFES_SNAP_START 1
#define SCAFES_SNAP_END 2
int scafes_gpu_step_snapshots(scafes_handle* h, int n_steps, int interval,
                              int flags, const char* path);
/* Grid size and number of snapshots in a snapshot file (host only). */
int scafes_snapshot_info(const char* path, int n_nodes[3], int* count);
/* Snapshot `index` of a file into a dense host array (n = nx*ny*nz), with
 * its step and time; usable as the initial iterate of scafes_gpu_upload. */
int scafes_snapshot_read(const char* path, int index, double* host, size_t n,
                         long long* step, double* time);

/* Sets the border rules of a SCAFES_BORDER_TABLE problem (64 entries,
 * indexed by class mask).  A rule with cf != 0 needs a source field; one
 * with cg_old or cg_new != 0 reads G (slots G_A .. G_E). */
int scafes_gpu_set_border_forms(scafes_handle* h,
                                const scafes_border_form forms[64]);

/* Border nodes of the grid of *cfg (within n_layers_at_border of a face):
 * the number of rules scafes_gpu_set_border_node_rules takes. */
int scafes_border_node_count(const scafes_cfg* cfg, long long* count);

/* Sets the per-node border rules of a SCAFES_BORDER_NODES problem: one rule
 * per border node, the border nodes in Fortran order (x fastest, i.e. the
 * order of idx = i + nx*(j + ny*k) restricted to border nodes);
 * n = scafes_border_node_count.  Replaces the per-node updateBorder calls
 * of evalTypeTwoAt (src/ScaFES_Problem.hpp:5399-5476) for borders that are
 * linear in the iterate with coefficients that change from node to node.
 * Copies the rules to the device (FP64, 64 bytes per border node). */
int scafes_gpu_set_border_node_rules(scafes_handle* h, const scafes_border_node_rule* rules,
                                     size_t n);

/* Time variable of the border field G of a SCAFES_BORDER_TABLE problem:
 *   G(t) = G_A + s*(G_B + s*(G_C + s*(G_D + s*G_E))),
 *   s = (time(t) - t_center) * t_rate   (two FP64 roundings, no FMA),
 * Horner in FP64 with FMA; slots not uploaded are 0.  Default t_center = 0,
 * t_rate = 1 (s = time(t)).  A polynomial fitted over the run's time span
 * with s in [-1, 1] represents a known field up to quartic in time, such as
 * the radiative border field of tests/system/PennesBioheatEqnFDM/Radiation/
 * TimeLinSpaceLin/TimeLinSpaceLin.hpp evalBorder.  Dirichlet and mirror
 * problems keep G = G_A + time*G_B and refuse another basis or the slots
 * G_C .. G_E at step time. */
int scafes_gpu_set_border_time_basis(scafes_handle* h, double t_center,
                                     double t_rate);

/* Advances the unknown field by n_steps time steps (one step = the update
 * phase of one iteration of iterateOverTime, src/ScaFES_Problem.hpp:
 * 2596-2603, including the border pass and the old/new swap).  Asynchronous
 * on the handle's stream. */
int scafes_gpu_step(scafes_handle* h, int n_steps);

/* Copies the current iterate (or another slot) back to the host; n as for
 * upload.  Synchronises the handle's stream. */
int scafes_gpu_download(scafes_handle* h, int field, double* host, size_t n);

/* No counterpart in the reference (its fields live in host memory).  The
 * unknown field's upload and download enqueued on the handle's stream
 * without waiting: the host array must stay valid and unchanged (upload) or
 * unread (download) until scafes_gpu_synchronize returns, and should be
 * page-locked (scafes_host_alloc, cudaHostAlloc) for the copy to overlap
 * other work.  With two handles on two streams a caller overlaps one
 * problem's copies with the other's sweeps. */
int scafes_gpu_upload_async(scafes_handle* h, const double* host, size_t n);
int scafes_gpu_download_async(scafes_handle* h, double* host, size_t n);
/* Waits for the handle's stream and reports a sweep that gave up waiting
 * for its loads (SCAFES_ERR_TIMEOUT), as scafes_gpu_download does. */
int scafes_gpu_synchronize(scafes_handle* h);

/* No counterpart in the reference (its node loop has no tunables): times
 * n_steps sweeps with each tile variant of the sweep kernel (32 x BY CTA
 * tile, R rows per thread) on the uploaded problem, keeps the fastest for
 * later scafes_gpu_step calls and returns it (1-based) in *chosen and the
 * per-variant ms per step in ms_per_tile[4] (may be NULL); then times
 * temporal blocking depth 2 where the problem allows it and keeps it if it
 * is faster per step (scafes_gpu_temporal_depth).  The iterate and the step
 * counter are restored afterwards.  Allocates one temporary copy of the
 * iterate. */
int scafes_gpu_autotune(scafes_handle* h, int n_steps, int* chosen,
                        float* ms_per_tile);

/* Temporal blocking of scafes_gpu_step: depth 1 runs one sweep per step;
 * depth 2 runs one pass per two steps (each CTA recomputes the
 * intermediate step on a one-node halo in shared memory, so the field is
 * read and written once per two steps; same results bit for bit).  Depth 2
 * applies to Dirichlet problems with one border layer and no F_B; other
 * problems, and an odd last step, run depth 1.  Default 1;
 * scafes_gpu_autotune keeps depth 2 when it is faster.  _temporal_depth
 * gives the depth that scafes_gpu_step will use. */
int scafes_gpu_set_temporal_depth(scafes_handle* h, int depth);
int scafes_gpu_temporal_depth(const scafes_handle* h, int* depth);

/* Number of steps taken since the last upload of the unknown field. */
int scafes_gpu_timestep(const scafes_handle* h, int* t);

/* Max-norm error of the current iterate against the exact-solution slots on
 * the device (DataField::compErrLinf, src/ScaFES_DataField.hpp:1440-1530):
 * *err = max|u - E(time(t))|, *max_ref = max|E(time(t))| over all nodes.
 * Uses a per-handle device scratch buffer for the partial maxima.
 * Synchronises the handle's stream. */
int scafes_gpu_err_linf(scafes_handle* h, double* err, double* max_ref);

/* Time of the last kernel sweep sequence, in ms, measured with CUDA events
 * on the handle's stream by the last scafes_gpu_step call. */
int scafes_gpu_last_step_ms(const scafes_handle* h, float* ms);

/* Number of kernel launches issued by the last scafes_gpu_step call. */
int scafes_gpu_last_step_launches(const scafes_handle* h, int* launches);

const char* scafes_gpu_last_error(const scafes_handle* h);
void scafes_gpu_destroy(scafes_handle* h);

/* Message of the most recent failure of any call made on this thread
 * (covers failures before a handle exists). */
const char* scafes_last_error(void);

/* ---- batched ensembles --------------------------------------------------
 *
 * No counterpart in the reference, which solves one problem per process
 * (its MCMC drivers, examples/MRIDataPBHEqnFDM/startMCMCFit.py, launch
 * runs one after the other).  An ensemble holds many independent
 * instances of the constant-coefficient 7-point update with a static
 * source field and a constant Dirichlet border -- the Pennes bioheat update
 * of examples/MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:143-169 with scalar
 * coefficients -- each with its own grid, time step and coefficients:
 *   u_new = c0*u + sum_p cp[p]*(u_{p-}+u_{p+}) + cf*F   (inner nodes)
 *   u_new = g_value                                     (border nodes)
 * All instances advance together; one step of the whole ensemble is one
 * launch of a persistent kernel that pulls (instance, tile, z-chunk) work
 * items from a device queue, and the time loop is replayed from a CUDA
 * graph. */
typedef struct scafes_batch_instance {
    int n_nodes[3];          /* nodes per axis, each in [3, 32767] */
    double coord_first[3];
    double coord_last[3];
    double tau;              /* time step of this instance */
    double c0, cp[3], cf;    /* star coefficients (scafes_batch_star7_coeffs) */
    double g_value;          /* Dirichlet value on the global border */
} scafes_batch_instance;

typedef struct scafes_batch scafes_batch;

/* Fills c0, cp, cf of one instance like scafes_star7_heat_coeffs:
 * cp = tau*coeff_a/h_p^2, c0 = 1 - 2*sum cp - tau*perf, cf = tau/rho_c. */
int scafes_batch_star7_coeffs(scafes_batch_instance* inst, double coeff_a,
                              double rho_c, double perf);

/* Allocates all instances (two iterates + the source field each, padded
 * layout, one device pool) and their TMA descriptors and work lists. */
int scafes_batch_create(const scafes_batch_instance* inst, int n_inst,
                        int precision, void* stream, scafes_batch** out);

/* Host <-> device copy of one instance's field: SCAFES_FIELD_U (the
 * iterate; uploading it resets the step counter) or SCAFES_FIELD_F_A (the
 * source F).  n = nodes of that instance.  Synchronises the stream. */
int scafes_batch_upload(scafes_batch* b, int inst, int field,
                        const double* host, size_t n);
int scafes_batch_download(scafes_batch* b, int inst, int field,
                          double* host, size_t n);

/* Advances every instance by n_steps: one persistent launch per step, the
 * whole loop recorded once per (n_steps, schedule) into a CUDA graph and
 * replayed.  Asynchronous on the batch's stream. */
int scafes_batch_step(scafes_batch* b, int n_steps);

/* Advances every instance by n_steps with one plain sweep launch per
 * instance per step (the schedule of running the instances one by one);
 * for comparison with scafes_batch_step. */
int scafes_batch_step_looped(scafes_batch* b, int n_steps);

/* Times every tile variant x {occupancy, 1, 2, 4} CTAs per SM at temporal
 * depth 1, then depth 2 (two steps per pass over each instance with the
 * plain sweep's depth-2 kernel, one launch per instance and pass on 16
 * parallel chains of the graph), for n_steps (rounded up to even) batched
 * steps, and keeps the fastest (iterates restored afterwards). */
int scafes_batch_autotune(scafes_batch* b, int n_steps, int* tile,
                          int* ctas_per_sm);
/* Sets the schedule directly: tile 1..4, ctas_per_sm 0 (= occupancy) .. 16. */
int scafes_batch_set_schedule(scafes_batch* b, int tile, int ctas_per_sm);
/* Temporal-blocking depth of scafes_batch_step: 1 or 2 (an odd last step
 * of a depth-2 call runs at depth 1). */
int scafes_batch_set_temporal_depth(scafes_batch* b, int depth);
/* The depth in use and the autotuner's best ms per depth (-1 before an
 * autotune); ms pointers may be NULL. */
int scafes_batch_temporal_depth(const scafes_batch* b, int* depth, float* ms_depth1,
                                float* ms_depth2);

/* ms of the last scafes_batch_step / _step_looped call (CUDA events). */
int scafes_batch_last_ms(const scafes_batch* b, float* ms);
/* Work items per step, kernel launches of the last step call, schedule and
 * total nodes of the ensemble. */
int scafes_batch_info(const scafes_batch* b, int* n_items, int* launches,
                      int* tile, int* ctas_per_sm, long long* n_nodes);
const char* scafes_batch_last_error(const scafes_batch* b);
void scafes_batch_destroy(scafes_batch* b);

/* The same ensemble assembled one instance at a time, the shape of the
 * reference's callers that start one run per parameter set
 * (examples/MRIDataPBHEqnFDM/startMCMCFit.py): create, enqueue every
 * instance with its initial iterate u0 and source f (n_nodes values each,
 * x fastest; f may be NULL for F = 0), then run.  The first run builds one
 * scafes_batch from the enqueued instances (enqueue after it is refused)
 * and every run advances all instances by n_steps (scafes_batch_step). */
typedef struct scafes_gpu_batch scafes_gpu_batch;
int scafes_gpu_batch_create(int precision, void* stream, scafes_gpu_batch** out);
int scafes_gpu_batch_enqueue(scafes_gpu_batch* q, const scafes_batch_instance* inst,
                             const double* u0, const double* f, int* index);
int scafes_gpu_batch_run(scafes_gpu_batch* q, int n_steps);
/* The current iterate of instance `index` (synchronises the stream). */
int scafes_gpu_batch_download(scafes_gpu_batch* q, int index, double* host,
                              size_t n);
/* The underlying ensemble once the first run built it (else NULL), for
 * scafes_batch_autotune / _last_ms / _info. */
scafes_batch* scafes_gpu_batch_ensemble(scafes_gpu_batch* q);
const char* scafes_gpu_batch_last_error(const scafes_gpu_batch* q);
void scafes_gpu_batch_destroy(scafes_gpu_batch* q);

/* ---- multi-field leapfrog workloads -------------------------------------
 *
 * Problems with several unknown fields and a second ("leapfrog") update
 * phase (src/ScaFES_Problem.hpp:2604-2619, :2875-2918):
 *  SCAFES_MF_LAME  Lame-Navier elastic wave, 3 displacement components,
 *     u^{n+1} = 2u^n - u^{n-1} + tau^2/rho [ (lambda+2mu) d_cc u_c
 *               + mu sum_{p!=c} d_pp u_c + (lambda+mu) sum_{q!=c} d_cq u_q ],
 *     central differences incl. the 4-point mixed difference, border 0
 *     (examples/LameNavierEqnFDM/LameNavierEqnFDM.hpp:269-378 is the
 *     reference's form; it cannot advance, :23-25).  p = {lambda, mu, rho}.
 *     Fields 0..2: u^n (x, y, z), 3..5: u^{n-1}.  FP64 or FP32 pairs.
 *  SCAFES_MF_YEE   Yee FDTD in a PEC box (eps = mu = 1), H half step then
 *     E step (examples/EMFDTD/EMFDTD.hpp:295-385 without CPML), soft
 *     current source Ez[src] -= tau*amp*exp(-((t-t0)/w)^2) sin(2 pi f t).
 *     p = {amp, t0, w, f}.  Fields 0..5: Ex, Ey, Ez, Hx, Hy, Hz.  FP64, FP32
 *     or FP32 pairs.
 * FP32 pairs (SCAFES_PREC_F32X2): each value hi + lo, 8 bytes as FP64, the
 * update in compensated FP32 arithmetic (errors of relative size ~2^-48 per
 * step) with no FP64 instruction. */
enum scafes_mf_kind { SCAFES_MF_LAME = 0, SCAFES_MF_YEE = 1 };

typedef struct scafes_mf_cfg {
    int kind;                /* enum scafes_mf_kind */
    int n_nodes[3];
    double coord_first[3];
    double coord_last[3];
    double tau;
    double t_start;
    int precision;           /* SCAFES_PREC_F64 or _F32X2 (both), SCAFES_PREC_F32 (Yee) */
    double p[8];             /* problem parameters, see above */
    int src[3];              /* Yee source node */
    void* stream;
} scafes_mf_cfg;

typedef struct scafes_mf scafes_mf;
int scafes_mf_create(const scafes_mf_cfg* cfg, scafes_mf** out);
int scafes_mf_upload(scafes_mf* h, int field, const double* host, size_t n);
int scafes_mf_download(scafes_mf* h, int field, double* host, size_t n);
int scafes_mf_step(scafes_mf* h, int n_steps);
int scafes_mf_last_ms(const scafes_mf* h, float* ms);
const char* scafes_mf_last_error(const scafes_mf* h);
void scafes_mf_destroy(scafes_mf* h);

/* ---- linear multi-field stencils, optional leapfrog phase --------------------
 *
 * The device form of update callbacks that couple several unknown fields,
 * recorded by the drop-in Problem from updateInner/updateBorder and, for a
 * leapfrog problem, updateInner2/updateBorder2 (src/ScaFES_Problem.hpp:
 * 2604-2619 and 2875-2918: the second phase runs on the first phase's
 * result after a pointer swap):
 *   u_new[f](i) = cst + sum_k w_k * u_old[src_k](i + (dx_k, dy_k, dz_k)),
 * offsets in {-1, 0, 1}, one rule per (phase, field, node class): class 0
 * the inner nodes, classes 1..63 the border nodes by the faces they lie on
 * (the bit order of scafes_border_form), one border layer.  A field a
 * phase leaves alone needs the rule u_new[f] = u_old[f] (the reference
 * copies every node before the update, :5078-5082).  FP64.  One step runs
 * every phase once; a rule missing at the first step is SCAFES_ERR_STATE. */
#define SCAFES_LIN_MAX_FIELDS 8
#define SCAFES_LIN_MAX_TERMS 32
typedef struct scafes_lin_term {
    int src;         /* source field */
    int dx, dy, dz;  /* neighbour offset, each in {-1, 0, 1} */
    double w;        /* weight */
} scafes_lin_term;
typedef struct scafes_lin scafes_lin;
int scafes_lin_create(const int n_nodes[3], int n_fields, int n_phases, void* stream, scafes_lin** out);
/* phase 1 or 2; cls 0 (inner) .. 63; n_terms <= SCAFES_LIN_MAX_TERMS.  A
 * term may not reach beyond a face its class lies on. */
int scafes_lin_set_rule(scafes_lin* h, int phase, int field, int cls, const scafes_lin_term* terms,
                        int n_terms, double cst);
int scafes_lin_upload(scafes_lin* h, int field, const double* host, size_t n);
int scafes_lin_download(scafes_lin* h, int field, double* host, size_t n);
int scafes_lin_step(scafes_lin* h, int n_steps);
int scafes_lin_last_ms(const scafes_lin* h, float* ms);
const char* scafes_lin_last_error(const scafes_lin* h);
void scafes_lin_destroy(scafes_lin* h);

/* ---- wider stencils, one width per field -----------------------------------
 *
 * The averaging update of the reference's per-field stencil-width test,
 * tests/system/HeatEqnFdmStencilWidthVar/HeatEqnFdmStencilWidthVar.hpp:
 * 120-165 (widths per data field as in src/ScaFES_Problem.hpp:1495-1514):
 * every node, inner or border, takes
 *   u' = 2 + (sum of the values within `width` nodes along each axis,
 *             truncated at the grid's faces, + u - cc) / count,
 * cc = the sum of the signed offsets added, count = 1 + values added,
 * evaluated in the reference's order (bit-exact). */
#define SCAFES_WIDE_MAX_WIDTH 8
typedef struct scafes_wide scafes_wide;
int scafes_wide_create(const int n_nodes[3], int n_fields, const int* widths,
                       void* stream, scafes_wide** out);
int scafes_wide_upload(scafes_wide* h, int field, const double* host, size_t n);
/* n_steps updates of every field (one launch per field per step). */
int scafes_wide_step(scafes_wide* h, int n_steps);
int scafes_wide_download(scafes_wide* h, int field, double* host, size_t n);
int scafes_wide_last_ms(const scafes_wide* h, float* ms);
const char* scafes_wide_last_error(const scafes_wide* h);
void scafes_wide_destroy(scafes_wide* h);

/* ---- adjoint (gradients) -------------------------------------------------
 *
 * Replaces the reference's ADOL-C gradient path (src/ScaFES_Problem.hpp:
 * 5843-5967 traceTypeTwo, :6633-6747 evalFovForwardTypeTwo with
 * ::fov_forward at :6714), which tapes the update and evaluates the tape
 * in forward mode, one direction per parameter.  Here the reverse-time
 * sweep is hand-written for the flux-form variable-conductivity heat
 * update
 *   u'_i = u_i + sum_p tau/h_p^2 [ kp (u_{i+p} - u_i) - km (u_i - u_{i-p}) ],
 *   kp = (k_i + k_{i+p})/2, km = (k_i + k_{i-p})/2, border nodes fixed,
 * for J = 1/2 ||u_T - target||^2, giving dJ/dk and dJ/du0 in one reverse
 * sweep.  Forward states are recomputed from snapshots held in device
 * memory on the optimal binomial (revolve) schedule; with n_snapshots >=
 * n_steps every state is stored and nothing is recomputed. */
typedef struct scafes_adj scafes_adj;

/* n_snapshots >= 2 forward states (one field each) are kept on the device. */
int scafes_adj_create(const int n_nodes[3], const double coord_first[3],
                      const double coord_last[3], double tau, int n_snapshots,
                      void* stream, scafes_adj** out);
/* Arithmetic of the forward and reverse sweeps: SCAFES_PREC_F64 (default;
 * the flux form above in FP64) or SCAFES_PREC_F32X2 (the same update in
 * its equivalent diagonal form  u'_i = d_i u_i + sum_f K_f u_nb,
 * d_i = 1 - sum_f K_f, on compensated FP32 pairs; states, snapshots and
 * gradient accumulators are pairs, host arrays stay FP64).  Clears the
 * conductivity: call before scafes_adj_set_conductivity. */
int scafes_adj_set_precision(scafes_adj* a, int precision);
/* Conductivity k at the nodes (dense host array, x fastest). */
int scafes_adj_set_conductivity(scafes_adj* a, const double* k, size_t n);
/* The same with k at every node (k > 0). */
int scafes_adj_set_conductivity_uniform(scafes_adj* a, double k);
/* Plain forward solve u0 -> u_T (n_steps steps); times itself. */
int scafes_adj_forward(scafes_adj* a, const double* u0, int n_steps,
                       double* uT, size_t n);
/* J and its gradients for the forward solve from u0 over n_steps steps. */
int scafes_adj_gradient(scafes_adj* a, const double* u0, const double* target,
                        int n_steps, double* J, double* grad_k,
                        double* grad_u0, size_t n);
/* The backward entry for any objective of u_T: given the forward solve
 * from u0 over n_steps and the cotangent dJ_duT = dJ/du_T (n values),
 * writes dJ/dk and dJ/du0 (the vector-Jacobian product of u0, k -> u_T),
 * with the same checkpoint schedule as scafes_adj_gradient. */
int scafes_adj_backward(scafes_adj* a, const double* u0, const double* dJ_duT,
                        int n_steps, double* grad_k, double* grad_u0, size_t n);
/* ms of the last forward solve and gradient, forward steps the last call
 * ran (including recomputation), adjoint steps, snapshots. */
int scafes_adj_stats(const scafes_adj* a, float* forward_ms, float* gradient_ms,
                     long long* forward_steps, long long* adjoint_steps,
                     int* snapshots);
/* Forward steps the binomial schedule needs for n_steps with n_snapshots. */
long long scafes_adj_schedule_cost(int n_steps, int n_snapshots);
const char* scafes_adj_last_error(const scafes_adj* a);
void scafes_adj_destroy(scafes_adj* a);

/* The backward entry of a plain handle, replacing the ADOL-C tape the
 * reference records around updateInner (src/ScaFES_Problem.hpp:5843-5967,
 * :6633-6747).  For a heat problem (the heat form c0 = 1 - 2 sum cp,
 * cp[p] = tau*a/h_p^2, no source, the Dirichlet border with one layer and a
 * value constant in time) run over the h->t steps since its last upload of
 * the unknown field, and a cotangent dJ_du_T = dJ/du_T (n = nx*ny*nz host
 * values, x fastest), writes dJ_dk -- the gradient with respect to the
 * conductivity as a field, k(x) = a being the handle's problem, in the
 * flux form of the adjoint engine above (so sum dJ_dk = dJ/da) -- and
 * dJ_du0.  Forward states are recomputed from n_checkpoints >= 2 snapshots
 * on the binomial schedule, in the handle's precision (F64 or F32X2).  The
 * initial iterate comes from the copy scafes_gpu_keep_initial keeps; its
 * border nodes must equal the Dirichlet value (SCAFES_ERR_UNSUPPORTED
 * otherwise).  The Dirichlet border resets every border node each step, so
 * a border value of u0 enters the first step only and dJ_du0 on border
 * nodes is that step's part (the derivative the reference's own
 * updateInner/updateBorder give with a differentiable scalar).  scafes_gpu_keep_initial(h, 1) makes every later upload of
 * the unknown field also keep an FP64 copy on the device (one more field of
 * device memory); 0 frees it. */
int scafes_gpu_keep_initial(scafes_handle* h, int on);
int scafes_gpu_adjoint(scafes_handle* h, const double* dJ_du_T, double* dJ_dk,
                       double* dJ_du0, int n_checkpoints);

/* No counterpart in the reference.  The same max-norm check as
 * scafes_gpu_err_linf, for callers that must not allocate device memory at
 * the point of the call -- a serving loop that forbids cudaMalloc after
 * start-up (it can synchronise the device and fail under memory pressure),
 * or a host whose device memory all comes from its own pool.  It allocates nothing: u and exact are
 * caller-owned device arrays of n doubles, out is a caller-owned device
 * array of 2 doubles that receives max|u - exact| and max|exact|, and the
 * partial maxima live in a fixed 256 KiB array in the library's device
 * image, which every GPU that loads the library holds until the process
 * exits.  n may be at most SCAFES_ERR_LINF_NOALLOC_MAX_N; larger n is
 * rejected with SCAFES_ERR_ARG and a message in scafes_last_error().  The
 * call is asynchronous on `stream` (NULL = legacy default stream).  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, which may load the module), and so does the first
 * call after that device's context was replaced (cudaDeviceReset): make
 * those calls before any stream capture.  All calls share the array: calls that
 * overlap on the GPU (e.g. on two streams without ordering) race on it and
 * give wrong results. */
#define SCAFES_ERR_LINF_NOALLOC_MAX_N (16384LL * 32768LL)
int scafes_err_linf_noalloc(const double* u, const double* exact, long long n,
                            double* out, void* stream);

/* No counterpart in the reference.  Page-locked host memory for the host
 * arrays of uploads and downloads, backed by huge pages: a copy engine
 * translates every host page it touches, and after a long solve the
 * translations of a 1 GiB buffer of 64 KB pages are no longer cached (the
 * first copy measured 45 - 160 ms on GB300 instead of the link's 5.2 ms);
 * huge pages keep the copies at the link rate.  Allocates at least `bytes`
 * (rounded up to the huge page size), zeroed; free with scafes_host_free.
 * The memory is registered with CUDA (cudaHostRegister), so any pointer
 * into it is pinned host memory for cudaMemcpyAsync. */
int scafes_host_alloc(size_t bytes, void** out);
void scafes_host_free(void* p);

/* No counterpart in the reference: measures the FP64 and FP32 FMA issue
 * rates of the current GPU (G op/s) with CUDA events, the compute ceilings
 * the benchmark reports beside the HBM roofline. */
int scafes_probe_pipe_rates(double* fp64_gops, double* fp32_gops);

/* No counterpart in the reference: runs the FP64 sweep's integer-pipe
 * binary64 addition (both operands of one sign, exponents at most 10
 * apart, the smaller exponent field in [1, 2035]; round to nearest even)
 * on the device for n pairs of bit patterns a[i], b[i] (host arrays,
 * 1 <= n <= 2^26).  ok[i] = 1
 * where the pair lies in that range, and then sum[i] holds the bits of
 * a[i] + b[i]; elsewhere the sweep adds in FP64 and sum[i] is undefined. */
int scafes_probe_dadd_int(const unsigned long long* a, const unsigned long long* b, unsigned long long* sum,
                          unsigned char* ok, long long n);

/* Failure-detection checks (no fault involved).  scafes_probe_wait_timeout
 * runs the bounded device wait of the sweep kernels on an mbarrier that
 * never completes, with a limit of limit_us (1 .. 1e6): *status receives
 * the status the kernel recorded (SCAFES_ERR_TIMEOUT) and *waited_ms the
 * time it waited.  scafes_gpu_inject_status writes `code` (<= 0) into a
 * handle's device status word, as a sweep that gave up does: later sweeps
 * of the handle skip their work and the next download reports the status
 * (and clears it). */
int scafes_probe_wait_timeout(unsigned limit_us, int* status, double* waited_ms);
int scafes_gpu_inject_status(scafes_handle* h, int code);
/* The same for an adjoint handle: its FP32-pair forward and adjoint steps
 * skip their work while the word is set, and the next scafes_adj_forward /
 * scafes_adj_gradient / scafes_adj_backward returns the status (and clears
 * it). */
int scafes_adj_inject_status(scafes_adj* a, int code);

#ifdef __cplusplus
}
#endif
#endif
