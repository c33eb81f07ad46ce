/*
 * pannde_gb300.h -- C ABI of the GB300 (sm_103a) rotated-staggered-grid (RSG)
 * elastodynamic leapfrog on hex meshes.
 *
 * This is the drop-in boundary for PanNDE's solver path
 *   HostSolver::HostRSGTDUT::solve  (modules/HostSolver/include/HostRSGTDUT.hpp:162-169)
 *   HostSolver::HostUTModel::solve  (modules/HostSolver/include/HostUTModel.hpp:186-193)
 * The entry points take plain C structs of host pointers and sizes: no C++,
 * no torch and no CUDA types cross this line (streams are passed as void*).
 * Every call returns an int status (PN_OK on success); on failure
 * pn_last_error() returns a message for the calling thread.  No exception
 * ever crosses the ABI; the C++ adapter (include/DeviceSolver.hpp) rethrows
 * the exception type the reference would have thrown, keyed on the status.
 *
 * All host-side floating-point inputs and outputs are IEEE double, as in the
 * reference's HostField/HostArray.  The device storage type is picked by the
 * precision argument of pn_solver_create.
 */
#ifndef PANNDE_GB300_H
#define PANNDE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PN_ABI_VERSION 3

/* ---- status codes ------------------------------------------------------ */
enum pn_status {
  PN_OK = 0,
  PN_ERR_INVALID = 1,    /* bad argument: null pointer, negative size, unknown enum */
  PN_ERR_SPACING = 2,    /* non-positive nodal spacing: reference throws
                            std::logic_error("DX"/"DY"/"DZ"), RightHex.hpp:305-307 */
  PN_ERR_RANGE = 3,      /* index out of range: reference throws std::out_of_range,
                            HexMesh.hpp:252-257 (invalid node id in a cell) */
  PN_ERR_RUNTIME = 4,    /* reference throws std::runtime_error, e.g. mismatched
                            signal arrays, HostUnivariate.hpp:80 */
  PN_ERR_CUDA = 5,       /* a CUDA runtime call failed */
  PN_ERR_ALLOC = 6,      /* device allocation failed or exceeds the HBM budget */
  PN_ERR_NOT_FINITE = 7, /* NaN/Inf in an input array (the call changes nothing) */
  PN_ERR_DEVICE_CHECK = 8/* a device-side bounds check recorded an error */
};

/* ---- precision / arithmetic forms -------------------------------------- */
enum pn_precision {
  /* FP64 state and arithmetic in the reference's exact operation order
     (no FMA contraction, divisions by the stored spacings): bit-identical
     to HostSolver on the same inputs.  Parity mode; slowest. */
  PN_PREC_F64_EXACT = 0,
  /* FP64 state and arithmetic with constants folded (dt*C, 0.25/h, dt/rho)
     and FMA: the drop-in fast path, <= 1e-10 relative L2 against HostSolver. */
  PN_PREC_F64 = 1,
  /* FP32 state, FP32 material tensors and FP32 arithmetic; traces are
     returned in FP64.  Roughly halves the bytes per step. */
  PN_PREC_F32 = 2,
  /* FP64-class form for GB300, whose FP64 pipe issues about 2 FMAs per SM
     per clock: state and arithmetic in double-float (each value the
     unevaluated sum of two floats, a 48-bit significand) on the FP32 pipes,
     8 bytes per value like FP64.  Host-side inputs and outputs stay FP64.
     Values must stay within the float exponent range (|x| < 3e38, and
     magnitudes below 1e-38 flush towards zero). */
  PN_PREC_DF64 = 3
};

/* Device forms; OR one into the precision argument of pn_solver_create*.
   The reference has a single (host) form; these choose how the device holds
   the same mesh. */
enum pn_form {
  /* the grid form when the mesh is a voxel grid (every node on a uniform
     lattice, every cell a lattice box in the reference corner order; several
     nodes may share a lattice site, as a crack modelled as disconnected faces
     has them, up to an eighth of the nodes), the fused kernel marches at most
     twice the mesh's cells in its lattice box (each tile column stops at its
     top solid layer) and the precision is not PN_PREC_F64_EXACT; else the
     table form */
  PN_FORM_AUTO = 0,
  /* connectivity tables on the device (cell -> 8 nodes, node -> 8 cell
     slots), two kernels per step; any hex mesh of at most 715,827,882 nodes
     and cells (PN_ERR_INVALID above that) */
  PN_FORM_TABLE = 0x100,
  /* implicit lattice indices, one fused kernel per step, double-buffered
     state; PN_ERR_INVALID when the mesh is not a voxel grid */
  PN_FORM_GRID = 0x200
};
#define PN_FORM_MASK 0xF00

/* Field storage types; numbering equals PanNDE::Field::FieldType
   (modules/PanNDE/include/Field.hpp, NODE=0, CELL=1, CONSTANT=2). */
enum pn_field_type { PN_FIELD_NODE = 0, PN_FIELD_CELL = 1, PN_FIELD_CONSTANT = 2 };

/* Source kinds. */
enum pn_source_kind {
  /* Force added in the velocity update at every node, evaluated at the centres
     of the node's existing incident cells with weight 0.125 each:
     HostRSGTDUT::evalXds (HostRSGTDUT.hpp:387-402), HostUTModel::evalXds
     (HostUTModel.hpp:404-419).  component = direction 0..2 (x,y,z). */
  PN_SOURCE_FORCE = 0,
  /* Moment-tensor term added in the stress update at every cell, evaluated at
     the cell's 8 corner nodes with weight 0.125 each: HostUTModel::evalMoments
     (HostUTModel.hpp:296-311).  component = Voigt index 0..5 (xx,yy,zz,yz,xz,xy). */
  PN_SOURCE_MOMENT = 1
};

/* ---- input descriptions ------------------------------------------------ */

/* Hex mesh; replaces PanNDE::Mesh as read by the solver (Mesh.hpp:98-226,
   HexMesh.hpp:75-352).  Cells list 8 corner node ids in the reference's
   corner order (PlateBuilder.hpp makeCell: 0=(0,0,0) 1=(1,0,0) 2=(1,1,0)
   3=(0,1,0) 4..7 the same at +z).  The node->cell links are built exactly as
   HexMesh::buildLinks (HexMesh.hpp:300-313): corner k of cell c goes to slot
   k^6 of that node, later cells overwrite earlier ones. */
typedef struct pn_mesh {
  int32_t n_nodes;
  int32_t n_cells;
  const double *x, *y, *z;     /* [n_nodes] node coordinates */
  const int32_t *hexes;        /* [n_cells * 8] corner node ids */
  const int32_t *node_owner;   /* [n_nodes] home partition, or NULL = all owned */
  int32_t partition_id;        /* nodes with node_owner != partition_id are not updated
                                  (HostRSGTDUT.hpp:339, updateVsAtNode) */
} pn_mesh;

/* One field of the domain bundle: NODE ([n_nodes]), CELL ([n_cells]) or
   CONSTANT ([1]) values, read with HostField's semantics (HostField.hpp:110-153). */
typedef struct pn_field {
  int32_t type;                /* enum pn_field_type */
  const double *data;
} pn_field;

/* Elastic material: ElasticMaterialNames (StandardNames.hpp:64-82).
   cij holds the 21 unique Voigt entries in upper-triangle row order
   C11 C12 C13 C14 C15 C16 C22 C23 C24 C25 C26 C33 C34 C35 C36 C44 C45 C46
   C55 C56 C66; the solver reads C[i][j] = C[j][i] as the reference does. */
typedef struct pn_material {
  pn_field density;
  pn_field cij[21];
} pn_material;

/* Indexed form of the same domain: cell c has density[cell_material[c]] and
   stiffness cij[cell_material[c]][0..20] (same 21-entry order as pn_material).
   Equivalent to CELL fields built from the table; this is how the reference's
   case makers write per-cell properties from a few materials
   (the py_utils/Case_Makers scripts: C_arr[:, cell] = C[:, Geom[i,j,k]-1]) without the
   caller expanding them to n_cells x 22 doubles. */
typedef struct pn_material_table {
  int32_t n_materials;
  const double *density;         /* [n_materials] */
  const double *cij;             /* [n_materials * 21] */
  const int32_t *cell_material;  /* [n_cells], values in [0, n_materials) */
} pn_material_table;

/* Piecewise-linear time series; replaces HostData::HostUnivariate
   (HostUnivariate.hpp:69-152): linear interpolation between samples, the
   last value held for t >= last sample time. Times need not be sorted;
   duplicate times keep the first value (std::map::emplace semantics). */
typedef struct pn_signal {
  int32_t n;
  const double *t;
  const double *v;
} pn_signal;

/* A windowed source with a separable time signal; replaces
   Stubs::HostNormalXDZ (HostNormalXDZ.hpp:117-145):
   evalAt(p,t) = signal(t) * [|p_z - cz| <= 0.75*ds] * [|p - c| < radius]. */
typedef struct pn_window_source {
  int32_t kind;        /* enum pn_source_kind */
  int32_t group;       /* transducer / moment-tensor index: accumulation order */
  int32_t component;   /* force direction 0..2 or Voigt component 0..5 */
  double center[3];
  double radius;
  double ds;
  pn_signal signal;
} pn_window_source;

/* A windowed source given by its window instead of its geometry, for callers
   that hold the reference's own PanNDE::MultiVariate objects: inside[] is the
   caller's MultiVariate::checkAt (MultiVariate.hpp:118-141) evaluated at every
   cell centre (PN_SOURCE_FORCE; centres as HostRSGTDUT::cellcenter,
   HostRSGTDUT.hpp:419-428) or at every node (PN_SOURCE_MOMENT).  Its signal
   values come per step from pn_solver_solve_signals. */
typedef struct pn_window_mask {
  int32_t kind;            /* enum pn_source_kind */
  int32_t group;
  int32_t component;
  const uint8_t *inside;   /* [n_cells] (force) or [n_nodes] (moment), 0 or 1 */
} pn_window_mask;

/* Read-only facts about a created solver. */
typedef struct pn_solver_info {
  int32_t n_nodes, n_cells;
  int32_t precision;
  int32_t n_materials;       /* unique stiffness rows after de-duplication */
  int32_t uniform_spacing;   /* 1: one (hx,hy,hz) for every cell and node */
  int32_t n_source_nodes;    /* nodes with a force source term */
  int32_t n_source_cells;    /* cells with a moment source term */
  int32_t n_sensors;
  int64_t algorithmic_bytes_per_step; /* HBM bytes one step must move in this form */
  int64_t device_bytes;      /* device memory held by the solver */
  double dt;
  double time;
  int32_t form;              /* PN_FORM_TABLE or PN_FORM_GRID */
  int32_t grid[3];           /* grid form: cells per axis */
  int32_t grid_kernel;       /* grid form: 1 classic (register prefetch), 2 tensor-copy staging, 3
                                tensor-copy staging in the FP64 form's two launches per step (its
                                double-float and its FP64 blocks); 0 table */
} pn_solver_info;

/* What pn_solver_create would build, computed on the host only. */
typedef struct pn_plan {
  int32_t n_nodes, n_cells;
  int32_t n_materials;
  int32_t uniform_spacing;
  double hx, hy, hz;                  /* the spacings when uniform_spacing */
  int64_t device_bytes;               /* device memory pn_solver_create allocates */
  int64_t algorithmic_bytes_per_step;
  int32_t form;                       /* the form PN_FORM_AUTO would pick */
  int32_t grid[3];                    /* grid form: cells per axis */
} pn_plan;

typedef struct pn_solver pn_solver;

/* ---- entry points ------------------------------------------------------ */

/* Library ABI version (PN_ABI_VERSION). */
int pn_abi_version(void);

/* Message for the last failed call on this thread ("" if none). */
const char *pn_last_error(void);

/* Validate a mesh and domain exactly as pn_solver_create does (same status
   codes and messages: "DX"/"DY"/"DZ", invalid node id, non-finite input)
   and report sizes, spacing and the device footprint, without any CUDA
   call.  Pass one of material / table (the other NULL).  Replaces nothing
   in the reference (whose constructor does this work, RightHex.hpp:80-90);
   serving admission uses the footprint before allocating. */
int pn_plan_solver(const pn_mesh *mesh, const pn_material *material,
                   const pn_material_table *table, double dt, int32_t precision,
                   pn_plan *out);

/* Source weights on the host, without any CUDA call: node_force_w[n*3+d] =
   0.125 * number of (incident cell, force source of direction d) pairs whose
   cell centre is in the window (HostRSGTDUT::evalXds, HostRSGTDUT.hpp:387-402);
   cell_moment_w[c*6+k] the same over (corner node, moment source of Voigt
   component k) pairs (HostUTModel::evalMoments, HostUTModel.hpp:296-311).
   Either output may be NULL. */
int pn_plan_sources(const pn_mesh *mesh, const pn_window_source *src, int32_t n,
                    double *node_force_w, double *cell_moment_w,
                    int32_t *n_source_nodes, int32_t *n_source_cells);

/* HostUnivariate::evalAt at n times (HostUnivariate.hpp:109-142), on the host. */
int pn_signal_eval(const pn_signal *signal, const double *t, int32_t n, double *out);

/* Build a solver on the current CUDA device: uploads connectivity, spacing,
   material and density tables.
   Replaces the constructors HostRSGTDUT(dt,domain,initial_condition,...)
   (HostRSGTDUT.hpp:119-146) and HostUTModel(dt,domain,initial_condition,comm)
   (HostUTModel.hpp:113-129) up to setup(): setupProperties, RightHex(mesh)
   nodePrep/cellPrep (RightHex.hpp:80-90, 253-309).  State starts at zero. */
int pn_solver_create(const pn_mesh *mesh, const pn_material *material, double dt,
                     int32_t precision, pn_solver **out);

/* Same as pn_solver_create with the domain given as a material table
   (pn_material_table); the result is identical to passing the equivalent
   CELL fields. */
int pn_solver_create_indexed(const pn_mesh *mesh, const pn_material_table *material,
                             double dt, int32_t precision, pn_solver **out);

/* Enqueue all subsequent work on this CUDA stream (cudaStream_t as void*;
   NULL = the legacy default stream). */
int pn_solver_set_stream(pn_solver *s, void *cuda_stream);

/* Upload the initial condition: V[3] = Vx,Vy,Vz ([n_nodes] each), S[6] =
   Sxx,Syy,Szz,Syz,Sxz,Sxy ([n_cells] each); a NULL pointer means zero.
   Arrays in page-locked host memory are read by the GPU directly, others are
   staged; returns when the transfer is done.  PN_ERR_NOT_FINITE (state left
   unchanged) when a value is NaN or infinite.  Replaces setupSolution
   (HostRSGTDUT.hpp:235-239). */
int pn_solver_set_state(pn_solver *s, const double *const *V, const double *const *S);

/* Add windowed sources.  Replaces the transducer constructor arguments
   (HostRSGTDUT.hpp:139-146), HostUTModel::applyTransducer (HostUTModel.hpp:138-141)
   and applyMomentExcitation (HostUTModel.hpp:152-170). */
int pn_solver_add_sources(pn_solver *s, const pn_window_source *src, int32_t n);

/* Add sources given by window masks (pn_window_mask).  They take part in
   every later solve like pn_solver_add_sources' sources, in addition order;
   their signal values must come from pn_solver_solve_signals.  Replaces the
   same constructor / apply calls as pn_solver_add_sources for arbitrary
   separable MultiVariate sources (evalAt(p,t) = checkAt(p) * signal(t)). */
int pn_solver_add_window_masks(pn_solver *s, const pn_window_mask *masks, int32_t n);

/* Record V at these nodes after every step (traces [step][sensor][3]).
   The reference records the transducer-node velocities at write times
   (TransducerModel.cpp:143-149); this records every step, fused into the
   velocity update.  capacity_steps bounds the device trace buffer. */
int pn_solver_set_sensors(pn_solver *s, const int32_t *nodes, int32_t n,
                          int32_t capacity_steps);

/* Advance nsteps leapfrog steps: velocity update, stress update, time += dt.
   Enqueue only (no device synchronisation); *time_out (may be NULL) receives
   the new time, accumulated on the host in FP64 exactly as the reference.
   Replaces Model::solve (Model.hpp:77-106; HostRSGTDUT.hpp:162-169). */
int pn_solver_solve(pn_solver *s, int32_t nsteps, double *time_out);

/* pn_solver_solve with the signal values of every source given by the caller
   for each step: values[k * n_sources + i] is source i's signal at the time
   of step k of this call (sources numbered in addition order, geometry
   sources and mask sources alike).  This is how a caller reproduces the
   reference's per-step MultiVariate::evalAt (HostRSGTDUT.hpp:387-402) with
   its own objects. */
int pn_solver_solve_signals(pn_solver *s, int32_t nsteps, const double *values, double *time_out);

/* Synchronise and download the state into caller-owned host arrays (same
   layout as pn_solver_set_state; NULL pointers are skipped; page-locked
   arrays are written by the GPU directly).  Replaces the
   host reads the runners make through Model::getStates() (Model.hpp:77-106,
   TransducerModel.cpp:143-149, VTKGrid.hpp:125-160). */
int pn_solver_get_state(pn_solver *s, double *const *V, double *const *S);

/* Synchronise and copy recorded traces ([n_records][n_sensors][3], FP64) into
   out (capacity max_records records); *n_records receives the count. */
int pn_solver_get_traces(pn_solver *s, double *out, int64_t max_records, int64_t *n_records);

/* Forget recorded traces (the next step writes record 0). */
int pn_solver_clear_traces(pn_solver *s);

/* Current simulation time (host-side FP64 accumulation). */
int pn_solver_get_time(pn_solver *s, double *time_out);

/* Facts about the solver (sizes, bytes per step, device memory). */
int pn_solver_get_info(pn_solver *s, pn_solver_info *info);

/* Device pointers of the current state arrays, for zero-copy interop; V[3],
   S[6] receive the pointers.  Element type by precision (double, float, or
   float2 (hi, lo) for PN_PREC_DF64); order by form: the caller's node / cell
   numbering in the table form, the lattice numbering (x fastest) in the grid
   form.  The FP64 grid form chooses per tile between FP64 and double-float
   arithmetic from the values its last step stored; this call puts every tile
   on the FP64 path for the next step, so values written through the pointers
   after this call and before the next solve are taken exactly -- call it
   again after writing between later steps. */
int pn_solver_device_state(pn_solver *s, void **V, void **S);

/* Energy audit of the current state, formed and summed in FP64 whatever the
   storage precision: kinetic = 1/2 sum_n m_n |V_n|^2 with the lumped nodal
   mass m_n = rho_n dx_n dy_n dz_n (rho_n the reference's nodal density,
   nodes of other partitions excluded); strain = 1/2 sum_c vol_c S_c . C_c+ S_c
   with C_c+ the pseudo-inverse of the cell's Voigt stiffness (engineering
   shear strain, so S . C+ S = sigma : epsilon; a fluid's missing shear
   stiffness contributes nothing).  Synchronises.  No counterpart in the
   reference: an audit the FP32 form reports beside its traces. */
int pn_solver_energy(pn_solver *s, double *kinetic, double *strain);

/* Block until all work enqueued by this solver is done; reports errors from
   the device-side checks. */
int pn_solver_synchronize(pn_solver *s);

/* Per-kernel device time.  While enabled, every launch of the velocity and
   the stress kernel is bracketed by CUDA events on the solver's stream.
   pn_solver_kernel_times synchronises, returns the summed milliseconds and
   the launch counts of [velocity, stress, fused grid step] since timing was
   enabled, and restarts the count.  Profiling aid; no counterpart in the
   reference. */
int pn_solver_enable_kernel_timing(pn_solver *s, int32_t enable);
int pn_solver_kernel_times(pn_solver *s, double *ms /* [3] */, int64_t *launches /* [3] */);

/* ---- batches ------------------------------------------------------------
   A batch advances many solvers together: each step is one launch per half
   step (table form) or one fused launch (grid form) covering every member,
   with work tiles spread over the GPU whatever the members' sizes.  Members
   are ordinary solvers (same precision and form) that keep their own state,
   sources, sensors, time and dt; they can join and leave between steps, and
   a member's results do not depend on the other members.  No counterpart in
   the reference, which runs one model per process. */
typedef struct pn_batch pn_batch;

int pn_batch_create(pn_batch **out);
/* Add / remove a member (the batch does not own it; destroy members after
   removing them or destroying the batch). */
int pn_batch_add(pn_batch *b, pn_solver *member);
int pn_batch_remove(pn_batch *b, pn_solver *member);
int pn_batch_size(pn_batch *b, int32_t *n_members);
/* Work on this stream (void* cudaStream_t; NULL = legacy default stream). */
int pn_batch_set_stream(pn_batch *b, void *cuda_stream);
/* Advance every member nsteps steps (their own signals, sensors, time). */
int pn_batch_solve(pn_batch *b, int32_t nsteps);

/* pn_batch_solve without any device allocation.  No counterpart in the
   reference (replaces nothing there; an addition for callers that cannot
   allocate device memory while they run: a serving loop that plans every
   byte of HBM up front with pn_plan_solver and must not have a solve grow
   buffers behind its back, or a host whose device memory is owned by a pool
   that forbids driver allocations after start-up -- cudaMalloc and cudaFree
   can also stall every stream of the device while they run).
   pn_batch_solve stages the members' argument blocks in buffers it grows
   with cudaMalloc; this call stages them in one fixed 256 KiB device array
   compiled into the library (room for about 270 grid-form or 550
   table-form members), looked up with
   cudaGetSymbolAddress on the first call on each device -- make that first
   call before any stream capture starts on the device.  The first call on a
   device may also load kernels the process has not launched yet (CUDA's lazy
   module loading), which the driver backs with memory of its own; later calls
   load nothing.  The looked-up address is kept for the life of the process's
   context on the device: do not call this again on a device after
   cudaDeviceReset.  Batches whose
   staging does not fit return PN_ERR_INVALID with the sizes, and so do
   members whose source tables or signal table have not been built yet (any
   one pn_batch_solve or pn_solver_solve step builds them; signal rows are
   then refilled in place, never grown).  Nothing in the scratch has to start
   at zero: every launch reads only bytes its call wrote before it.  All
   batches of a process share the scratch: overlapping calls (from several
   host threads) would race on it, so the call holds a process-wide lock and
   they run one after another; each call waits for its GPU work before it
   returns, so the scratch is idle between calls.  Results are identical to
   pn_batch_solve. */
int pn_batch_solve_noalloc(pn_batch *b, int32_t nsteps);
int pn_batch_synchronize(pn_batch *b);
/* Launch planning of pn_batch_solve: the launch shape (how one step's work is
   spread over the GPU) is autotuned once per class of batch (form,
   precision, member count and work size) by timing candidates on real steps,
   and a chunk of steps whose launch sequence repeats the previous chunk's is
   captured as a CUDA graph and replayed (work on a created stream only).
   Grid-form shapes are a block tile of 32 x tile_rows threads (rows 8, or 16
   with FP32 storage and the tensor-copy kernel; the members are re-tiled to
   try and to keep a shape) times z chunks per tile column (0: as many as
   one wave of resident blocks needs); table-form shapes are resident blocks
   per SM.  Neither changes results.  Reports the graph replays and captures
   so far, the number of tuned classes, and the shape of the last chunk run:
   tile_rows (0 for the table form) and shape (grid: z chunks per column, 0 =
   the launcher's choice; table: blocks per SM).  Any pointer may be NULL. */
int pn_batch_plan_stats(pn_batch *b, int64_t *graph_launches, int64_t *graph_captures, int32_t *tuned_classes,
                        int32_t *tile_rows, int32_t *shape);
int pn_batch_destroy(pn_batch *b);

/* ---- partitioned solve ----------------------------------------------------
   One mesh solved as n_parts partitions on the current device, with the
   reference's domain decomposition (MetisHexPartitioner.hpp) and its single
   exchange per step (HostUTModel.hpp:316-326): nodes get a home partition by
   recursive coordinate bisection (in place of METIS); a partition's local
   mesh is every cell touching a home node plus those cells' nodes; a step
   updates the velocity of home nodes in every partition, copies each halo
   node's velocity from its home partition on the device, then updates the
   stress of every local cell (halo cells recomputed, as the reference does).
   Results equal the single-partition solve.  Precision PN_PREC_F64,
   PN_PREC_F32 or PN_PREC_DF64 (table form); the mesh must not carry
   node_owner.  Replaces the reference's MPI decomposition for one device; on
   several devices the exchange lists are the messages to send. */
typedef struct pn_partitioned pn_partitioned;

int pn_partitioned_create(const pn_mesh *mesh, const pn_material_table *materials, double dt, int32_t precision,
                          int32_t n_parts, pn_partitioned **out);
int pn_partitioned_add_sources(pn_partitioned *p, const pn_window_source *sources, int32_t n);
int pn_partitioned_set_sensors(pn_partitioned *p, const int32_t *nodes, int32_t n, int32_t capacity_steps);
int pn_partitioned_set_state(pn_partitioned *p, const double *const *V, const double *const *S);
int pn_partitioned_solve(pn_partitioned *p, int32_t nsteps, double *time_out);
int pn_partitioned_get_state(pn_partitioned *p, double *const *V, double *const *S);
int pn_partitioned_get_traces(pn_partitioned *p, double *out, int64_t max_records, int64_t *n_records);
/* partitions, halo node copies, local cells summed over partitions */
int pn_partitioned_info(pn_partitioned *p, int32_t *n_parts, int64_t *halo_nodes, int64_t *local_cells);
int pn_partitioned_destroy(pn_partitioned *p);

/* Blocks of the FP64 grid form's step kernel that took the FP64 path and the
   double-float path since the solver was created (both 0 in other forms).
   No counterpart in the reference: the FP64 form computes each tile in
   double-float arithmetic (48-bit significand, |error| well inside the
   1e-10 contract) unless the tile or a neighbour holds values outside
   double-float's range or a source term this step does, and then in IEEE
   double. */
int pn_solver_path_counts(pn_solver *s, int64_t *fp64_blocks, int64_t *df64_blocks);

/* ---- diagnostics -------------------------------------------------------------
   Issue rates of the arithmetic pipes the step kernels lean on, measured on
   the current device (no counterpart in the reference; a measurement aid for
   choosing an arithmetic form).  Fills min(n, 6) rates in thread-level
   operations per second: [0] FP64 fused multiply-add, [1] FP64 add, [2] FP32
   fused multiply-add, [3] conversion double -> float, [4] conversion float ->
   double (each of [3], [4] alongside two integer instructions), [5] a
   32-bit integer xor + add pair.  Takes about a second and a few MB of
   device memory. */
int pn_measure_pipe_rates(double *rates, int32_t n);

/* Free all device memory of the solver. */
int pn_solver_destroy(pn_solver *s);

#ifdef __cplusplus
}
#endif

#endif /* PANNDE_GB300_H */
