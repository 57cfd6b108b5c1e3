/*
 * lbm_gb300.h - C ABI of the GB300-native lattice Boltzmann engine.
 *
 * The engine replaces the numerical core of the PV2013 solver: STL reading,
 * ray-parity voxelization and boundary classification (class Geometry,
 * ComplexGeometry.h:25-78), lattice construction (class SubDomain,
 * Subdomain.h:63-133) and the BGK time loop with its Zou-He and bounce-back
 * boundaries (class Simulation, Simulation.h:10-44).  The reference exposes a
 * C++ class surface whose constructors do all the work (LBM.cpp:253-256); this
 * header splits the same stages into explicit calls on opaque handles so that
 * any language with a C FFI can bind them.  A header-only C++ facade with the
 * reference's class names sits on top (include/pv2013/pv2013.hpp).
 *
 * Conventions
 *  - Every call returns lbm_status; no exception crosses the ABI.  The
 *    reference printed and continued (GeometryReader.cpp:36-39,
 *    Simulation.cpp:237-239).  lbm_last_error() gives a message for the last
 *    failing call on the calling thread.
 *  - Host buffers are owned by the caller and passed with a capacity.
 *    Buffers returned by the library (lbm_stl_read_*) are released with
 *    lbm_free().
 *  - Grid points are addressed by x-major linear index i*Ny*Nz + j*Nz + k,
 *    the order of the reference's pointsBox loops (ComplexGeometry.cpp:439-441).
 *    Fluid nodes are numbered in the same order (Subdomain.cpp:638-651).
 *  - A handle is not thread-safe; distinct handles are.  GPU work runs on the
 *    stream passed in (a cudaStream_t, given as void*; NULL = legacy stream).
 *  - One GPU per process (the current device at handle creation).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_ABI_VERSION 3

typedef enum lbm_status {
    LBM_OK = 0,
    LBM_ERR_IO = 1,        /* file cannot be opened / written */
    LBM_ERR_PARSE = 2,     /* malformed input file */
    LBM_ERR_NOMEM = 3,     /* host or device allocation failed */
    LBM_ERR_CUDA = 4,      /* a CUDA call failed (message has the CUDA error) */
    LBM_ERR_DIVERGED = 5,  /* divergence monitor tripped (NaN/Inf or mass drift) */
    LBM_ERR_TIMEOUT = 6,   /* a bounded device-side wait gave up */
    LBM_ERR_ARG = 7,       /* invalid argument / size / capacity */
    LBM_ERR_STATE = 8,     /* call not valid in the handle's state */
    LBM_ERR_NODEV = 9      /* no CUDA device, or the kernels are not built for it */
} lbm_status;

/* Message for the last failing call on this thread ("" if none). */
const char* lbm_last_error(void);
/* Static name of a status code. */
const char* lbm_status_string(lbm_status s);
/* Releases a buffer allocated by this library. */
void lbm_free(void* p);
/* ABI version of the loaded library (LBM_ABI_VERSION). */
int lbm_abi_version(void);

/* ------------------------------------------------------------------------ */
/* Triangles.  Same field order as the reference's Triangle (Struct.h:77-82):
 * three vertices then the facet normal as written in the file.             */
typedef struct lbm_tri {
    double x1, y1, z1;
    double x2, y2, z2;
    double x3, y3, z3;
    double nx, ny, nz;
} lbm_tri;

/* ASCII STL reader; replaces Reader::readSTLASCII (GeometryReader.cpp:33-117)
 * with the same facet grammar (a facet counts only when facet/outer loop/3
 * vertex/endloop/endfacet lines parse in sequence) and correctly rounded
 * decimal conversion.  *tris is allocated by the library (lbm_free).       */
lbm_status lbm_stl_read_ascii(const char* path, lbm_tri** tris, size_t* n);

/* The same reader with the parsing on the GPU (no counterpart in the
 * reference, whose reader is GeometryReader.cpp:33-117): the file is copied
 * to the device, facets are located and checked line by line in parallel,
 * and the numbers are converted with exact integer arithmetic (bit-identical
 * to the host reader's correctly rounded conversion).  Files outside the
 * canonical facet layout, or holding a number outside the exact converter's
 * scope (more than 19 significant digits, |decimal exponent| > 27), are
 * parsed by the host grammar instead; *on_device (may be NULL) is 1 when the
 * GPU produced the result.  The result equals lbm_stl_read_ascii's in every
 * case.  Work runs on `stream` (a cudaStream_t, NULL = default stream);
 * LBM_ERR_NODEV without a CUDA device. */
lbm_status lbm_stl_read_ascii_device(const char* path, void* stream, lbm_tri** tris, size_t* n,
                                     int32_t* on_device);
/* Binary STL reader; replaces Reader::readSTLBinary (GeometryReader.cpp:
 * 119-176): float vertices widened to double, normals renormalised in float. */
lbm_status lbm_stl_read_binary(const char* path, lbm_tri** tris, size_t* n);
/* ASCII STL writer (17 significant digits, so a write/read round trip is exact). */
lbm_status lbm_stl_write_ascii(const char* path, const lbm_tri* tris, size_t n, const char* solid_name);

/* ------------------------------------------------------------------------ */
/* Geometry: voxelization and boundary classification on the GPU.
 * Replaces Geometry::Geometry (ComplexGeometry.cpp:7-32).                  */

/* Explicit grid: point (i,j,k) sits at min + (i,j,k)*spacing.  When no grid is
 * given the reference's tight grid is used: bounding box of the triangles,
 * dims = ceil(extent/spacing)+1 (ComplexGeometry.cpp:40-73).               */
typedef struct lbm_grid {
    double min[3];
    int32_t dims[3];
} lbm_grid;

/* Plane predicate selecting boundary points into a list, the form of every
 * test in Geometry::getInOutBP (ComplexGeometry.cpp:579-638):
 *   |p[axis] - plane| <= tol   (evaluated exactly: plane is plane_hi+plane_lo,
 *                               a double-double, so the reference's long
 *                               double constants are represented exactly)
 *   and lo[a] < p[a] < hi[a] for the two other axes (NaN disables a bound).
 * A boundary point may match several lists, as in the reference. */
typedef struct lbm_bc_predicate {
    int32_t list_id;   /* 0..63 */
    int32_t axis;      /* 0=x 1=y 2=z */
    double plane_hi, plane_lo;
    double tol;
    double lo[3], hi[3];
} lbm_bc_predicate;

typedef struct lbm_geometry lbm_geometry;

/* Voxelizes the triangles on the GPU (+z ray parity with the reference's
 * exact FP64 crossing test, ComplexGeometry.cpp:264-330 and :431-506),
 * extracts boundary points (26-neighbourhood, :509-556) and evaluates the
 * predicates (:559-638).  grid may be NULL (tight grid). */
lbm_status lbm_geometry_create(const lbm_tri* tris, size_t ntris, double spacing, const lbm_grid* grid,
                               const lbm_bc_predicate* preds, size_t npreds, void* stream, lbm_geometry** out);
/* The PV2013 preset: the reference's seven hard-coded predicates
 * (ComplexGeometry.cpp:587-633) as list ids 0 (inlet) .. 6 (outlet 6). */
lbm_status lbm_predicates_pv2013(lbm_bc_predicate* out, size_t cap, size_t* n);

typedef struct lbm_geometry_info {
    int32_t dims[3];
    double bbox[6];          /* min_x,max_x,min_y,max_y,min_z,max_z of the grid */
    double spacing;
    int64_t n_points;        /* Nx*Ny*Nz */
    int64_t n_fluid;
    int64_t n_boundary;
    int64_t n_wall;
    int64_t list_size[64];
    int32_t n_lists;         /* 1 + highest list id used */
    double voxelize_ms;      /* device time of the voxelization pass */
    double classify_ms;      /* boundary extraction + predicates */
} lbm_geometry_info;

lbm_status lbm_geometry_info_get(const lbm_geometry* g, lbm_geometry_info* info);
/* Node-type field, 1 = Fluid, 0 = NotFluid, x-major (Nx*Ny*Nz bytes). */
lbm_status lbm_geometry_flags(const lbm_geometry* g, uint8_t* host_out, size_t cap);
/* Ordered boundary-point lists as x-major linear indices.
 * list = LBM_LIST_BOUNDARY: every boundary point (findBoundaryPoints order);
 * list = LBM_LIST_WALL: boundary points in no predicate list (excludeInletOutlet);
 * list = 0..63: points matching that predicate list (getInOutBP order). */
#define LBM_LIST_BOUNDARY (-1)
#define LBM_LIST_WALL (-2)
lbm_status lbm_geometry_list(const lbm_geometry* g, int32_t list, int64_t* host_out, size_t cap, size_t* n);
void lbm_geometry_destroy(lbm_geometry* g);

/* ------------------------------------------------------------------------ */
/* Simulation.  Replaces SubDomain::SubDomain (Subdomain.cpp:3-33) and
 * Simulation::Simulation/Iterate (Simulation.cpp:3-13, 903-932).           */

typedef enum lbm_precision {
    LBM_F64 = 0,     /* FP64 storage and math: bit-exact with the reference's step */
    LBM_F32 = 1,     /* FP32 storage, FP32 math */
    LBM_F16S = 2,    /* FP16 storage of (f - w)*2^15, FP32 math */
    LBM_BF16S = 3    /* BF16 storage of (f - w), FP32 math */
} lbm_precision;

typedef enum lbm_pattern {
    LBM_PULL = 0,    /* two-lattice pull */
    LBM_AA = 1,      /* AA in-place (one lattice) */
    LBM_AUTO = 2     /* chosen by the autotuner */
} lbm_pattern;

/* Boundary-condition kinds: the reference's own routines, each for the one
 * face orientation the reference wrote it for (five D3Q19 routines, one
 * D3Q27 routine). */
typedef enum lbm_bc_kind {
    LBM_BC_NONE = 0,            /* list is treated as wall */
    LBM_BC_VEL_NEGY = 1,        /* Boundary::ApplyBc D3Q19, Boundary.cpp:129-148: unknowns -y */
    LBM_BC_PRESS_NEGY = 2,      /* ApplyOutletBc list 1, Simulation.cpp:966-1019: unknowns -y */
    LBM_BC_PRESS_POSY = 3,      /* ApplyOutletBc list 2, Simulation.cpp:1029-1083: unknowns +y */
    LBM_BC_PRESS_POSX = 4,      /* ApplyOutletBc lists 3-5, Simulation.cpp:1093-1279: unknowns +x
                                   (keeps the reference's f10 in place of f16 in Nxz) */
    LBM_BC_PRESS_POSZ = 5,      /* ApplyOutletBc list 6, Simulation.cpp:1290-1346: unknowns +z */
    LBM_BC_VEL_POSX = 6,        /* Boundary::ApplyBc D3Q27, Boundary.cpp:87-123: unknowns +x (Q=27) */
    LBM_BC_VELOCITY = 7,        /* any face, Q=19 or 27: the reference's velocity routine with the
                                   axes relabelled (face field of lbm_list_bc) */
    LBM_BC_PRESSURE = 8         /* any face, Q=19 or 27: the reference's pressure routine with the
                                   axes relabelled; for D3Q27, which has no pressure routine in
                                   the reference, its velocity routine's coefficients */
} lbm_bc_kind;

/* Face of the LBM_BC_VELOCITY / LBM_BC_PRESSURE kinds: the unknown populations
 * are those with c along this signed axis (the inlet at the top of a vessel
 * running along -y has unknowns -y: LBM_FACE_NEGY). */
typedef enum lbm_face {
    LBM_FACE_POSX = 0, LBM_FACE_NEGX = 1, LBM_FACE_POSY = 2,
    LBM_FACE_NEGY = 3, LBM_FACE_POSZ = 4, LBM_FACE_NEGZ = 5
} lbm_face;

/* Per-list boundary setting.  Velocity lists: the velocity of list node m at
 * step t is (amp[t mod amp_len] * profile[m]) * dir, computed in FP64
 * (profile NULL = 1 for every node, amp NULL = constant 1).  Pressure lists:
 * density rho. */
typedef struct lbm_list_bc {
    int32_t list_id;
    int32_t kind;              /* lbm_bc_kind */
    double rho;                /* outlet density (the reference hard-codes 1.01, Simulation.cpp:954) */
    double dir[3];             /* inlet velocity direction, components in {-1,0,1} */
    const double* profile;     /* per-node factor in list order, or NULL */
    size_t profile_len;
    const double* amp;         /* amplitude per step (periodic), or NULL */
    size_t amp_len;
    int32_t face;              /* lbm_face, for LBM_BC_VELOCITY and LBM_BC_PRESSURE */
    int32_t reserved;
} lbm_list_bc;

typedef struct lbm_sim_params {
    int32_t Q;                 /* 19 or 27 */
    int32_t precision;         /* lbm_precision */
    int32_t pattern;           /* lbm_pattern */
    double tau;                /* relaxation time; omega = 1/tau (Simulation.cpp:11) */
    const lbm_list_bc* bcs;
    size_t nbcs;
    int32_t warps_per_block;   /* 1..8; 0 = default (4, or 1 for nodes_per_lane 2) */
    int32_t run_axis;          /* node numbering axis (chunks are runs along it):
                                  1 = y, 2 = z (the reference's x-major order),
                                  0 = the one giving fewer chunks */
    int32_t staging;           /* 0 = TMA-staged pipeline (default), 1 = direct loads */
    int32_t nodes_per_lane;    /* 1 = one node per lane (staging applies);
                                  2 = two adjacent nodes per lane with packed
                                      FP32 arithmetic (FP32 and 16-bit storage,
                                      direct loads); 0 = default: 2 for FP32
                                      and 16-bit storage, 1 for FP64 */
    int32_t corrections;       /* 0 = the reference's behaviour (parity mode); bits:
                                  LBM_FIX_BB_ALL_DIRS: bounce back every moving direction
                                    (the reference skips direction 0, Simulation.cpp:1361);
                                  LBM_FIX_LIST_NODES: bounce back the missing populations of
                                    inlet/outlet nodes before their Zou-He routine (the
                                    reference leaves them at their initial value) */
    int32_t piece_slots;       /* two nodes per lane: node slots per chunk piece (8, 16 or 32;
                                  a piece is one run segment served by piece_slots/2 lanes,
                                  so shorter pieces leave fewer idle lanes at run ends and
                                  read more descriptor bytes); 0 = default (8).  Results do
                                  not depend on it. */
} lbm_sim_params;

#define LBM_FIX_BB_ALL_DIRS 1
#define LBM_FIX_LIST_NODES 2

typedef struct lbm_sim lbm_sim;

/* Builds the device lattice from a geometry: node typing by first match in
 * list order then wall (Subdomain.cpp:399-477), neighbour structure
 * (Subdomain.cpp:481-505, here run tables instead of pointers) and the
 * initial state f = w (Node.cpp:30-37). */
lbm_status lbm_sim_create(const lbm_geometry* g, const lbm_sim_params* p, void* stream, lbm_sim** out);

/* Ensemble: n independent lattices advanced by one launch per step
 * (one packed node list, per-instance tau and boundary settings). */
lbm_status lbm_batch_create(const lbm_geometry* const* g, const lbm_sim_params* p, size_t n, void* stream,
                            lbm_sim** out);

/* Advances nsteps time steps.  One step is one Iterate() body of the
 * reference: Collision, Streaming, ApplyZouHeBc, ApplyWallBc, ApplyOutletBc
 * (Simulation.cpp:909-915), fused into one kernel launch per step. */
#define LBM_STEP_GRAPH 1u      /* replay the steps as a captured CUDA graph */
#define LBM_STEP_MONITOR 2u    /* run the divergence monitor after the last step */
lbm_status lbm_sim_step(lbm_sim* s, int64_t nsteps, uint32_t flags, void* stream);
/* Captures now the CUDA graph a later lbm_sim_step(s, nsteps, LBM_STEP_GRAPH)
 * from the current state replays (at most 64 launches long), so that call
 * spends no time on the capture.  The state does not change; a call with
 * another step count may capture again.  No counterpart in the reference. */
lbm_status lbm_sim_prepare_graph(lbm_sim* s, int64_t nsteps, void* stream);

typedef struct lbm_sim_info {
    int64_t n_nodes;
    int64_t n_instances;
    int64_t steps_done;
    int64_t n_chunks;          /* chunks of the step kernel in use */
    int32_t Q, precision, pattern, warps_per_block, run_axis;
    int64_t state_bytes;       /* device bytes of the population arrays */
    double algorithmic_bytes_per_update;  /* 2*Q*storage bytes */
    int64_t n_lattice_nodes;   /* fluid + ghost nodes (the population arrays' length) */
    int32_t nodes_per_lane;
    int32_t piece_slots;       /* node slots per chunk piece (two nodes per lane), else 0 */
} lbm_sim_info;
lbm_status lbm_sim_info_get(const lbm_sim* s, lbm_sim_info* info);

/* Autotuner: times every step-kernel variant the handle can run -- one node
 * per lane with direct loads or TMA staging, two nodes per lane (FP32 and
 * 16-bit storage) with 8-, 16- and 32-slot pieces, each with 1, 2, 4 and 8
 * warps per block, in the current streaming pattern and in the other one
 * where the state converts now (lbm_sim_set_pattern) and its memory fits --
 * for `launches` launches on scratch copies of the state (the simulation does
 * not advance), and keeps the fastest for later steps (converting the state
 * when the pattern changes; results are unchanged).  The layout (structure
 * of arrays) is not a candidate: a blocked layout measured 6 % slower.
 * entries (may be NULL) receives up to cap results, *n (may be NULL) their
 * number.  Needs device memory for one or two more copies of the populations
 * (LBM_ERR_NOMEM otherwise, nothing changed). */
typedef struct lbm_tune_entry {
    int32_t nodes_per_lane, staging, warps_per_block, chosen;
    int32_t pattern;           /* lbm_pattern of the candidate */
    int32_t piece_slots;       /* two nodes per lane: node slots per piece, else 0 */
    double ms_per_launch;
} lbm_tune_entry;
lbm_status lbm_sim_autotune(lbm_sim* s, int32_t launches, void* stream, lbm_tune_entry* entries, size_t cap,
                            size_t* n);

/* Host copies of the current post-boundary state f_n (the reference's
 * m_distributions after n iterations) and of rho, u computed from it with the
 * reference's collision formulas (Simulation.cpp:32-79).  Node order.  Any
 * pointer may be NULL.  For a batch, nodes of all instances are concatenated. */
lbm_status lbm_sim_fields(lbm_sim* s, double* rho, double* u, double* f, size_t n_nodes, void* stream);
/* rho and u as lbm_sim_fields gives them, for callers that must not allocate
 * device memory: the library writes them into one fixed device array of its
 * own (at most 524288 nodes; larger lattices: LBM_ERR_ARG) and copies them to
 * the caller's buffers, with no device allocation (neither the driver's
 * allocator nor the library's memory pool, which lbm_sim_fields draws on
 * and may grow).  The array is shared
 * by every call and keeps the last call's values, so calls whose GPU work
 * overlaps race.  The handle's device must be current.  The call
 * synchronises `stream` before it returns, so it cannot be used inside a
 * stream capture; the first call on a device may load the library's device
 * module.  No counterpart in the reference. */
lbm_status lbm_sim_fields_noalloc(lbm_sim* s, double* rho, double* u, size_t n_nodes, void* stream);
/* Node positions: x-major grid index of every node (per instance, concatenated). */
lbm_status lbm_sim_nodes(const lbm_sim* s, int64_t* grid_index, size_t cap);
/* First node of each instance (n_instances+1 offsets). */
lbm_status lbm_sim_instance_offsets(const lbm_sim* s, int64_t* off, size_t cap);

typedef struct lbm_monitors {
    int64_t step;
    double mass;               /* FP64 sum of rho over all nodes */
    double inlet_flux;         /* FP64 sum over velocity-boundary nodes of rho*|u| */
    double outlet_flux;        /* FP64 sum over pressure-boundary nodes of rho*|u| */
    double max_speed;
    int32_t nonfinite;         /* 1 if any rho/u was NaN or Inf */
} lbm_monitors;
/* Computes the monitors of the current state (FP64 device reductions). */
lbm_status lbm_sim_monitors(lbm_sim* s, lbm_monitors* out, void* stream);
/* Checkpoint / restart: the current populations and step count, written to
 * a file; lbm_sim_restart loads one into a handle built from the same
 * geometry and parameters (checked: lattice size, storage, pattern and a hash
 * of the node positions), after which stepping continues exactly as it would
 * have from the checkpointed state.  Replaces nothing in the reference (it
 * has no restart); writes whole files, synchronises the stream. */
lbm_status lbm_sim_checkpoint(lbm_sim* s, const char* path, void* stream);
lbm_status lbm_sim_restart(lbm_sim* s, const char* path, void* stream);

/* Divergence monitor used with LBM_STEP_MONITOR: the step call returns
 * LBM_ERR_DIVERGED when a value is non-finite or |mass/mass0 - 1| > rel_tol. */
lbm_status lbm_sim_set_divergence_tolerance(lbm_sim* s, double rel_tol);

/* Poll limit of the bounded waits in the TMA-staged step kernel (staging 0):
 * a warp that tests a stage's mbarrier this many times (non-blocking tests)
 * without the staged copies arriving stops, after draining its copies in flight, and the next
 * monitor, fields or checkpoint call returns LBM_ERR_TIMEOUT (once; the
 * state is then incomplete).  0 restores the default (2^22 polls).  The
 * reference has no counterpart: its exchange errors print and continue
 * (Simulation.cpp:237-239). */
lbm_status lbm_sim_set_wait_limit(lbm_sim* s, uint32_t polls);

/* Failure-test hook (no counterpart in the reference): while enabled, the
 * TMA-staged step kernel leaves each warp's first stage unissued, so that
 * stage's bounded wait runs out (no copy is in flight on it) and the next
 * monitor, fields or checkpoint call reports LBM_ERR_TIMEOUT.  The state of
 * such a step is incomplete; restore it (lbm_sim_restart) after disabling. */
lbm_status lbm_sim_test_stall(lbm_sim* s, int32_t enable);

/* Self-check hook (no counterpart in the reference): fills every population
 * slot that belongs to no fluid node -- the ghost layer, the padding of the
 * pair alignment, the slack at both ends of the arrays -- with NaN, in every
 * plane of every lattice buffer.  No kernel may use such a value (a read of a
 * ghost slot is a missing population, replaced by the boundary rule), so a
 * correct build gives bit-identical results after it. */
lbm_status lbm_sim_poison_ghosts(lbm_sim* s, void* stream);

/* Converts the state to another streaming pattern (LBM_PULL or LBM_AA); the
 * run continues with the same results.  After an AA even (node-local)
 * launch the AA state is the pull state with its population planes
 * permuted, so AA -> pull needs that state (an odd number of steps done
 * since the AA run started; LBM_ERR_STATE otherwise) and memory for the
 * second lattice; pull -> AA always works and frees one lattice.  No
 * counterpart in the reference, which has one streaming scheme
 * (Simulation.cpp:184-198). */
lbm_status lbm_sim_set_pattern(lbm_sim* s, int32_t pattern, void* stream);

void lbm_sim_destroy(lbm_sim* s);

/* ------------------------------------------------------------------------ */
/* Output: wall shear stress and VTK snapshots (OutputFile.cpp:16-137).      */

/* Wall shear stress of the current state at every wall node, in the wall
 * list's order (lbm_geometry_list(LBM_LIST_WALL), instances concatenated):
 * |mu g| with g the mean of u(x + c_q) - u(x) over the neighbours that are
 * fluid points (q = 0..Q-1, the rest direction included) and
 * mu = (2 tau - 1)/6 (Simulation.cpp:1374-1421).  u is the velocity of the
 * current populations -- the value the reference's next Collision stores, so
 * after n steps this is the reference's wall shear stress of iteration n.
 * wss may be NULL to query *n. */
lbm_status lbm_sim_wall_shear_stress(lbm_sim* s, double* wss, size_t cap, size_t* n, void* stream);

/* Point-data .vtu writer: n points (xyz, 3 floats each), VTK_VERTEX cells,
 * Float64 arrays; raw appended binary. */
typedef struct lbm_vtu_array {
    const char* name;
    int32_t components;
    int32_t reserved;
    const double* data;        /* n * components values */
} lbm_vtu_array;
lbm_status lbm_vtu_write(const char* path, size_t n, const float* xyz, size_t narrays, const lbm_vtu_array* arrays);

/* Asynchronous snapshots.  lbm_snapshot_capture enqueues, on the caller's
 * stream, one snapshot launch of the current state (rho, u and, with
 * LBM_SNAP_WSS, the wall shear stress) into device buffers of the snapshot,
 * then copies them to the snapshot's pinned host buffers on a stream of its
 * own and returns: the simulation can keep stepping on its stream while the
 * copy runs.  lbm_snapshot_wait blocks until the host buffers hold the
 * capture; the write functions wait, then write the reference's files:
 *   fields: points at the nodes' lattice indices, x fastest (the loop order of
 *           WriteVTK_LocalData), arrays Velocity, Pressure (c_s^2 rho),
 *           VelocityMagnitude, Density -- all of the captured state (the
 *           reference's Pressure is summed from the populations one step
 *           later than its other arrays, OutputFile.cpp:64);
 *   wss:    the wall nodes in wall-list order, array WallShearStress.
 * One capture in flight per snapshot; a batch writes one instance per file. */
#define LBM_SNAP_FIELDS 1
#define LBM_SNAP_WSS 2
typedef struct lbm_snapshot lbm_snapshot;
lbm_status lbm_snapshot_create(lbm_sim* s, uint32_t what, lbm_snapshot** out);
lbm_status lbm_snapshot_capture(lbm_snapshot* snap, void* stream);
lbm_status lbm_snapshot_wait(lbm_snapshot* snap);
/* Host views of the last capture (valid until the next capture or destroy). */
lbm_status lbm_snapshot_data(lbm_snapshot* snap, const double** rho, const double** u, const double** wss,
                             size_t* n_nodes, size_t* n_wall, int64_t* step);
lbm_status lbm_snapshot_write_fields_vtu(lbm_snapshot* snap, const char* path, int32_t instance);
lbm_status lbm_snapshot_write_wss_vtu(lbm_snapshot* snap, const char* path, int32_t instance);
void lbm_snapshot_destroy(lbm_snapshot* snap);

/* ------------------------------------------------------------------------ */
/* Synthetic geometry generators (seeded, deterministic).                    */

/* Triangulated cylinder: radius r, length len, `segments` facets around,
 * axis 0/1/2, centred at c; caps are triangle fans.  Vertices are placed at
 * half-segment angles so no side facet is axis-aligned. */
lbm_status lbm_synth_cylinder(double r, double len, int32_t segments, int32_t axis, const double c[3],
                              lbm_tri** tris, size_t* n);

/* Union of capsules meshed as one watertight surface by marching tetrahedra
 * on a grid of pitch h over [lo, hi] (grid origin shifted by a seeded jitter
 * below h/100 so mesh vertices avoid lattice lines).  seg holds nseg records
 * of 10 doubles: ax,ay,az, bx,by,bz, r, cut_axis, cut_pos, cut_sign.  With
 * cut_axis in {0,1,2} that capsule alone is clipped to the half-space
 * cut_sign*(p[cut_axis]-cut_pos) <= 0, which gives a flat, axis-aligned inlet
 * or outlet face; cut_axis = -1 leaves it whole. */
lbm_status lbm_synth_capsules(const double* seg, size_t nseg, const double lo[3], const double hi[3], double h,
                              uint64_t seed, lbm_tri** tris, size_t* n);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
