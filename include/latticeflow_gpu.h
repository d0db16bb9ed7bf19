/*
 * latticeflow_gpu.h -- C ABI of the GB300 lattice max-flow engine.
 *
 * Plain pointers and sizes only; every entry point returns an LF_* status
 * code (0 = LF_OK) unless noted, and lf_last_error() gives the message of the
 * last failure on the calling thread.  One handle owns one CUDA stream and
 * all of its device state; a handle is not thread-safe, different handles are
 * independent.  All array arguments are HOST pointers unless the name ends in
 * _device.
 *
 * Each entry point names the reference interface it replaces (paths within
 * the latticeflow project).
 */
#ifndef LATTICEFLOW_GPU_H
#define LATTICEFLOW_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The C++ adapter turns LF_ERR_BAD_NAME into
 * BadSolverOrKernelName (solver/interface.hpp:152-168) and LF_ERR_RANGE from
 * the TV path into std::out_of_range (solver/tv/tv_solver.hpp:202-206). */
enum {
  LF_OK = 0,
  LF_ERR_BAD_NAME = 1,       /* unknown solver or kernel name               */
  LF_ERR_SHAPE = 2,          /* dimension count / sizes do not fit          */
  LF_ERR_RANGE = 3,          /* value outside the representable range,
                                non-submodular pairwise term, bad lambda     */
  LF_ERR_NO_CONVERGENCE = 4, /* an iteration cap was reached                */
  LF_ERR_OOM = 5,            /* device allocation failed                    */
  LF_ERR_CUDA = 6,           /* other CUDA runtime error                    */
  LF_ERR_INVALID = 7,        /* null handle / pointer, bad argument         */
  LF_ERR_STATE = 8           /* call out of order (e.g. getCut before run)  */
};

typedef struct lf_lattice lf_lattice;

/* Last error message on this thread ("" if none). */
const char* lf_last_error(void);

/* ------------------------------------------------------------------ factory
 * solver/interface.hpp:170-191 and the generated factory
 * (install/templates/factory/file.cpp:26-95).  Solver names accepted:
 *   "LatticeEnergyMinimizer"  binary cut (energy.hpp:39-49)       -> GPU push-relabel
 *   "LatticeLevelReductions"  parametric flow (pf_policies.hpp:31-46) -> GPU parametric flow
 *   "GPUPushRelabel", "GPULevelReductions"  the same engines under GB300 names.
 * Kernel names follow install/code_setup.py:40 ("Full2d_4", "Star2d_16",
 * "Full3d_6", ...); "Full3d_26" is the 3x3x3 neighbourhood. */
int lf_is_valid_solver(const char* name);           /* 1 / 0 */
int lf_is_valid_kernel(const char* name);           /* 1 / 0 */
int lf_kernel_dimension(const char* kernel);        /* interface.hpp:189; -1 if unknown */
/* Writes '\n'-separated names into buf (size len), returns the needed length. */
size_t lf_valid_kernel_names(char* buf, size_t len);  /* interface.hpp:190 */
size_t lf_valid_solver_names(char* buf, size_t len);  /* interface.hpp:191 */
/* Kernel table in lattice order (kernellattice.hpp:61-96): K offsets, the
 * positive half first in ascending linear-jump order, entry i + K/2 the
 * reverse of entry i.  deltas: K*nd ints, geocut_weights: K doubles (either
 * may be NULL).  Returns K, or -1 for an unknown name. */
int lf_kernel_info(const char* kernel, int* nd, int* deltas, double* geocut_weights,
                   int* geocut_applicable);

/* getLatticeFlowInterface(solver, kernel, dims...) (interface.hpp:170-184).
 * nd must equal the kernel's dimension; dims row-major, last fastest. */
int lf_create(const char* solver, const char* kernel, int nd, const size_t* dims,
              lf_lattice** out);
void lf_destroy(lf_lattice* h);

/* ----------------------------------------------------- lattice metadata
 * interface.hpp:25-44. */
int lf_n_dimensions(const lf_lattice* h);
int lf_shape(const lf_lattice* h, size_t* dims_out);
size_t lf_n_nodes(const lf_lattice* h);
int lf_n_filling_edges(const lf_lattice* h);
/* edgeDeltas(): K/2 * nd ints, entry [i*nd + j] = offset of filling edge i in dim j. */
int lf_edge_deltas(const lf_lattice* h, int* deltas_out);

/* -------------------------------------------------------------- filling
 * addEnergyPotentials(long* unary, long* binary) (interface.hpp:49-61,
 * direct_interface.hpp:60-95).  unary: 2*N int64 (E0 = off, E1 = on per
 * node), binary: N*(K/2)*4 int64 (E00, E01, E10, E11 per node and filling
 * edge; E01 = source node off, destination on).  Edges leaving the lattice are
 * ignored.  Repeated calls accumulate.  Pairwise terms must be submodular
 * (E00 + E11 <= E01 + E10, network_flow_node.hpp:450) -> else LF_ERR_RANGE. */
int lf_add_energy_potentials(lf_lattice* h, const int64_t* unary, const int64_t* binary);
/* Same, with the two arrays already in device memory (no host copy). */
int lf_add_energy_potentials_device(lf_lattice* h, const int64_t* unary_device,
                                    const int64_t* binary_device);
/* Capacity form of the fill (the intent of addCapacityFromSource /
 * addCapacityToSink / addCapacityOfEdge, energy_base.hpp:51-105):
 * source[N] = cost of the node being off, sink[N] = cost of it being on,
 * edge[N*(K/2)] = symmetric capacity of each filling edge.  int32, >= 0.
 * Any pointer may be NULL.  Accumulates. */
int lf_add_capacities(lf_lattice* h, const int32_t* source, const int32_t* sink,
                      const int32_t* edge);

/* --------------------------------------------------------------- control
 * run() / runTime() (interface.hpp:111-113).  runTime is the device-side
 * solve time of the last run in seconds (CUDA events), not CPU time. */
int lf_run(lf_lattice* h);
double lf_run_time(const lf_lattice* h);

/* ---------------------------------------------------------------- results
 * getCut() (interface.hpp:120, direct_interface.hpp:97-106): int[N], 1 = on.
 * For the binary cut this is the unique MINIMAL on-set (forward residual
 * reachability from the excess nodes; equals the bundled BK solver's
 * labelling).  For the parametric solver it is reduction < 0
 * (network_flow_node.hpp:50-55 with on_by_reduction). */
int lf_get_cut(const lf_lattice* h, int* cut_out);
/* The unique MAXIMAL on-set (nodes that cannot reach a deficit node). */
int lf_get_cut_max(const lf_lattice* h, int* cut_out);
/* Max-flow value and the minimum energy E(cut), both int64. */
int lf_get_flow(const lf_lattice* h, int64_t* flow, int64_t* energy);
/* Parametric solver: final 2x-scaled node values r (pf_flow_node.hpp:233-235). */
int lf_get_levels(const lf_lattice* h, int64_t* r_out);
/* Parametric solver: the level set of every node (int[N], row-major), the
 * level sets numbered in the order ParametricFlowSolver::run returns them
 * (parametricflow/pf_solver.hpp:180-203). */
int lf_get_level_sets(const lf_lattice* h, int32_t* sets_out);
/* Statistics of the last run: epochs (global relabels), push-relabel
 * launches, BFS passes.  Any pointer may be NULL. */
int lf_get_stats(const lf_lattice* h, int64_t* epochs, int64_t* pr_launches,
                 int64_t* bfs_passes);

/* Zero the accumulated energies: the lattice is as freshly created (the
 * reference builds a new interface object per problem). */
int lf_clear(lf_lattice* h);

/* --------------------------------------------------------------- profiling
 * With profiling on, every kernel launch of run() is bracketed by CUDA
 * events on the handle's stream.  lf_get_profile fills
 *   ms[0] push/relabel tile kernels, ms[1] global-relabel passes,
 *   ms[2] cut-set closure passes, ms[3] whole run (device time)
 *   counts[0] push/relabel launches, counts[1] tiles processed by them,
 *   counts[2] BFS passes, counts[3] closure passes,
 *   counts[4] kernel launches since the handle was created (fills included),
 *   counts[5] tiles processed by BFS.
 * (ms: 4 doubles, counts: 6 int64.) */
int lf_set_profiling(lf_lattice* h, int enable);
int lf_get_profile(const lf_lattice* h, double* ms, int64_t* counts);
/* Device layout of the last run: tile extents (3, C fastest; a 2-d lattice
 * is 1 x nx x ny), padded extents (3) and working capacity bytes (4 or 8). */
int lf_get_layout(const lf_lattice* h, int* tile_dims, size_t* padded_dims, int* elem_bytes);
/* The handle's CUDA stream (a cudaStream_t), so that callers can order or
 * time their own work against the solver's. */
int lf_get_stream(const lf_lattice* h, void** stream_out);

/* --------------------------------------------------------------- tuning
 * Runtime knobs of the solve (tile rows, local sweeps per launch, launches
 * per global relabel); 0 keeps the current/auto value. */
int lf_set_tuning(lf_lattice* h, int tile_rows, int local_sweeps, int launches_per_relabel);
/* One knob by name: "tile_rows", "local_sweeps", "launches_per_relabel",
 * "height_slack", "pass_chunk", "tail_active" (at most this many active
 * nodes switch an epoch to routing their excess along BFS trees; 0 = 64,
 * negative = never), "tail_tree_nodes" (nodes of one such tree at most;
 * 0 = 65,536), "max_epochs" (global relabels per solve before the
 * solve gives up with LF_ERR_NO_CONVERGENCE; 0 = 1,000,000; the handle stays
 * usable), "pr_kernel" (push/relabel pass of 2-d 3x3 lattices: 0 = staged by
 * bulk tensor copies, 40 registers; 1 = generic tile kernel; 2 = staged, 32
 * registers; 3 = staged, one warp per tile, launched one pass at a time; 3-d
 * lattices with a radius-1 neighbourhood: 0, 2 and 3 = staged, 1 = generic),
 * "bfs_kernel" (global-relabel pass of those lattices: 0 =
 * staged, 1 = generic), "device_loops" (1 = the staged passes of a relabel or
 * an epoch run as one CUDA graph with a device-side loop; 0 = one launch per
 * pass, the default), "fill_kernel" (energy fill of device-resident arrays:
 * 0 = gathered with one lane per filling edge, 1 = gathered per node, 2 =
 * scattered with atomics, the form always used for pinned host arrays read
 * in place), "host_stage" (pinned host energies: 0 = read in place by the
 * fill kernel, the default; 1 = copied into device memory by the copy
 * engine first, then filled from there).  Results never depend on these.
 * LF_ERR_INVALID for an unknown name. */
int lf_set_param(lf_lattice* h, const char* name, int value);

/* -------------------------------------------------------------- batches
 * Many independent lattices of uneven shapes solved together: one instance
 * pool, every pass of the solve one launch over the queued tiles of ALL
 * lattices.  No reference counterpart (the reference solves one lattice per
 * interface object); each lattice's results equal a plain solve of it.
 * Lattices are added before the first fill; a batch mixes at most two kernel
 * sizes (Full2d_4 with Full2d_8).  Fill and result calls take the lattice
 * index returned by lf_batch_add. */
typedef struct lf_batch lf_batch;
int lf_batch_create(lf_batch** out);
void lf_batch_destroy(lf_batch* b);
int lf_batch_add(lf_batch* b, const char* kernel, int nd, const size_t* dims, int* index_out);
int lf_batch_size(const lf_batch* b);
int lf_batch_add_energy_potentials(lf_batch* b, int index, const int64_t* unary,
                                   const int64_t* binary);
int lf_batch_add_capacities(lf_batch* b, int index, const int32_t* source, const int32_t* sink,
                            const int32_t* edge);
/* Every lattice's capacities at once: source / sink hold all lattices' nodes
 * back to back in index order (sum of N_i ints each), edge all lattices'
 * filling edges (sum of N_i * K_i/2 ints); any pointer may be NULL.  One
 * copy per array instead of one call per lattice.  Accumulates. */
int lf_batch_add_capacities_packed(lf_batch* b, const int32_t* source, const int32_t* sink,
                                   const int32_t* edge);
/* Every lattice's minimal (maximal = 0) or maximal (maximal = 1) on-set,
 * back to back in index order (sum of N_i ints). */
int lf_batch_get_cuts_packed(lf_batch* b, int* cuts_out, int maximal);
/* Every lattice's flow value and minimum energy (lf_batch_size entries each;
 * either pointer may be NULL). */
int lf_batch_get_flows(lf_batch* b, int64_t* flows, int64_t* energies);
int lf_batch_clear(lf_batch* b);
int lf_batch_run(lf_batch* b);
double lf_batch_run_time(const lf_batch* b);
int lf_batch_get_cut(lf_batch* b, int index, int* cut_out);
int lf_batch_get_cut_max(lf_batch* b, int index, int* cut_out);
int lf_batch_get_flow(lf_batch* b, int index, int64_t* flow, int64_t* energy);
int lf_batch_set_param(lf_batch* b, const char* name, int value);
/* epochs, push/relabel passes, BFS passes of the last run */
int lf_batch_get_stats(const lf_batch* b, int64_t* epochs, int64_t* pr_passes, int64_t* bfs_passes);

/* -------------------------------------------------------------- serving
 * No reference counterpart.  A request server for TV-denoise (single lambda)
 * and graph-cut requests of any 2-d size: requests are queued as submitted
 * and admitted when a worker is idle and their device footprint fits in the
 * HBM budget still free (budget 0 = half the free device memory; a request
 * larger than the budget runs alone).  Admitted requests run concurrently
 * on the workers' own CUDA streams, so their kernels overlap on the device;
 * each worker keeps the engines of the shapes it has served.  TV requests
 * of one kernel and shape that wait together are solved as one stacked
 * problem (continuous batching, groups of 1, 2, 4, ... up to max_group,
 * default 8); each result equals the request's own solve.  Inputs are
 * copied at submission; results stay until lf_server_release.  Latency =
 * completion - submission (queueing included). */
typedef struct lf_server lf_server;
int lf_server_create(int workers, size_t hbm_budget_bytes, lf_server** out);
void lf_server_destroy(lf_server* s);
int lf_server_submit_tv(lf_server* s, const char* kernel, size_t nx, size_t ny, const double* f,
                        double lambda, int64_t* ticket);
int lf_server_submit_cut(lf_server* s, const char* kernel, size_t nx, size_t ny,
                         const int32_t* source, const int32_t* sink, const int32_t* edge,
                         int64_t* ticket);
/* LF_OK when finished (latency_s set), LF_ERR_STATE on timeout, else the
 * request's own error. */
int lf_server_wait(lf_server* s, int64_t ticket, double timeout_s, double* latency_s);
int lf_server_get_tv(lf_server* s, int64_t ticket, double* out, int64_t* levels);
int lf_server_get_cut(lf_server* s, int64_t ticket, int* cut, int64_t* flow, int64_t* energy);
int lf_server_release(lf_server* s, int64_t ticket);
/* Drop a request that is still queued: its wait then returns LF_ERR_STATE
 * ("request cancelled").  LF_ERR_STATE if it was admitted already. */
int lf_server_cancel(lf_server* s, int64_t ticket);
/* Host-side fault injection: the next `count` engine creations of the
 * workers fail as a failed device allocation would; the request that needed
 * the engine finishes with LF_ERR_OOM and the server carries on. */
int lf_server_inject_alloc_failures(lf_server* s, int count);
int lf_server_stats(lf_server* s, double* p50_ms, double* p99_ms, double* solves_per_s,
                    int64_t* completed, int64_t* max_in_flight);
/* max_group = 1 turns grouping off. */
int lf_server_set_max_group(lf_server* s, int max_group);
/* groups: stacked solves run so far; grouped: requests they held. */
int lf_server_group_stats(lf_server* s, int64_t* groups, int64_t* grouped);

/* ------------------------------------------------------ no allocation
 * No counterpart in the reference.  A binary cut of one small 2-d lattice
 * (Full2d_4 / Full2d_8 and their Star aliases, int32 capacities) that
 * allocates no memory: for callers that must not allocate device memory
 * while they run -- code living inside another framework's memory budget or
 * pool, real-time or embedded hosts that forbid allocation after start-up,
 * plugins whose host process owns every allocation.  Inputs and outputs are
 * the caller's DEVICE buffers: source/sink[nx*ny] and edge[nx*ny*(K/2)]
 * capacities as lf_add_capacities, cut[nx*ny] receives the minimal on-set
 * (as lf_get_cut), flow_energy[2] the flow value and the minimum energy.
 * All intermediate state lives in one static device array of 8.5 MiB per GPU,
 * enough for 65,536 padded nodes (sides rounded up to 32, e.g. 256 x 256);
 * larger lattices return LF_ERR_RANGE.  Every call looks the array's device
 * address up; the first call on a device also loads the array there (make
 * that first call before any stream capture).  The array is shared by all
 * calls and keeps the last call's contents; each call clears what must start
 * at zero.  Calls whose GPU work overlapped would race on it: the call holds
 * a process-wide lock and synchronises `stream` (a cudaStream_t, NULL =
 * legacy default stream) before returning, on error returns too. */
int lf_cut_2d_noalloc(const char* kernel, size_t nx, size_t ny, const int32_t* source_device,
                      const int32_t* sink_device, const int32_t* edge_device,
                      int32_t* cut_device, int64_t* flow_energy_device, void* stream);

/* ------------------------------------------------------------------- TV
 * calculate2dTV<Kernel, int64>(nx, ny, f, lambda) (tv/tv_solver.hpp:650-655):
 * the single-lambda TV solve on the GPU.  f, out: nx*ny doubles, row-major.
 * levels_out (may be NULL): the final 2x-scaled fixed-point values r. */
int lf_tv_2d(const char* kernel, size_t nx, size_t ny, const double* f, double lambda,
             double* out, int64_t* levels_out);
/* The same, also giving the level set of every pixel (sets_out: nx*ny
 * int32, may be NULL), numbered in the order the reference's parametric
 * solver returns them (parametricflow/pf_solver.hpp:180-203). */
int lf_tv_2d_level_sets(const char* kernel, size_t nx, size_t ny, const double* f,
                        double lambda, double* out, int64_t* levels_out, int32_t* sets_out);

/* calculate2dTV<Kernel, int64>(nx, ny, f, vector<double> lambdas)
 * (tv/tv_solver.hpp:657-681): the reference's regularisation path,
 * out[n_lambda][nx][ny].  Solved once at the largest lambda, then tracked
 * downwards with the reference's event heap of region segments (joins,
 * splits found by region max-flow probes and integer bisection,
 * tv/tv_regpath_node.hpp), the probes and all lattice work on the GPU; the
 * output is each pixel's segment line at every lambda, as the reference
 * traces it (these values are not the single-lambda solutions: for those,
 * call lf_tv_2d_batch with f_stride = 0).  As in the reference a negative
 * lambda counts as 0 and n_lambda = 0 returns at once. */
int lf_tv_2d_path(const char* kernel, size_t nx, size_t ny, const double* f, size_t n_lambda,
                  const double* lambdas, double* out);
/* The same, with statistics (stats: 10 int64, may be NULL): path segments,
 * region probes (device max-flows), events applied, initial level sets,
 * probes of regions too large for one block, and the microseconds spent in
 * those probes, in the one-block probes and in segment set-ups, and the
 * epochs and BFS levels run by the one-block probes. */
int lf_tv_2d_path_stats(const char* kernel, size_t nx, size_t ny, const double* f,
                        size_t n_lambda, const double* lambdas, double* out, int64_t* stats);

/* Many single-lambda TV problems of one shape solved together on the GPU:
 * problem p is the image at f + p * f_stride (f_stride = 0: one image for
 * all problems) at lambda lambdas[p]; out (and levels_out, may be NULL) hold
 * count * nx * ny values, problem-major.  Small problems are stacked into
 * one lattice of at most max_nodes nodes (0 = 2^18; stacked problems advance
 * in lockstep, so large ones are not stacked), and the stacks run as
 * independent solves on up to 8 host threads with their own CUDA streams.
 * No reference counterpart (the reference solves one image per call). */
int lf_tv_2d_batch(const char* kernel, size_t nx, size_t ny, size_t count, const double* f,
                   size_t f_stride, const double* lambdas, double* out, int64_t* levels_out,
                   size_t max_nodes);

#ifdef __cplusplus
}
#endif

#endif /* LATTICEFLOW_GPU_H */
