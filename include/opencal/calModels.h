/*
 * calModels.h -- entry points of libopencal_models.so: the reference's
 * example programs built on the C API (cal2D.h / cal3D.h) as callable
 * drivers, plus the calibration machinery of SCIDDICA-T.
 *
 * The reference ships these programs as executables with a main()
 * (OpenCAL-OMP/examples/calomp_sciddicaT/source/sciddicaT.c,
 * OpenCAL-OMP/examples/calomp_life/source/life.c, ...); none of the functions
 * below has a counterpart in the reference's library.  They exist so that
 * tests, the benchmark and calibration code can run those programs on given
 * inputs and read the results back.  Arrays are host memory unless a comment
 * says device; every function returns 0 (CAL_SUCCESS) or an error code
 * unless it returns a handle (NULL on failure).
 */
#ifndef calModels_h
#define calModels_h

#ifdef __cplusplus
extern "C" {
#endif

/* ---- SCIDDICA-T (OpenCAL-OMP/examples/calomp_sciddicaT/source/sciddicaT.c) ---- */

/* mode: 0 = the reference program (device elementary processes registered
 * with calAddElementaryProcess2D, steering, calRun2D); 1 = the same program
 * with the split step as its global transition (with ac: the active-cells
 * split step, which keeps its own active set and returns it in row-major
 * order, the reference's order).  graph: 0 =
 * launch sequence per step, 1 = recorded step replayed, 2 = device-driven
 * loop bounded by the final step, 3 = device loop ended by a device stop
 * condition, 4 = every step in one cooperative launch (mode 1 only).  n_active / cells_out: the active cells after the run (ac). */
int cal_sciddicaT_run(int rows, int cols, int toroidal, int ac, int steps, double p_r, double p_eps, const double* z0,
                      const double* h0, double* z_out, double* h_out, long* n_active, int* cells_out, int mode,
                      int graph, double* ms);
/* the reference example's main() as written: z and h loaded from text files
 * (calLoadSubstate2Dr), the run (calRun2D; graph 1 replays the recorded
 * step), h saved with calSaveSubstate2Dr to output_path */
int cal_sciddicaT_run_files(int rows, int cols, int toroidal, int steps, double p_r, double p_eps,
                            const char* dem_path, const char* source_path, const char* output_path, int graph);
/* how many device-loop runs fell back to a launch sequence per step */
int cal_sciddicaT_device_loop_fallbacks(void);

/* A session: the program created once, reset to its initial state and rerun.
 * The program's substates are globals, as in the reference's example: one
 * session is open at a time. */
void* cal_sciddicaT_open(int rows, int cols, int toroidal, int ac, double p_r, double p_eps, const double* z0,
                         const double* h0, int mode);
int cal_sciddicaT_reset(void* session);
/* graph: as for cal_sciddicaT_run, plus 4 = every step in one cooperative
 * launch of the persistent split-step kernel (mode 1, plain) */
int cal_sciddicaT_steps(void* session, int steps, int graph);
/* 1 when a grid barrier of the last persistent run gave up (synchronises) */
int cal_sciddicaT_persist_failed(void* session);
int cal_sciddicaT_set_params(void* session, double p_r, double p_eps);
/* 1: models created afterwards (cal_sciddicaT_run, cal_sciddicaT_open,
 * processes mode) declare the two plain processes pure
 * (calSetElementaryProcessPure2D), so that the engine skips quiet tiles;
 * 0 (default): the reference program as it stands */
int cal_sciddicaT_set_pure(int on);
/* 1: models created afterwards (processes mode) declare what the two plain
 * processes read (calSetElementaryProcessReads2D: z and h; h and the four
 * outflows), so that their kernels stage those substates by TMA; 0
 * (default): global reads */
int cal_sciddicaT_set_staged(int on);
/* 1: models created afterwards (processes mode) declare the flows
 * process's early return on cells with h <= epsilon
 * (calSetElementaryProcessGuard2Dr), so that its kernel runs it on each
 * tile's wet cells packed into consecutive threads; 0 (default): off */
int cal_sciddicaT_set_guard(int on);
/* launch grids of the split step's kernels: k1_blocks and k2_blocks
 * 256-thread blocks of the outflow and the update kernel (0 = the defaults
 * 608 / 608) */
int cal_sciddicaT_set_split_grid(void* session, int k1_blocks, int k2_blocks);
void* cal_sciddicaT_stream(void* session); /* cudaStream_t of the model */
/* the dense step's TMA-staged form (flat grids, rows a multiple of 16 bytes;
 * OPENCAL_SDT_TMA=0 keeps plain loads): launches queued so far and tiles
 * whose copies timed out (synchronises the device) */
int cal_sciddicaT_tma_stats(long long* launches, int* timeouts);
int cal_sciddicaT_host_run(void* session, const double* z_host, const double* h_host, int steps, int graph,
                           double* h_out);
int cal_sciddicaT_kernel_times(void* session, int n, float* ms_outflows, float* ms_update);
int cal_sciddicaT_wet_count(void* session);
/* `steps` plain split steps from the current state with a trace after each
 * (flat grids of at least 5 x 5 cells): outflux[t] = mass that left the grid
 * in step t + 1 (border cells' outflows towards absent neighbours), wet[t] =
 * wet cells processed in it, *edge_step = first step after which a cell of
 * the two-cell edge band holds h != 0, or -1.  Host arrays. */
int cal_sciddicaT_trace(void* session, int steps, double* outflux, int* wet, int* edge_step);
int cal_sciddicaT_read(void* session, double* h_out);
void cal_sciddicaT_close(void* session);

/* ---- SCIDDICA-T adjoint (one grid; device arrays) ---- */
void* cal_sdt_adj_create(int rows, int cols, int steps, int toroidal);
void cal_sdt_adj_destroy(void* work);
int cal_sdt_adj_forward(void* work, const double* z_dem, const double* h0, double p_r, double p_eps, double* hT,
                        void* stream);
int cal_sdt_adj_backward(void* work, const double* dL_dhT, double* dL_dh0, double* dL_dpr, double* dL_dpeps,
                         void* stream);

/* ---- SCIDDICA-T ensembles (many grids, one launch per step) ----
 * dims: 2B ints (rows, cols); params: 2B doubles (p_r, p_eps); z_dem, h0:
 * the instances' values back to back (unpadded, row-major).  Device arrays
 * of the ensemble use the padded layout given by cal_sdt_batch_cells. */
void* cal_sdt_batch_create(int B, const int* dims, const double* params, const double* z_dem, const double* h0,
                           int steps);
void cal_sdt_batch_destroy(void* ensemble);
long long cal_sdt_batch_cells(void* ensemble, long long* offsets /* B + 1, or NULL */);
void* cal_sdt_batch_stream(void* ensemble);
int cal_sdt_batch_shape(void* ensemble);
int cal_sdt_batch_set_shape(void* ensemble, int shape /* 0: 32x16, 1: 64x16, 2: 64x32 */);
int cal_sdt_batch_autotune(void* ensemble, int probe_steps, float* ms /* 5: 32x16, 64x16, 64x32, 16x8, 32x8 */);
int cal_sdt_batch_set_params(void* ensemble, const double* params);
int cal_sdt_batch_forward(void* ensemble, double* hT /* device, or NULL */);
int cal_sdt_batch_active_tiles(void* ensemble, int* counts /* steps + 1 */);
int cal_sdt_batch_loss_grad(void* ensemble, const double* target /* device */, double* loss /* B */,
                            double* grad /* 2B */, double* dL_dh0 /* device, or NULL */);
/* 1 (default): cal_sdt_batch_loss_grad is one launch of a recorded CUDA graph
 * (forward, loss, tape layout computed on the device, reverse sweep, results
 * to pinned host memory); 0: launch by launch.  Segmented tapes of more than
 * 32 steps a segment (rollouts over 1024 steps) are laid out on the host and
 * run launch by launch. */
int cal_sdt_batch_set_graph(void* ensemble, int on);
int cal_sdt_batch_graph_stats(void* ensemble, long long* launches, long long* nodes);
/* What the adjoint's tape holds: -1 (default) the whole rollout (the
 * backward recomputes nothing) while that tape fits in half of the free
 * device memory, else sqrt(T) segments recomputed from checkpoints; 0 always
 * segments; 1 always the whole rollout. */
int cal_sdt_batch_set_tape(void* ensemble, int mode);
/* info[0] = 1 when the last evaluation taped the whole rollout, info[1] =
 * tape capacity (bytes), info[2] = tape bytes the last evaluation needed */
int cal_sdt_batch_tape_info(void* ensemble, long long* info /* 3 */);

/* ---- SCIARA-fv2 (OpenCAL-OMP/examples/calomp_sciara-fv2/source/Sciara.cpp) ----
 * params: Pclock, PTsol, PTvent, Pr(Tsol), Pr(Tvent), Phc(Tsol), Phc(Tvent),
 * Pcool, Prho, Pepsilon, Psigma, Pcv (the .cfg order), Pc (cell size).
 * vent_xy: (x = column, y = row) pairs in the reference's vent order; rates:
 * nvents x nphases m^3/s; max_steps 0 runs until the emission ends. */
int cal_sciara_run(int rows, int cols, int ac, int max_steps, const double* params, int nvents, const int* vent_xy,
                   unsigned emission_time, int nphases, const double* rates, const double* z0, const double* slt0,
                   const double* st0, double* z_out, double* slt_out, double* st_out, double* msl_out,
                   int* steps_done, long* n_active, int* cells_out, int graph, double* ms);

/* form of the transcendental parts for the following cal_sciara_run calls:
 * 0 (default) identities suited to the FP64 pipe (exp10, the shear test
 * without atan / cos, T*T*T, cbrt); 1 pow, atan and cos written as the
 * reference writes them (Sciara.cpp:18-21, 61, 85, 147-150) */
int cal_sciara_set_math(int form);

/* The reference example's input files (OpenCAL-OMP/examples/calomp_sciara-fv2/
 * source/io.cpp:357-404): `path` names the .cfg (or the prefix to which
 * "_000000000000.cfg" is appended); Morphology.stt, Vents.stt and
 * EmissionRate.txt beside it are required, Thickness / Temperature /
 * SolidifiedLavaThickness.stt optional.  cal_sciara_read_sizes gives the
 * sizes to allocate; cal_sciara_read fills params (the 12 .cfg parameters
 * and Pc, cal_sciara_run's order), z, vent_xy (x, y per vent in the
 * reference's order), rates (nvents x nphases, shorter lists padded with 0)
 * and the emission time, and the optional grids where present[k] is set.
 * Returns CAL_ERROR_IO when a file is missing or malformed. */
int cal_sciara_read_sizes(const char* path, int* rows, int* cols, int* nvents, int* nphases);
int cal_sciara_read(const char* path, double* params, double* z, int* vent_xy, double* rates,
                    unsigned* emission_time, double* slt, double* st, double* msl, int* present);

/* SCIARA-fv2 scenarios by the split step (vents, flows of the lava cells,
 * update of the flagged tiles); one scenario or many in the same launches.
 * dims: 2B ints; z0 / slt0 / st0: the scenarios' grids back to back (slt0,
 * st0 may be NULL); vents: scenario index and (x, y) per vent, in each
 * scenario's vent order; rates: nvents x nphases.  list_fraction: capacity
 * of the lava list as a fraction of all cells. */
void* cal_sciara_batch_create(int B, const int* dims, const double* z0, const double* slt0, const double* st0,
                              const double* params, int nvents, const int* vent_inst, const int* vent_xy,
                              unsigned emission_time, int nphases, const double* rates, double list_fraction);
void cal_sciara_batch_destroy(void* batch);
int cal_sciara_batch_run(void* batch, int max_steps, int* steps_done, float* ms);
int cal_sciara_batch_read(void* batch, double* z, double* slt, double* st, double* msl);
/* L_b = sum (Slt_T - target)^2 per scenario and dL/drate of every vent and
 * phase (caller's vent order), by the adjoint with the forward's decisions
 * (elimination sets, shear test, solidification, border) frozen; undo tape
 * of tape_slots tiles (0: default) */
int cal_sciara_batch_loss_grad(void* batch, const double* target, int max_steps, double* loss, double* grad,
                               int* steps_done, long long tape_slots, float* ms);
int cal_sciara_batch_lava_cells(void* batch);

/* ---- mbusu, 3D subsurface flow (OpenCAL/examples/cal_mbusu-glut/source/mbusu.c) ----
 * steps: 0 = until the stop condition (10 days), > 0 = at most that many, < 0 =
 * none; mode: 0 = launch sequence per step, 1 = recorded step replayed, 2 =
 * device-driven loop ended by the device stop condition.  state: 8 x 624000
 * doubles (teta, moist_cont, psi, k, h, dqdh, convergence, moist_diff, each
 * slice-major 130 x 160 x 30) or NULL; tail: step reached, delta_t, delta_t_cum. */
int cal_mbusu_run(int steps, int mode, double* state, double* tail, double* ms);

/* ---- Game of Life (OpenCAL-OMP/examples/calomp_life) and the 3D rule ---- */
int cal_life2d_run(int rows, int cols, int toroidal, int as_int, int steps, const unsigned char* s0,
                   unsigned char* s_out, int mode, int block, int graph, double* ms);
/* declarations for the reference program's process in runs started
 * afterwards: bit 0 pure, bit 1 reads its state substate (staged by TMA);
 * 0: the program as it stands */
int cal_life2d_set_declarations(int flags);
int cal_life3d_run(int rows, int cols, int slices, int nbhd, int toroidal, int steps, int r1, int r2, int r3, int r4,
                   const unsigned char* s0, unsigned char* s_out, int graph);

/* SCIDDICA-T in the reference's unsafe form
 * (OpenCAL/examples/cal_sciddicaT-unsafe/source/sciddicaT.c) */
int cal_sciddicaT_unsafe_run(int rows, int cols, int toroidal, int steps, double p_r, double p_eps, const double* z0,
                             const double* h0, double* z_out, double* h_out, int graph);

/* ---- measurement aid ----
 * FP64 instructions per second of op 0 (DFMA), 1 (DADD) or 2 (DMUL) on the
 * current GPU (independent dependency chains on every SM, CUDA events);
 * *ms: duration of the timed launch */
int cal_fp64_peak(int op, double* instr_per_s, float* ms);

#ifdef __cplusplus
}
#endif

#endif
