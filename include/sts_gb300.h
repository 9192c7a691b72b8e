/*
 * C ABI of the GB300 SIMPLE-TS time step (libsts_gb300.so).
 *
 * The reference solver (SIMPLE_TS_MPI.cpp) has no library interface: its seam
 * is the process and the files in its working directory.  EnteredData.txt and
 * the body files go in (SIMPLE_TS_MPI.cpp:5241-5561, Objects_for_Solving.h:306-412),
 * the field dumps u/v/p/Temper/vol_inf_fb come out (SIMPLE_TS_MPI.cpp:5564-5731),
 * and the time loop of main() (SIMPLE_TS_MPI.cpp:3230-4691) does the work.  The
 * entry points below replace that loop and keep the file formats.
 *
 * Conventions: plain pointers and sizes; fields are double[Nx*Ny] with
 * index i + j*Nx (x fastest), exactly the reference's layout.  Every call
 * returns STS_OK (0) or a negative STS_ERR_* code; sts_last_error() gives the
 * message of the last failure on the calling thread.  A context owns its
 * device buffers and one CUDA stream; one context must not be used from two
 * threads at once, different contexts are independent.  Host buffers are
 * owned by the caller and only copied.
 */
#ifndef STS_GB300_H
#define STS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define STS_OK 0
#define STS_ERR_ARG (-1)       /* bad argument or unknown field name */
#define STS_ERR_INPUT (-2)     /* missing or malformed case file */
#define STS_ERR_CUDA (-3)      /* CUDA runtime error (no device, launch failure, ...) */
#define STS_ERR_NONFINITE (-4) /* a residual went NaN/Inf during the steps just taken */
#define STS_ERR_TIMEOUT (-5)   /* a bounded device-side wait (the sweep loop's grid barrier) gave up;
                                  the context's state is no longer consistent and it stops stepping */

typedef struct sts_ctx sts_ctx;

typedef struct sts_options {
  /* 1: the sweep loop runs exactly N_I_p_c sweeps (the shipped build, FIXED_NUMBER_OF_ITERATIONS_LOOP_3
   *    defined, SIMPLE_TS_MPI.cpp:56 and :4099-4100);
   * 0: it stops on MaxError_p_c / MaxError_T after at least 2 sweeps (SIMPLE_TS_MPI.cpp:4101-4106). */
  int fixed_sweeps;
  /* 1: run the steps as one CUDA graph with conditional nodes (no host round trip per sweep);
   * 0: launch kernel by kernel from the host. */
  int use_graph;
  /* CUDA device ordinal. */
  int device;
  /* 1: sts_run_case writes dumps and logs into the case directory like the reference. */
  int write_files;
  /* 0: FP64, bit-exact with the reference (default).
   * 1: FP64 with reciprocal multiplies and fused multiply-adds in the assembly and the
   *    flux/diffusion kernels (a few ulps from the reference per step).
   * 2: as 1, and the p-T sweeps of the tolerance-terminated loop run in FP32 on correction
   *    fields over FP64 base fields; the sweep that meets the tolerance is recomputed in FP64,
   *    so the stopping residual is an FP64 update.  Fixed sweep counts run as mode 1.
   * 3: as 2, with the FP64 arithmetic of the assembly, the velocity correction, the
   *    flux/diffusion kernel and the FP64 sweeps done in double-float (pairs of FP32 numbers,
   *    about 47 significant bits) on the FP32 pipes; fields stay FP64 in memory. */
  int precision;
  /* Initial iterate of every step's p-T sweeps (no counterpart in the reference, which starts from
   * the previous step's p and T):
   * 0: the previous step's values (the reference);
   * 1: linear extrapolation in time, p_n + (p_n - p_{n-1}), on the solved cells;
   * 2: quadratic extrapolation, 3 (p_n - p_{n-1}) + p_{n-2} (linear on the second step);
   * 3: a linear predictor learned from the run itself: p_n + sum_k w_k (p_{n-k} - p_{n-k-1}),
   *    k = 0..2, with w refitted every step by least squares on the last 6 steps (separately
   *    for p and T; quadratic extrapolation until the history is long enough);
   * 4: a 3x3 convolutional predictor learned from the run itself: where the solution moves (cells
   *    within 3 cells of one whose last change exceeds 0.1 of the largest), the step's change is a
   *    linear function of 36 features of the cell's neighbourhood in the last four changes,
   *    refitted every step by least squares on the last 6 steps; elsewhere mode 2.  Tracks fronts
   *    that move across cells, which extrapolation in time cannot.
   * 5: warm_start 4, its start corrected on a window around the moving front (64 x 256 cells, or the
   *    mesh when smaller, centred on the largest change of p) by a U-Net (3 levels, 16 base
   *    channels, BF16 tensor-core kernels) that predicts the stencil's error from the last three
   *    changes and the stencil's prediction; the solver stores every step's window and the
   *    stencil's error there as a training pair (a ring of 256), sts_warm_net_train trains the
   *    network on them and sts_warm_net_enable switches the correction on.  Single cases only.
   * The sweeps still iterate to the same tolerance, so the result moves only within it; the
   * sweep count falls.  Meaningful for tolerance-terminated loops (fixed_sweeps = 0). */
  int warm_start;
  /* 1: sts_run_case's periodic dumps (WriteSolvedDataToFile, SIMPLE_TS_MPI.cpp:4625-4646) are
   *    written from a host thread while the next steps run (see sts_write_outputs_async);
   *    the run still returns only after every file is complete (default);
   * 0: each save is on disk before stepping resumes, as in the reference. */
  int async_save;
  /* 1: the first steps of the run choose the launch shapes -- the sweep loop's CTAs per SM and the
   *    assembly kernel's block shape -- by timing each candidate on real steps launched kernel by
   *    kernel (1 + 3 x max(CTAs per SM that fit, 3) steps); results do not depend on launch shapes,
   *    so the run is the same bit for bit; the graph is built with the chosen shapes (default);
   * 0: the largest number of CTAs that fit and 32x8 blocks. */
  int autotune;
} sts_options;

/* Fills *opt with the defaults (fixed_sweeps 1, use_graph 1, device 0, write_files 1, precision 0,
 * warm_start 0, async_save 1, autotune 1). */
void sts_default_options(sts_options* opt);

/* Reads a case directory (EnteredData.txt, solve_*_b.txt, restart dumps when
 * ToReadSolvedDataFromFile = 1) and prepares the device state up to the first
 * time step.  Replaces main() up to the time loop, SIMPLE_TS_MPI.cpp:1796-3227. */
int sts_open_case(const char* case_dir, const sts_options* opt, sts_ctx** out);

/* Advances up to nsteps time steps (SIMPLE_TS_MPI.cpp:3230-4691 per step).  Stops
 * early when the reference's continue rule ends the run (Nt reached or the
 * steady-state stop MaxError_to_stop_program, SIMPLE_TS_MPI.cpp:4442-4449);
 * *steps_done (optional) receives the count taken. */
int sts_step(sts_ctx* ctx, int nsteps, int* steps_done);

/* sts_step with a CUDA event pair on the context's stream around the work;
 * *device_ms receives the elapsed device time. */
int sts_step_timed(sts_ctx* ctx, int nsteps, int* steps_done, double* device_ms);

/* Runs up to nsteps steps kernel by kernel with an event pair around every launch and
 * returns per-kernel device time and launch counts, indexed 0 step_begin, 1 assemble,
 * 2 sweep loop (all p-T sweeps of an outer iteration, one launch), 3 correct, 4 face_rho,
 * 5 boundary, 6 flux_diff, 7 step_end (8 entries each).
 * The steps are real: the state advances exactly as with sts_step. */
int sts_profile_steps(sts_ctx* ctx, int nsteps, double* kernel_ms, int* kernel_launches, int* steps_done);

/* Copies a field to host memory.  Names: u v p T rho sqrt_T rho_u rho_v Fx Fy D_ux D_uy
 * D_vx D_vy DTx DTy Gamma_xf Gamma_yf ScT1 apx apy bpx bpy u_pseudo v_pseudo d_p_c_12
 * d_p_c_34 Tw_u Tw_v p_pr T_pr u_pr v_pr rho_pr (Nx*Ny doubles); hx x_v (Nx); hy y_v (Ny). */
int sts_get_field(sts_ctx* ctx, const char* name, double* host_out);

/* Overwrites u, v, p or T from host memory (Nx*Ny doubles); rho and sqrt_T follow on the next step.
 * With a warm start (sts_options.warm_start), setting p or T starts its history over. */
int sts_set_field(sts_ctx* ctx, const char* name, const double* host_in);

/* The state the reference dumps -- u, v, p, T (Nx*Ny doubles each) -- to or from host memory in
 * one call that returns once the data has moved (one synchronisation instead of four).  For
 * callers that exchange the whole state every step.  Host buffers the device can address
 * (pinned by cudaHostAlloc / cudaMallocHost, or registered with cudaHostRegister) are read or
 * written by one kernel that moves all four fields at once; other host memory goes through four
 * copies.  sts_set_state has sts_set_field's effect on each field (a warm start's history
 * starts over). */
int sts_set_state(sts_ctx* ctx, const double* u_in, const double* v_in, const double* p_in, const double* T_in);
int sts_get_state(sts_ctx* ctx, double* u_out, double* v_out, double* p_out, double* T_out);

/* sts_set_state, sts_step and sts_get_state in one call, for a host loop that hands the library
 * the state, advances it and takes it back every time (the three calls' results, bit for bit):
 * the input move, the steps and the output move are queued on the context's stream and the call
 * synchronises once, at the end, instead of three times.  The outputs take the direct kernel path
 * when they are device-addressable host memory and the steps run as the step graph; otherwise
 * (steps of the autotuner, use_graph 0, other host memory) the state is fetched after the steps as
 * sts_get_state does.  For one step with device-addressable inputs and outputs, the state is read
 * from the inputs inside the step's first kernel and written to the outputs while the step's last
 * kernels run.  Input and output buffers may be the same.  Returns sts_step's status; after
 * STS_OK or STS_ERR_NONFINITE the outputs hold the state at the end of the steps taken. */
int sts_step_exchange(sts_ctx* ctx, int nsteps, const double* u_in, const double* v_in, const double* p_in,
                      const double* T_in, double* u_out, double* v_out, double* p_out, double* T_out,
                      int* steps_done);

/* Global conservation sums of the current state over the fluid cells, in FP64 on the device in a
 * fixed order (each row in chunks of 64 cells in x order, the chunks of a row in order, the rows in
 * y order), so the same state always gives the same bits: out5[0] mass sum rho A, [1] and [2]
 * momentum sums rho A u_c and rho A v_c, [3] internal energy sum rho A T / (gamma - 1), [4] kinetic
 * energy sum rho A (u_c^2 + v_c^2); A = hx hy, u_c and v_c the means of a cell's two face
 * velocities (energies in units of rho0 R T0 per unit area, velocities being in units of
 * sqrt(2 R T0)).  No counterpart in the reference, whose SolveContinuityEquation
 * (SIMPLE_TS_MPI.cpp:10621-10714) gives the local continuity residual. */
int sts_conservation(sts_ctx* ctx, double* out5);

/* Mesh size. */
int sts_dims(sts_ctx* ctx, int* Nx, int* Ny);

/* Statistics of the last step: [Iter, Iter_p_c, res_p first sweep, res_p last sweep,
 * res_T first, res_T last, res_u, res_v, time] (the numbers of Tmp.txt, SIMPLE_TS_MPI.cpp:5887-5928). */
int sts_stats(sts_ctx* ctx, double* out9);

/* Jacobi sweeps taken by each of the last steps (oldest first, at most cap, at most 4096). */
int sts_sweep_history(sts_ctx* ctx, unsigned int* out, int cap, int* n_out);

/* Applies the output-time wall-temperature overwrite and writes u.bin v.bin p.bin
 * Temper.bin vol_inf_fb.bin it_begin.txt into the case directory (WriteSolvedDataToFile,
 * SIMPLE_TS_MPI.cpp:5564-5731). */
int sts_write_outputs(sts_ctx* ctx);

/* sts_write_outputs without waiting for the files: the wall-temperature overwrite and a
 * device-to-device snapshot of u, v, p, T are queued on the context's stream, a second stream
 * copies the snapshot to pinned host memory and a host thread writes the files, while the
 * caller goes on stepping.  The files hold the state of the call, not of later steps.  Two
 * snapshots can be pending; a third call waits for the older one.  Memory, made at the first
 * save: 64 bytes per cell on the device and 64 pinned on the host.  Saves are written in call
 * order.  The files are complete after sts_wait_outputs, sts_write_outputs or sts_destroy.
 * Asynchronous counterpart of WriteSolvedDataToFile (SIMPLE_TS_MPI.cpp:5564-5731). */
int sts_write_outputs_async(sts_ctx* ctx);

/* Waits until every save of the context is on disk; returns the first error among them. */
int sts_wait_outputs(sts_ctx* ctx);

/* The launch shapes in use: tuning steps still to come (sts_options.autotune), the sweep loop's
 * CTAs per SM and the assembly kernel's block (x, y).  No counterpart in the reference. */
int sts_autotune_result(sts_ctx* ctx, int* steps_left, int* ctas_per_sm, int* asm_block_x, int* asm_block_y);

/* Whole drop-in run of a case directory: open, step until the run ends, with the
 * periodic saves and logs of the reference (Tmp.txt, Iterations_in_loops.txt), and the
 * final dumps.  Equivalent to running the serial reference binary in case_dir. */
int sts_run_case(const char* case_dir, const sts_options* opt);

/* Synchronises the context's stream (the steps are asynchronous otherwise). */
int sts_sync(sts_ctx* ctx);

/* Releases the device buffers. */
void sts_destroy(sts_ctx* ctx);

/* Message of the last failure on this thread ("" if none). */
const char* sts_last_error(void);

/* Inputs of the coupled p-T Jacobi sweeps as device arrays owned by the caller (fields are
 * Nx*Ny doubles in the reference layout, hx: Nx, hy: Ny; cls uses the class-byte layout of
 * sts_inspect_case).  p and T hold the initial iterate and receive the final one. */
typedef struct sts_sweep_fields {
  int Nx, Ny;
  int periodic;               /* Periodic_boundary_conditions_about_OX */
  int given_u_xb, given_u_xe; /* Given_velocity_on_xb / _xe */
  int Nx_o0, Nx_o1;           /* p/T solve range in x (define_area_for_solving) */
  double ht, gamma1;
  const unsigned char* cls;
  const double *hx, *hy;
  const double *Fx, *Fy, *DTx, *DTy, *u, *v, *rho, *ScT1, *apx, *apy, *bpx, *bpy, *p_pr, *T_pr, *Tw_u, *Tw_v;
  double *p, *T;
} sts_sweep_fields;

/* The p-T sweep loop of one outer iteration (SIMPLE_TS_MPI.cpp:3786-4131) on caller-owned
 * device arrays, bit-exact with the reference: fixed_sweeps = 1 runs exactly max_sweeps
 * sweeps; 0 stops after at least 2 sweeps once max|dp| <= tol_p and max|dT| <= tol_T (or at
 * max_sweeps).  Work is queued on `stream` (a cudaStream_t, NULL for the legacy stream) and the
 * call returns when it is done.  Scratch (a second iterate, the sweep invariants and the
 * reduction words: 10*Nx*Ny doubles + 20 KB) is allocated stream-ordered and freed by the call. */
int sts_pt_sweeps(const sts_sweep_fields* f, int max_sweeps, int fixed_sweeps, double tol_p, double tol_T,
                  void* stream, int* sweeps_done, double* res_p, double* res_T);

/* Sweeps per tile load of the FP32 correction sweeps (precision 2 and 3, tolerance-terminated loops,
 * single cases): k = 2 runs two sweeps per round of the persistent loop -- each CTA loads its tile
 * of the corrections with a margin of two cells by TMA and sweeps it twice, halving the grid-wide
 * barriers -- and the loop still stops at the same sweep with the same iterate (the residuals of
 * both sweeps are kept and the stop rule is applied after each); k = 1 one sweep per round; k = 0
 * the autotuner's choice (it times both on the run's first steps).  The results are the same bits
 * either way.  The reference sweeps one sweep at a time (SIMPLE_TS_MPI.cpp:3788-4131). */
int sts_set_sweep_blocking(sts_ctx* ctx, int k);
/* The sweeps per tile load in use (1 or 2). */
int sts_get_sweep_blocking(sts_ctx* ctx, int* k);

/* warm_start 5: `iters` Adam steps (learning rate lr) of the network on batches of 8 training pairs
 * drawn from the pairs the solver has stored (the mean squared error of the predicted stencil error
 * on the window's flagged cells); *loss_out (optional) receives the last batch's loss.  Runs on the
 * context's stream between steps.  No counterpart in the reference. */
int sts_warm_net_train(sts_ctx* ctx, int iters, float lr, float* loss_out);
/* warm_start 5: the network's mean loss over every stored training pair, and the loss of a zero
 * correction (the stencil alone) on the same pairs. */
int sts_warm_net_eval(sts_ctx* ctx, float* loss_net, float* loss_zero);
/* warm_start 5: on = 1 applies the network's correction from the next step on (the training pairs
 * are stored either way); off by default. */
int sts_warm_net_enable(sts_ctx* ctx, int on);
/* warm_start 5: training pairs stored so far, the window's size and the network's parameter count. */
int sts_warm_net_info(sts_ctx* ctx, int* pairs, int* win_h, int* win_w, long long* nparams);
/* warm_start 5: steps whose window took the network's correction of p and of T so far.  The
 * correction of p is applied on a step's window only if, on the window completed at that step, it
 * had left a smaller largest error than the stencil's own start (the sweep count follows the
 * largest error of the start); the correction of T is not applied. */
int sts_warm_net_gate(sts_ctx* ctx, int* steps_on_p, int* steps_on_T);
/* warm_start 5: the network's FP32 parameters (layout of sts_net_get_params) out and/or in (NULL to skip). */
int sts_warm_net_params(sts_ctx* ctx, float* out, const float* in);

/* Largest mesh (Nx*Ny cells) that sts_pt_sweeps_noalloc accepts. */
#define STS_NOALLOC_MAX_CELLS 32768

/* sts_pt_sweeps for callers that must not allocate device memory: no cudaMalloc, cudaFree or
 * other allocating call is made.  This entry point has no counterpart in the reference (which
 * runs on the host only); it exists for programs whose device memory is owned by someone else
 * -- a framework's caching pool or an embedding application that has reserved the device
 * memory it is allowed to use -- and for time-critical loops that cannot afford the
 * device-wide synchronisation and latency an allocation or free can cause.
 * Inputs and outputs are the caller's device arrays, as for sts_pt_sweeps.  The scratch lives
 * in one fixed device array inside the library, sized for STS_NOALLOC_MAX_CELLS cells (about
 * 2.6 MB, held on every GPU that loads the library until the process exits); larger meshes are
 * rejected with STS_ERR_ARG.  Every call looks up that array's device address on the current
 * device (cudaGetSymbolAddress), so a device reset between calls leaves no stale address; the
 * first call on a device may also load the library's device code there, so make that first call
 * before any stream capture.  All calls share the one array and it keeps the last call's contents (each call
 * clears the counters it needs), so calls whose work overlaps on the GPU -- from several
 * threads or streams at once -- race and must be serialised by the caller. */
int sts_pt_sweeps_noalloc(const sts_sweep_fields* f, int max_sweeps, int fixed_sweeps, double tol_p, double tol_T,
                          void* stream, int* sweeps_done, double* res_p, double* res_T);

/* Self-check of the library's division through correctly rounded reciprocals (used by the FP64
 * kernels for divisors fixed by the mesh or by the outer iteration; Markstein's method) and of
 * its IEEE division with zero dividends answered directly, against IEEE division on `device`:
 * n pseudo-random operand pairs from `seed` (zero dividends and zero, infinite and NaN divisors
 * among them), *mismatches receives the number of results that differ in any bit (0 is the only
 * passing answer).  No counterpart in the reference, which divides with the host's IEEE
 * division. */
int sts_check_division(unsigned long long n, unsigned long long seed, int device, unsigned long long* mismatches);

/* Self-check of the BF16 tensor-core GEMM of the learned warm start's network (tcgen05 MMAs fed by
 * TMA, FP32 accumulation in tensor memory) on `device`: D[M x N] = A[M x K] * B[N x K]^T (+ bias[n],
 * then max(., 0) if relu), A and B row-major BF16 bit patterns on the host (K a multiple of 8),
 * D row-major FP32 on the host; bias may be NULL.  STS_ERR_TIMEOUT if a pipeline wait gave up.
 * No counterpart in the reference. */
int sts_tc_gemm(const unsigned short* A, const unsigned short* B, int M, int N, int K, int relu, const float* bias,
                float* D, int device);

/* The convolutional network of the learned warm start, on host arrays: a U-Net (levels L, base
 * channels C0, C_l = C0 2^l; two 3x3 convolutions with ReLU per level, 2x2 average pooling down,
 * nearest-neighbour upsampling and concatenation with the encoder output up, a 1x1 head) with BF16
 * weights and activations and FP32 accumulation; every convolution is a tcgen05 tensor-core GEMM
 * (sts_tc_gemm).  Images are batches of B crops of H x W pixels, NHWC (channels contiguous), FP32
 * on the host.  in_ch, out_ch <= 8; C0 a multiple of 8; H, W multiples of 2^(L-1).  Parameters
 * (FP32 master copy) in layer order: per convolution Wt[(3 (dy+1) + (dx+1)) C_in + c][C_out] then
 * the bias [C_out]; the head's Wt [C0][8] then its bias [8] (outputs beyond out_ch held at 0).
 * No counterpart in the reference, which starts every step's sweeps from the previous step. */
typedef struct sts_net sts_net;
int sts_net_create(int in_ch, int out_ch, int base_ch, int levels, int max_batch, int H, int W, unsigned long long seed,
                   int device, sts_net** out);
long long sts_net_param_count(sts_net* net);
int sts_net_get_params(sts_net* net, float* out);
int sts_net_set_params(sts_net* net, const float* in);
/* y [B][H][W][out_ch] = net(x [B][H][W][in_ch]). */
int sts_net_forward(sts_net* net, const float* x, int B, float* y);
/* After sts_net_forward with the same B: the parameter gradients of sum(gy * y) into grads. */
int sts_net_backward(sts_net* net, const float* gy, int B, float* grads);
/* One Adam step (learning rate lr) on the mean squared error against target [B][H][W][out_ch];
 * *loss receives the loss before the step. */
int sts_net_train_step(sts_net* net, const float* x, const float* target, int B, float lr, float* loss);
void sts_net_destroy(sts_net* net);

/* Self-check of the bounded wait of the sweep loop's grid barrier on `device`: one cooperative
 * launch of one CTA per multiprocessor meets `rounds` grid barriers, each wait limited to
 * spin_limit polls (about 0.1-1 us each).  CTA skip_cta (none when negative) leaves without
 * arriving, so the others' first wait runs out; they record the timeout and end, the device stays
 * usable.  Returns STS_OK when every barrier completed, STS_ERR_TIMEOUT when a wait gave up.  The
 * same bounded wait guards every grid barrier of the sweep loops (about a second there), which
 * then end the step with STS_ERR_TIMEOUT instead of hanging.  No counterpart in the reference. */
int sts_check_barrier_timeout(int device, int skip_cta, unsigned spin_limit, int rounds);

/* FP64 throughput of `device`, measured: gops[0..2] receive the rates (10^9 operations per
 * second) of dependent-free FP64 adds, multiplies and fused multiply-adds in a loop that keeps
 * the FP64 unit busy (about 2 ms in all).  The roofline of the bit-exact kernels, which are
 * bound by the FP64 unit rather than by memory, is taken against these rates.  No counterpart
 * in the reference. */
int sts_fp64_rates(int device, double* gops);

/* Self-check of the double-float arithmetic of precision mode 3 against FP64 on `device`: n
 * pseudo-random operand pairs from `seed` (random signs, magnitudes 2^-40 .. 2^40); max_rel_err[0..4]
 * receive the largest relative errors of the FP64 -> double-float conversion, add (relative to
 * |a| + |b|), multiply, divide and square root.  No counterpart in the reference. */
int sts_check_double_float(unsigned long long n, unsigned long long seed, int device, double* max_rel_err);

/* Batches: many independent cases advanced together on one GPU.  Every kernel of a step is
 * launched once for all cases and the p-T sweep loops of all cases run in one cooperative
 * launch, each case with its own stop rule; the step loop is one CUDA graph.  The reference
 * runs one case per process (or per MPI job); a batch is the GB300 form of running many such
 * jobs side by side, with the same results as running each case alone.  Restrictions: at most
 * 256 cases, N_I = 1 in every case, one sweep mode (opt->fixed_sweeps) and one precision for
 * the whole batch.  opt->use_graph = 0 launches the kernels step by step from the host (same
 * results; for per-kernel profiling); opt->write_files is ignored. */
typedef struct sts_batch sts_batch;
int sts_open_batch(const char* const* case_dirs, int ncases, const sts_options* opt, sts_batch** out);

/* Advances every case by up to nsteps time steps; a case whose run ended (Nt, steady-state stop)
 * stays where it stopped.  *steps_done receives the most steps any case took. */
int sts_batch_step(sts_batch* b, int nsteps, int* steps_done);

/* sts_batch_step with a CUDA event pair around the work; *device_ms receives the device time. */
int sts_batch_step_timed(sts_batch* b, int nsteps, int* steps_done, double* device_ms);

/* The context of case `index` (borrowed: valid until sts_batch_destroy).  sts_get_field,
 * sts_set_field, sts_dims, sts_stats, sts_sweep_history and sts_write_outputs work on it;
 * sts_step and sts_profile_steps return STS_ERR_ARG, and sts_destroy leaves it to the batch. */
int sts_batch_case(sts_batch* b, int index, sts_ctx** out);

/* Releases the batch and its cases. */
void sts_batch_destroy(sts_batch* b);

/* sts_autotune_result for a batch: its tuning steps still to come, its sweep loop's CTAs per SM
 * and its assembly block (x, y).  No counterpart in the reference. */
int sts_batch_autotune_result(sts_batch* b, int* steps_left, int* ctas_per_sm, int* asm_block_x, int* asm_block_y);

/* Host-only inspection of a case directory (no device use): dims, obstacle ids
 * (vol_inf_fb, Nx*Ny), per-cell classes (Nx*Ny bytes: bits 0-1 u, 2-3 v, 4-5 p/T with
 * 0 unsolved, 1 interior, 2 boundary; bit 6 fluid) and the mesh (hx, x_v: Nx; hy, y_v: Ny).
 * Pass NULL for outputs not wanted; call once with all NULL to learn the dims. */
int sts_inspect_case(const char* case_dir, int* Nx, int* Ny, unsigned int* vol_out, unsigned char* cls_out,
                     double* hx_out, double* hy_out, double* xv_out, double* yv_out);

#ifdef __cplusplus
}
#endif

#endif /* STS_GB300_H */
