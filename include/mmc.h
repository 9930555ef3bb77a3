/*
 * mmc.h -- C ABI of the GB300 micromagnetic Monte Carlo annealer.
 *
 * The reference program (chg-hou/Micromagnetic-GPU-Monte-Carlo) is a single
 * CUDA executable whose only public surface is its command line, its ini file
 * and its output files; its GPU work is done by file-scope kernels.  Each entry
 * point below replaces one of those pieces and cites the reference interface
 * it stands in for (paths are relative to the reference project).
 *
 * Conventions
 *  - Every function that can fail returns an int status (MMC_OK == 0) and never
 *    calls exit(); mmc_last_error() gives a message for the calling thread.
 *  - Host arrays are caller-owned and copied; device memory is owned by the
 *    handle.  One handle per host thread; the library starts no threads.
 *  - Lattice arrays on the host are indexed x fastest, then y, then z:
 *    i = x + nx*(y + ny*z) (the OVF data order).  The reference's own host
 *    arrays were z fastest (src/mx_init.h:98-153); callers holding that order
 *    transpose before calling.
 *  - Fields are in A/m, energies in J, temperatures in K, lengths in m.
 */
#ifndef MMC_H_
#define MMC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MMC_ABI_VERSION 2

enum mmc_status {
  MMC_OK = 0,
  MMC_ERR_INVALID = 1,      /* bad argument or config value */
  MMC_ERR_CONFIG = 2,       /* ini syntax error or missing key */
  MMC_ERR_IO = 3,           /* file could not be opened / read / written, malformed OVF */
  MMC_ERR_CUDA = 4,         /* CUDA runtime error */
  MMC_ERR_NO_DEVICE = 5,    /* no usable CUDA device */
  MMC_ERR_UNSUPPORTED = 6,  /* e.g. an FFT length with a prime factor above 31 */
  MMC_ERR_INTERRUPTED = 7,  /* mmc_request_stop() was called */
  MMC_ERR_TIMEOUT = 8,      /* a device-side wait ran out of its iteration budget */
  MMC_ERR_STATE = 9,        /* call made in the wrong order (e.g. demag not built) */
  MMC_ERR_OOM = 10          /* device allocation failed */
};

/* Field / energy terms for mmc_get_field(). */
enum mmc_term {
  MMC_TERM_EXCHANGE = 0,
  MMC_TERM_DMI = 1,
  MMC_TERM_ANISOTROPY = 2,
  MMC_TERM_ZEEMAN = 3,
  MMC_TERM_DEMAG = 4,
  MMC_TERM_TOTAL = 5
};

enum mmc_ovf_format { MMC_OVF_BINARY4 = 0, MMC_OVF_BINARY8 = 1, MMC_OVF_TEXT = 2 };

/* How sweeps are executed.  AUTO picks FUSED for films (nz = 1, demag on, two
 * sublattice colours) and KERNELS otherwise.  Both give bit-identical results. */
enum mmc_engine {
  MMC_ENGINE_AUTO = 0,
  MMC_ENGINE_KERNELS = 1,  /* one kernel per transform pass and colour, replayed from CUDA graphs */
  MMC_ENGINE_FUSED = 2     /* one persistent cooperative kernel per chunk of sweeps */
};

/*
 * Simulation parameters.  The first block holds exactly the 26 ini keys of the
 * reference (src/parse_input_ini.h:15-41, example README.md:44-86) with the
 * same names and meaning; bools are ints (0/1).  The second block holds
 * optional keys added by this library; their defaults reproduce the reference
 * behaviour.
 */
typedef struct mmc_config {
  int nx, ny, nz;
  double dx, dy, dz;
  double Bextx, Bexty, Bextz;              /* applied field, T */
  int pbc_x, pbc_y, pbc_z;                 /* 0: open (zero-padded), >0: periodic with that many images, <0: periodic, no images */
  double ms, Aex, Dind;                    /* A/m, J/m, J/m^2 */
  double anisUx, anisUy, anisUz, Ku1;      /* axis (normalised internally), J/m^3 */
  int use_random_init;
  long long randomseed;                    /* < 0: time(NULL) (src/main.cu:246-250) */
  char ovf_filename[1024];
  double Temperature_start, Temperature_end, Temperature_step;
  long long circle_per_stage;              /* sweeps per temperature stage */
  long long terminal_output_period;
  long long energy_output_period;
  long long ms_output_period;
  int rand_block_size;                     /* accepted and ignored: it sized the reference's pre-generated
                                              random pools (src/main.cu:351-385), which counter-based
                                              Philox proposals do not need */
  int cal_demag_flag;
  int Temperature_use_exp;                 /* 1: T *= step, 0: T -= step */

  /* ---- optional keys (not in the reference) ---- */
  int precision;                           /* 32 (default, the reference's FLOAT_=float) or 64 */
  int ovf_format;                          /* enum mmc_ovf_format, default MMC_OVF_BINARY4 */
  int use_reference_pi;                    /* 1: pi = 3.14159265358 as src/constant.h:21 */
  char tensor_cache[1024];                 /* directory for the demag tensor cache ("" = off) */
  int sweep_engine;                        /* enum mmc_engine, default MMC_ENGINE_AUTO */
  int fused_band;                          /* rows per CTA of the fused film engine, 0 = auto */
  int tensor_far_radius;                   /* 0 (default): every tensor term by the exact 64-term
                                              sum, as the reference; R >= 12: image offsets at least
                                              R cells away by the far-field expansion (more accurate
                                              there, and far cheaper; see mmc_build_demag) */
  int debug_h_field;                       /* 1: the stage loop writes the per-term field dumps at
                                              every energy output, as the reference's DEBUG_H_FIELD
                                              build does (see mmc_run_anneal); default 0 */
  int tensor_sum;                          /* how each image's 64-term Newell sum is formed (see
                                              mmc_build_demag): 0 term by term in the reference's
                                              order; 1 (default) as the 27-point stencil of f / g
                                              evaluated once per lattice node, ~20x cheaper, the same
                                              sum to FP64 rounding */
} mmc_config;

typedef struct mmc_observables {
  double e_total;                          /* J, sum of the five terms */
  double e_exchange, e_dmi, e_anisotropy, e_zeeman, e_demag;
  double m[3];                             /* average reduced magnetisation */
  double q;                                /* topological charge per layer (Berg-Luescher) */
  unsigned long long accepted, proposed;   /* Metropolis counts since the last mmc_energy() */
} mmc_observables;

typedef struct mmc_handle mmc_handle;

int mmc_abi_version(void);
/* sizeof(mmc_config) as compiled into the library (binding sanity check). */
size_t mmc_config_size(void);
const char* mmc_status_string(int status);
/* Message of the last failing call on this thread ("" if none). */
const char* mmc_last_error(void);

/* Fill every field with the reference's README example values and the optional defaults. */
void mmc_config_defaults(mmc_config* cfg);

/* Replaces parse_input_ini (src/parse_input_ini.h:15-47).  All 26 reference
 * keys are required; unknown keys are an error; the optional keys above may be
 * given as well. */
int mmc_config_load_ini(const char* path, mmc_config* cfg);

/* Replaces cout_input_ini (src/parse_input_ini.h:49-114): writes the
 * "key: value" echo into buf (NUL-terminated, truncated to len). */
int mmc_config_format(const mmc_config* cfg, char* buf, size_t len);

/* Padded dimensions of the tensor grid (src/main.cu:254-263): n -> 2n-1 on
 * open axes, n on periodic ones -- the grid of mmc_get_tensor and of the
 * tensor cache.  The transforms may pad an open axis further: see
 * mmc_transform_dims. */
int mmc_padded_dims(const mmc_config* cfg, int out[3]);
/* Dimensions of the grid the demag transforms run on (no device needed).
 * No counterpart in the reference, which transforms on the tensor grid.  An
 * open axis whose tensor length t = 2n-1 exceeds 16 is padded to the next
 * power of two when that is at most 256; when it would be 512 or 1024, t is
 * kept if its prime factors are all at most 31 (the mixed-radix transforms),
 * else padded.  Periodic axes and t <= 16 are kept.  The tensor is re-wrapped
 * onto this grid (offsets |o| <= n-1 kept, the rest 0), which gives the same
 * linear convolution. */
int mmc_transform_dims(const mmc_config* cfg, int out[3]);

/* Allocates the device state for one lattice on CUDA device `device`
 * (the -gpu= flag, src/GPU_selector.h:35-76).  m starts at +z. */
int mmc_create(const mmc_config* cfg, int device, mmc_handle** out);
void mmc_destroy(mmc_handle* h);

/* The CUDA stream the handle enqueues its work on.  A handle creates a
 * non-blocking stream of its own; mmc_set_stream moves its work to `stream`
 * (a cudaStream_t the caller created on the handle's device -- e.g. a
 * framework's current stream -- and keeps alive while the handle uses it), and
 * NULL moves it back.  The new stream first waits for the work already
 * enqueued on the old one, so calls stay in order.  The legacy and per-thread
 * default streams are refused (MMC_ERR_INVALID): the sweep graphs are captured
 * on the handle's stream.  Calls that return results still synchronize that
 * stream.  The reference ran everything on the default stream
 * (src/main.cu:868-884, 1101-1120). */
int mmc_set_stream(mmc_handle* h, void* stream);

/* Replaces randInitMx (src/mx_init.h:21-97): every cell gets an independent
 * direction uniform on the sphere, from Philox4x32-10 keyed on the seed. */
int mmc_init_random(mmc_handle* h, long long seed);

/* Host <-> device copies of m (replace copyMxtoMxpadded / copyMxpaddedtoMx,
 * src/mx_init.h:98-153).  Arrays hold nx*ny*nz values, x fastest. */
int mmc_set_m(mmc_handle* h, const double* mx, const double* my, const double* mz);
int mmc_get_m(mmc_handle* h, double* mx, double* my, double* mz);

/* Newell demag tensor with periodic images (ktensorCPU / ktensorKernel2_*,
 * src/demag_cu.cu:119-248, src/main.cu:419-573) and its FFT (src/main.cu:589-675).
 * With a non-empty cache_dir (the -tensorcache= flag) the tensor is read from /
 * written to cache_<nxp>_<nyp>_<nzp>-<dx>_<dy>_<dz>-<pbcx>_<pbcy>_<pbcz>.ovf
 * in the reference's raw layout.  Called implicitly by the first call that
 * needs it when cal_demag_flag is set.
 * With tensor_far_radius = R > 0, every image offset whose cell-centre
 * distance is at least R times the largest cell side is summed with the
 * far-field expansion of the 64-term sum (derivatives of 1/r up to order 8,
 * truncation error O((d/r)^8): 4e-13 of the term at 32 cells against
 * 60-digit evaluations), where the exact FP64 sum loses (r/d)^6 x 1e-16 to
 * cancellation (1e-6 at 32 cells, 0.2 at 300 cells).  Such a tensor is cached
 * under the reference's name with a "_far<R>" suffix.
 * tensor_sum = 1 (default) forms each image's 64-term sum as the 27-point
 * stencil sum_s w(sx) w(sy) w(sz) F(offset + s), s in {-1,0,1}^3, w(0) = 2,
 * w(+-1) = -1 -- the same sum regrouped, with each of the six potentials
 * evaluated once per lattice node and tile instead of 64 times per offset
 * (the 256^2 film with 20 images: seconds instead of ~37 s).  Its rounding
 * differs from the term-by-term form (tensor_sum = 0, the reference's order)
 * by as much as either differs from the exact tensor; both are cached under
 * the same name. */
int mmc_build_demag(mmc_handle* h, const char* cache_dir);

/* The real-space tensor: 6 blocks (xx,xy,xz,yy,yz,zz) of nxp*nyp*nzp doubles,
 * x fastest within a block (built first if needed). */
int mmc_get_tensor(mmc_handle* h, double* k6);

/* Replaces calDemagMirrorTensor (src/demag_mirror.h:18-24): the tensor at zero
 * offset including periodic images, order xx,xy,xz,yy,yz,zz. */
int mmc_self_tensor(mmc_handle* h, double k6[6]);

/* One demag convolution of the current m (src/main.cu:868-884 plus the
 * inverse transform and crop that the reference never executed). */
int mmc_compute_demag(mmc_handle* h);

/* Device-pointer form of the demag convolution, the kernel-level contract of
 * calHexchangeKernel + the cuFFT calls around it (src/demag_cu.h:36-39,
 * src/main.cu:868-884): hdev = K * mdev for this handle's lattice, using the
 * handle's tensor spectrum.  mdev and hdev hold 3*nx*ny*nz values of the
 * handle's precision (float for precision 32, double for 64), SoA, x fastest;
 * hdev is dimensionless (H_demag = ms * hdev).  scratch is a caller-owned
 * device buffer of at least mmc_demag_scratch_bytes() bytes.  The work is
 * enqueued on `stream` (a cudaStream_t; NULL means the handle's stream) and
 * the call returns without synchronising. */
int mmc_demag_scratch_bytes(mmc_handle* h, size_t* bytes);
int mmc_demag_apply(mmc_handle* h, const void* mdev, void* hdev, void* scratch, size_t scratch_bytes,
                    void* stream);
/* Size of the device array behind mmc_demag_apply_static(): 16 MiB, enough
 * for the spectrum of any lattice with 3 * nspec * 2 * sizeof(real) at most
 * this size (a 1024 x 1024 periodic film in FP32, a 512 x 512 open film in
 * FP32 -- transform grid 1023 x 1023, 12.6 MB -- or a 256 x 256 open film in
 * FP64). */
#define MMC_DEMAG_STATIC_SCRATCH_BYTES (16u * 1024u * 1024u)
/* mmc_demag_apply() for callers that cannot allocate device memory at the
 * point of the call: code that runs inside a device-memory budget owned by
 * another allocator (a framework's caching pool that has claimed the free
 * memory), or a latency-bound loop where cudaMalloc/cudaFree would
 * synchronise the device.  No counterpart in the reference, which keeps its
 * FFT buffers for the whole run (src/main.cu:689-712, 744-755); this entry point and
 * mmc_demag_apply share its transforms.
 *
 * The spectrum lives in a file-scope array of MMC_DEMAG_STATIC_SCRATCH_BYTES
 * that the CUDA runtime reserves when it loads the library's module on a
 * device; nothing is allocated per call, and the tensor is not built here.
 * Rules:
 *   - build the tensor first (mmc_build_demag or any field/run call): building
 *     allocates, so an unbuilt tensor is MMC_ERR_STATE;
 *   - lattices whose spectrum (mmc_demag_scratch_bytes) exceeds the array are
 *     MMC_ERR_INVALID: use mmc_demag_apply with caller scratch;
 *   - the first call on a device looks the array up (cudaGetSymbolAddress),
 *     which may load the module there: make that first call before any stream
 *     capture;
 *   - every call on a device, from every handle, uses the same array: calls
 *     that overlap in time (different streams, threads or handles without an
 *     ordering between them) race on it; calls on one stream are ordered and
 *     safe.  The array needs no initial contents: each call writes every value
 *     it reads.
 * mdev, hdev and stream are as for mmc_demag_apply (NULL stream = the
 * handle's own stream); the work is enqueued, not waited for. */
int mmc_demag_apply_static(mmc_handle* h, const void* mdev, void* hdev, void* stream);

/* Per-term effective field in A/m for the current m, the DEBUG_H_FIELD dumps of
 * src/main.cu:965-1086.  MMC_TERM_DEMAG and MMC_TERM_TOTAL use the demag field
 * of the last mmc_compute_demag() / sweep. */
int mmc_get_field(mmc_handle* h, int term, double* hx, double* hy, double* hz);

/* Energy and observables of the current m (calEnergyKernel + thrust::reduce,
 * src/effective_H.h:35-43, src/main.cu:902-956).  Recomputes the demag field
 * first.  Resets the acceptance counters. */
int mmc_energy(mmc_handle* h, mmc_observables* out);
/* Gradient of the total energy (the five terms of mmc_energy) with respect to
 * m and to the material scalars -- the adjoint the reference does not have
 * (its energy kernel, src/effective_H.h:35-43, computes values only).  The
 * three components of every cell are treated as free variables:
 * dE/dm_i = -mu0 Ms V H_i, with the demag part of H the convolution with the
 * symmetrised tensor (K(r) + K(-r)) / 2 (spectrum Re K^), which is what the
 * energy's derivative needs when periodic images make K slightly
 * non-symmetric.  dE_dm: 3 n doubles (x block, y block, z block; x fastest
 * within a block) or NULL.  dE_dparams: d/d(Aex, Dind, Ku1, Ms, Bextx, Bexty,
 * Bextz) in SI units (J per J/m, J per J/m^2, J per J/m^3, J per A/m, J per T).
 * Accumulated in FP64 from the working-precision m. */
int mmc_grad(mmc_handle* h, double* dE_dm, double dE_dparams[7]);
/* Energy minimisation from the current m: projected steepest descent on the
 * unit sphere (direction P = t - (t.m) m with t = H / Ms, m renormalised every
 * step) with Barzilai-Borwein step lengths s.s / s.y, until
 * max_i |m_i x H_i| / Ms < torque_tol or max_iter updates.  H uses the
 * symmetrised demag field, so P is the projected negative gradient of the
 * energy.  iters receives the updates made, max_torque the last torque (either
 * may be NULL); not reaching torque_tol is not an error -- check max_torque.
 * No counterpart in the reference. */
int mmc_relax(mmc_handle* h, double torque_tol, long long max_iter, long long* iters, double* max_torque);

/* nsweeps Metropolis sweeps at `temperature` (mcKernel2, src/mc_sampling.h:27-41,
 * launched src/main.cu:1101-1120), each preceded by a demag refresh when
 * cal_demag_flag is set.  Random numbers are keyed on (seed, stage, sweep, cell),
 * so splitting a stage into several calls gives the same result. */
int mmc_run_sweeps(mmc_handle* h, double temperature, long long stage, long long sweep0,
                   long long nsweeps);

/* The sweep engine chosen at creation: out[0] = enum mmc_engine (never AUTO),
 * out[1] = rows per CTA of the fused engine, out[2] = its CTA count. */
int mmc_engine_info(mmc_handle* h, int out[3]);

/* Device time, in ms, of the last mmc_run_sweeps() call: CUDA events recorded
 * on the handle's stream around the enqueued sweeps. */
int mmc_last_run_ms(mmc_handle* h, double* ms);

/* Runs nsweeps sweeps like mmc_run_sweeps() but without graphs, timing each
 * group of kernels with CUDA events: out_ms[0] = total of the demag
 * convolutions, out_ms[1] = total of the sweep (Metropolis) kernels,
 * out_ms[2] = whole run.  Used to attribute time per kernel family. */
int mmc_profile_sweeps(mmc_handle* h, double temperature, long long stage, long long sweep0, long long nsweeps,
                       double out_ms[3]);

/* Profiling hook of the fused film engine: runs nsweeps (<= 1024) sweeps in
 * one launch and returns device timestamps (ns) of the phase boundaries of the
 * first 16 sweeps for the first and the last CTA: stamps[(s*9 + p)*2 + c],
 * points p = 0 row phase start, 1 copies landed, 2 demag field ready,
 * 3 Metropolis done, 4 spectrum rows stored, 5 after barrier, 6 column copies
 * landed, 7 column phase done, 8 after barrier.  stamps holds 288 words. */
int mmc_profile_fused(mmc_handle* h, double temperature, long long stage, long long sweep0, long long nsweeps,
                      unsigned long long* stamps);

/* The whole temperature-stage loop of src/main.cu:801-1139 with its outputs
 * (energy.txt, %06ld_%.2fK_%ld.ovf snapshots) written into output_dir.
 * verbose != 0 prints progress lines to stdout.  With cfg.debug_h_field the
 * loop also writes, at every energy output and over the same files, the
 * per-term dumps of the reference's DEBUG_H_FIELD build (src/main.cu:965-1086):
 * B_demag.ovf, B_anis.ovf, B_exch.ovf, B_dmi.ovf, B_effective.ovf (mu0 H in T,
 * B_effective including B_ext) and E_density.ovf (J/m^3 in all three columns;
 * e_i = -(mu0 Ms/2) m_i.(H_ex + H_dm + H_an + H_d) - Ms m_i.B_ext, which sums
 * times V to the total energy), in cfg.ovf_format. */
int mmc_run_anneal(mmc_handle* h, const char* output_dir, int verbose);

/* Asks a running call on another thread (or a signal handler) to stop at the
 * next sweep boundary; that call returns MMC_ERR_INTERRUPTED. */
void mmc_request_stop(mmc_handle* h);

/* ---------------------------------------------------------------- batches
 * No counterpart in the reference, which runs one lattice per process.  A
 * batch advances nrep replicas of one geometry together (every kernel launch
 * covers all replicas), for seed ensembles and parallel tempering.  Replicas
 * share nx, ny, nz, cell size, pbc, precision and the demag flag; material,
 * field, seed and temperature are per replica.  Each replica's trajectory is
 * the one a single handle with the same config produces (same Philox streams,
 * same arithmetic). */
typedef struct mmc_batch mmc_batch;
int mmc_batch_create(const mmc_config* cfgs, int nrep, int device, mmc_batch** out);
void mmc_batch_destroy(mmc_batch* b);
/* As mmc_set_stream, for the batch's work (the replica parts of a launch
 * shape with 2-4 streams fork from this stream and join it again). */
int mmc_batch_set_stream(mmc_batch* b, void* stream);
int mmc_batch_size(mmc_batch* b);
int mmc_batch_build_demag(mmc_batch* b, const char* cache_dir);
/* Per-replica temperatures (K); default Temperature_start of each config. */
int mmc_batch_set_temperatures(mmc_batch* b, const double* T);
int mmc_batch_get_temperatures(mmc_batch* b, double* T);
/* Parallel tempering: nladders ladders of per_ladder replicas; ladder l's
 * replicas[l*per_ladder + k] starts at temps[l*per_ladder + k] (ascending).
 * After every swap_interval sweeps (counted by the global sweep index) the
 * device evaluates all energies and attempts swaps of neighbouring
 * temperatures, alternating even and odd pairs, keyed by `seed`. */
int mmc_batch_set_ladders(mmc_batch* b, int nladders, int per_ladder, const int* replicas, const double* temps,
                          int swap_interval, long long seed);
/* Current replica at each ladder slot and the swap counts {attempted, accepted}. */
int mmc_batch_ladder_state(mmc_batch* b, int* replicas, unsigned long long counts[2]);
int mmc_batch_run_sweeps(mmc_batch* b, long long stage, long long sweep0, long long nsweeps);
/* The stage loop of mmc_run_anneal (src/main.cu:801-1139) for every replica at
 * once: replica r writes energy.txt and its snapshots into
 * <output_dir>/replica_<rrr>/, the same files a single run of its config
 * writes (and with the same numbers: a replica's trajectory is the single
 * run's).  All replicas must share the temperature schedule and the output
 * periods.  Parameter sweeps (the CLI's -farm-Bz= / -farm-D=) run this way. */
int mmc_batch_run_anneal(mmc_batch* b, const char* output_dir, int verbose);
int mmc_batch_last_run_ms(mmc_batch* b, double* ms);
/* Runs nsweeps sweeps without graphs and times each kernel family with CUDA
 * events on the batch's stream (totals in ms).  One kernel per pass:
 * out_ms[0] forward x transform, [1] column passes (y/z transforms with the
 * tensor product), [2] inverse x transform, [3] Metropolis colours.  Film row
 * kernel (launch shape out[5] > 0): [0] row kernel, [1] column pass, [2] = [3]
 * = 0.  [4] = sum. */
int mmc_batch_profile_sweeps(mmc_batch* b, long long stage, long long sweep0, long long nsweeps, double out_ms[5]);
/* Launch shape of the batch's pass kernels: rows per CTA and threads of the x
 * passes, kx columns per tile of the y and z passes, threads of the column
 * passes, the band of the film row kernel (0 when sweeps use one kernel per
 * pass), and the Metropolis form: 0 one launch per colour, 1 both colours of
 * a film in one tile launch, 2 one vectorised launch per colour (films with
 * nx a multiple of 4), 3 the same with each CTA's rows staged in shared
 * memory by asynchronous copies (nx also at most 1024), 4 both colours of a
 * film in one launch over strips of rows (nx a multiple of 4, at most 2048,
 * row kernel off), 5 the staged form run by persistent CTAs with the rows
 * fetched by bulk asynchronous copies (as 3; a run whose buffer wait runs out
 * of its time limit returns MMC_ERR_TIMEOUT), whether the pass kernels expand their transforms in
 * line (1) or call them out of line (0), whether the column passes
 * transform in place reading the tensor from global memory (1; 2 the same,
 * with film y lines of length 64 or 256 held in registers, other lines as 1;
 * 3 as 2 with one component per thread),
 * and the number of streams (1-4) the batch's replicas are split over. */
int mmc_batch_launch_shape(mmc_batch* b, int out[10]);
/* Autotuner: times each launch shape this batch can run with (the film row
 * kernel with each band that fits; the pass kernels with 1-16 rows per x-pass
 * CTA and 1-8 kx columns per column-pass tile, then -- one dimension at a
 * time from the fastest so far -- the transforms in and out of line, the
 * in-place column passes, every Metropolis form, 2-4 streams) for `sweeps`
 * sweeps (the faster of two repetitions; replays of the 32-sweep graph that
 * runs execute, so `sweeps` is rounded up to a multiple of 32) from the
 * current state, keeps the fastest and restores m and the acceptance
 * counters.  Every shape gives bit-identical results, so the choice changes
 * only the speed.  best_ms_per_sweep and candidates may be NULL.  No
 * counterpart in the reference, whose block shape is fixed in the source
 * (src/main.cu:275-286). */
int mmc_batch_autotune(mmc_batch* b, int sweeps, double* best_ms_per_sweep, int* candidates);
/* Sets the launch shape (the ten values of mmc_batch_launch_shape), e.g. one
 * an earlier autotune chose.  Accepted: 1-16 rows per x-pass CTA (a power of
 * two) with 128 or 256 threads, 1-64 kx columns per y- and z-pass tile (powers
 * of two dividing the column-pass thread count, 32-512 threads), tiles whose
 * shared memory fits 220 KB in the chosen column-pass form, a row-kernel band
 * this batch offers, a Metropolis form the lattice qualifies for, 0/1 for the
 * in-line transform flag, 0-3 for the column-pass form and 1-4 streams;
 * anything else is rejected.  Results do
 * not depend on the shape.  No counterpart in the reference. */
int mmc_batch_set_launch_shape(mmc_batch* b, const int shape[10]);

/* Replica farms: batches of different lattice sizes advanced together.  One
 * call runs nsweeps sweeps of every batch (each with its own temperatures,
 * ladders and launch shape); the batches' graphs are enqueued in turn on their
 * own streams so the GPU runs them concurrently.  The farm does not own the
 * batches, which must live on one device; results equal separate
 * mmc_batch_run_sweeps calls.  last_run_ms is host wall time of the whole
 * call.  No counterpart in the reference, which runs one lattice per process
 * (src/main.cu:97-105). */
typedef struct mmc_farm mmc_farm;
int mmc_farm_create(mmc_batch* const* batches, int nbatches, mmc_farm** out);
void mmc_farm_destroy(mmc_farm* f);
int mmc_farm_run_sweeps(mmc_farm* f, long long stage, long long sweep0, long long nsweeps);
int mmc_farm_last_run_ms(mmc_farm* f, double* ms);
void mmc_farm_request_stop(mmc_farm* f);
void mmc_batch_request_stop(mmc_batch* b);
/* Observables of every replica (out holds nrep entries). */
int mmc_batch_energy(mmc_batch* b, mmc_observables* out);
int mmc_batch_set_m(mmc_batch* b, int replica, const double* mx, const double* my, const double* mz);
int mmc_batch_get_m(mmc_batch* b, int replica, double* mx, double* my, double* mz);

/* OVF 1.0/2.0 reader (parseOvfFile, src/ovf_io.h:88-91): text, binary 4 and
 * binary 8 data; dimensions must match and step sizes agree within 1e-5
 * relative (src/ovf_io.h:35-64). */
int mmc_ovf_read(const char* path, int nx, int ny, int nz, double dx, double dy, double dz,
                 double* mx, double* my, double* mz);

/* OVF 2.0 writer (writetoOvfFile, src/ovf_io.h:93-98). */
int mmc_ovf_write(const char* path, int nx, int ny, int nz, double dx, double dy, double dz,
                  const double* mx, const double* my, const double* mz, int format,
                  const char* title);

/* Test hook of failure detection (no counterpart in the reference): runs one
 * CTA that waits at a device barrier for an arrival that never comes, with a
 * budget of spin_limit polls (1 .. 2^24); the wait runs out, the kernel
 * records the timeout and returns, and *status receives MMC_ERR_TIMEOUT (or
 * MMC_OK if the wait had completed).  The device stays usable afterwards --
 * this is how the film engine's barriers report MMC_ERR_TIMEOUT. */
int mmc_selftest_barrier_timeout(int device, long long spin_limit, int* status);

/* Test hook of failure detection (no counterpart in the reference): one
 * thread waits on a shared-memory transaction barrier (mbarrier) that expects
 * an arrival that never comes -- the wait the pipelined Metropolis form makes
 * for its staged rows -- for at most limit_ns nanoseconds (1 .. 1e9) of the
 * device's global timer; *status receives MMC_ERR_TIMEOUT when the wait gave
 * up (MMC_OK if it had completed).  No copy is in flight, and the device stays
 * usable afterwards.  A run whose pipelined buffer wait gives up returns
 * MMC_ERR_TIMEOUT the same way. */
int mmc_selftest_mbar_timeout(int device, long long limit_ns, int* status);

/* Test hook (no counterpart in the reference, whose random pools came from
 * cuRAND's host API, src/main.cu:351-385): evaluates Philox4x32-10 on device
 * `device` for n counters ctr[4*i..4*i+3] and key (k0, k1).  out receives this
 * library's result and out_curand cuRAND's curand_Philox4x32_10; either may be
 * NULL.  Both arrays hold 4*n words. */
int mmc_selftest_philox(int device, long long n, const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out,
                        uint32_t* out_curand);

#ifdef __cplusplus
}
#endif
#endif /* MMC_H_ */
