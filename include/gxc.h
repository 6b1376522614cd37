/*
 * gxc.h — C ABI of the GB300 FX correlator engine (libgxcorr.so).
 *
 * This is the drop-in boundary for the reference's FxKernel API
 * (fxkernel/src/fxkernel.h:29-64): configure antennas, channels and the delay
 * model, process one sub-integration of packed dual-pol voltages, accumulate
 * visibilities.  Plain C types only (a CUDA stream is passed as void*), status
 * codes instead of exit(), caller-owned buffers, all device work on the
 * caller's stream.  A handle is not thread-safe: use one per host thread, as
 * the reference uses one FxKernel per thread (fxkernel/src/bench_fxkernel.cpp:93-139).
 *
 * Input format (per antenna, one buffer of (nfft+1) FFT windows):
 *   2-bit real:    4 samples per byte, A_t | B_t<<2 | A_t+1<<4 | B_t+1<<6,
 *                  levels {-3.3359,-1,+1,+3.3359} (fxkernel/src/fxkernel.cpp:15-28);
 *                  nchan*(nfft+1) bytes, as fxkernel/src/common.cpp:82.
 *   8-bit complex: int8 A.re, A.im, B.re, B.im per time sample;
 *                  4*nchan*(nfft+1) bytes.
 * Delay model: per antenna poly[3] = coefficients of t^2, t, 1 (seconds, t in
 *   FFT intervals) and a file-start offset fso (seconds) (fxkernel/src/common.h:38-39).
 * Output layout GXC_LAYOUT_FXKERNEL: complex float (re,im interleaved)
 *   [nbl][4][nchan]; cross baselines in fxkernel order (0,1),(0,2)..(nant-2,nant-1)
 *   (fxkernel/src/fxkernel.cpp:328-355), products AA,AB,BA,BB = X_j,l * conj(X_k,m);
 *   when autos are on, nant auto baselines (0,0),(1,1).. follow.
 *   Each baseline is divided by its count of FFTs where both antennas were
 *   valid (fxkernel/src/fxkernel.cpp:358-367).
 */
#ifndef GXC_H
#define GXC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gxc_status {
  GXC_OK = 0,
  GXC_ERR_INVALID_ARGUMENT = 1, /* bad configuration or argument (reference: exit(1), fxkernel.cpp:46-63) */
  GXC_ERR_UNSUPPORTED = 2,      /* valid request this build does not implement */
  GXC_ERR_CUDA = 3,             /* a CUDA runtime call failed; see gxc_last_error */
  GXC_ERR_OUT_OF_MEMORY = 4,
  GXC_ERR_STATE = 5,            /* call order: process() before set_input()/set_delays() */
  GXC_ERR_TIMEOUT = 6,          /* a bounded device-side wait gave up */
  GXC_END_OF_DATA = 7           /* a raw-file reader reached the end of a file (fxkernel/src/common.cpp:43-44) */
} gxc_status;

enum { GXC_PRECISION_FP32 = 0, GXC_PRECISION_FP16 = 1, GXC_PRECISION_FP8 = 2 };
/* EXACT: linear fringe phase per sample; FXKERNEL: the reference's sub/step
 * rotator table including its real-data half-rate step (fxkernel.cpp:112,553-558). */
enum { GXC_ROTATOR_EXACT = 0, GXC_ROTATOR_FXKERNEL = 1 };
/* X-stage engine.  TENSOR: tcgen05 MMAs with FP32 accumulation in tensor memory;
 * FP16 data uses kind::f16, FP32 data a hi/lo TF32 split (hi.hi + lo.hi + hi.lo,
 * every product exact; tensor memory is drained every 128 FFTs, which bounds the
 * bias of its round-towards-zero accumulation at about 3e-6 relative).
 * TENSOR covers up to 64 antennas with FP16 data and up to 32 with FP32 data.
 * CUDA_CORE: plain FP32 FMAs.  AUTO: TENSOR when the shape fits, else CUDA_CORE. */
enum { GXC_XENGINE_AUTO = 0, GXC_XENGINE_CUDA_CORE = 1, GXC_XENGINE_TENSOR = 2 };
/* F-stage FFT engine.  TENSOR: the FFT as two dense DFT products on tcgen05 (FP16
 * operands, FP32 accumulation), for FP16 / FP8 channelised output of 8192-point
 * windows of 2-bit real data (nchan 4096); it adds four FP16 roundings inside the
 * FFT.  CUDA_CORE: the FP32 register FFT of every shape.  AUTO: TENSOR where it
 * runs, the faster of the two on GB300 (16 antennas, nchan 4096, FP16: 36.2 against
 * 40.1 ms per sub-integration), else CUDA_CORE. */
enum { GXC_FFT_AUTO = 0, GXC_FFT_CUDA_CORE = 1, GXC_FFT_TENSOR = 2 };
/* FFT-range split of the FP16 / FP8 tensor-core X-stage: each channel group's FFTs of a block go to
 * two CTAs, the second accumulating into a second plane that finalisation adds.  AUTO: split when
 * the channel groups are fewer than the SMs.  OFF: never.  ON: whenever the block holds at least
 * four K chunks of FFTs (more CTAs than the groups alone give, each paying its own pipeline fill). */
enum { GXC_XSPLIT_AUTO = 0, GXC_XSPLIT_OFF = 1, GXC_XSPLIT_ON = 2 };
/* Scaling of FP8 (E4M3) channelised data.  CHANNEL: every process() first channelises its first
 * few FFTs in FP32 (up to 64, fewer for very large arrays), measures each channel's RMS over those
 * FFTs and all streams, and casts each channel with its own power of two that puts that RMS near 4
 * (E4M3's largest finite value is 448); finalisation divides each channel by its scale squared,
 * exactly.  A band with a steep bandpass keeps every channel in E4M3's normal range.  HANDLE: one
 * power of two for every channel, from the FFT length and the sample format. */
enum { GXC_FP8_SCALE_CHANNEL = 0, GXC_FP8_SCALE_HANDLE = 1 };
enum { GXC_LAYOUT_FXKERNEL = 0 };

typedef struct gxc_config {
  int nant;        /* antennas (>= 1) */
  int nchan;       /* output channels; FFT length is 2*nchan (real) or nchan (complex), a power of two */
  int nfft;        /* FFTs per sub-integration */
  int nbit;        /* 2 (real) or 8 (complex) */
  int is_complex;  /* 0 real-sampled, 1 complex-sampled */
  double lo_hz;    /* local oscillator frequency (Hz) */
  double bw_hz;    /* bandwidth (Hz) */
  int precision;   /* GXC_PRECISION_*: element type of the channelised data fed to the X-stage */
  int rotator;     /* GXC_ROTATOR_* */
  int autos;       /* 1: append autocorrelations */
  int x_engine;    /* GXC_XENGINE_* */
  int fft_block;   /* FFTs per F/X pass; 0 = automatic */
  int device;      /* CUDA device ordinal; -1 = current device */
  int fft_engine;  /* GXC_FFT_* */
  int x_split;     /* GXC_XSPLIT_* */
  int fp8_scaling; /* GXC_FP8_SCALE_* (FP8 precision only) */
} gxc_config;

typedef struct gxc_handle gxc_handle;

/* Defaults: 2-bit real, FP32, exact rotator, autos on, automatic engines and block. */
void gxc_config_init(gxc_config *cfg);
/* Checks a configuration without touching the GPU. */
gxc_status gxc_validate_config(const gxc_config *cfg);
/* Bytes of packed input per antenna for one sub-integration (see header comment). */
size_t gxc_input_bytes_per_antenna(const gxc_config *cfg);
/* Output baselines: nant*(nant-1)/2 crosses (+ nant autos when enabled). */
int gxc_num_baselines(const gxc_config *cfg);
/* Bytes from the start of every antenna's input buffer that the FFTs [t0, t0+nt) of one
 * sub-integration read, for the delay model (poly [nant][3], fso [nant]) as passed to
 * gxc_set_delays: an upper bound from the delay polynomial's extremes over those FFTs (the exact
 * windows, fxkernel/src/fxkernel.cpp:288-309, are computed on the device).  A caller that loads
 * the input in time order may start the F-stage of those FFTs once this prefix of every antenna
 * is in place; the streaming pipeline does so.  Returns 0 for invalid arguments. */
long long gxc_input_bytes_for_ffts(const gxc_config *cfg, const double *poly, const double *fso, int t0, int nt);
const char *gxc_status_string(gxc_status s);

/* FxKernel::FxKernel (fxkernel/src/fxkernel.cpp:30-180): allocates device state. */
gxc_status gxc_create(const gxc_config *cfg, gxc_handle **out);
/* FxKernel::~FxKernel. */
gxc_status gxc_destroy(gxc_handle *h);

/* FxKernel::setInputData (fxkernel/src/fxkernel.cpp:242-245): per_ant[a] points at
 * bytes_per_ant bytes for antenna a, host (pageable or pinned) or device memory.
 * Device buffers are borrowed, must be 16-byte aligned and must outlive process(); host buffers are
 * copied to the device inside every process() call, on the handle's own copy stream (forked from and
 * joined back to the caller's stream) in time-ordered chunks that the F-stage starts on as they land;
 * pinned host memory gives the fastest copies. */
gxc_status gxc_set_input(gxc_handle *h, const uint8_t *const *per_ant, size_t bytes_per_ant);
/* FxKernel::setDelays (fxkernel/src/fxkernel.cpp:247-251): poly [nant][3], fso [nant]
 * (host memory).  Values are copied at this call. */
gxc_status gxc_set_delays(gxc_handle *h, const double *poly, const double *fso);
/* Optional per-antenna frame validity, e.g. from gxc_vdif_depacketize: valid[a]
 * points at uint8 [nframes] device flags of antenna a's input (frame f holds
 * samples [f*samples_per_frame, (f+1)*samples_per_frame) of the buffer; a null
 * entry means all valid).  Every FFT whose window touches a zero flag is flagged
 * like a window outside the buffer (not correlated, not counted).  nframes must
 * cover the (nfft+1)*F samples of the buffer.  valid == NULL removes the flags.
 * The reference has no such input: its data windows are only flagged by the
 * delay geometry (fxkernel/src/fxkernel.cpp:288-309). */
gxc_status gxc_set_frame_validity(gxc_handle *h, const uint8_t *const *valid, size_t nframes,
                                  int64_t samples_per_frame);
/* FxKernel::process (fxkernel/src/fxkernel.cpp:253-368): one sub-integration,
 * enqueued asynchronously on `stream` (a cudaStream_t; NULL = default stream).
 * Overwrites the handle's visibilities. */
gxc_status gxc_process(gxc_handle *h, void *stream);
/* Waits for the last process() on its stream. */
gxc_status gxc_sync(gxc_handle *h);
/* FxKernel::accumulate (fxkernel/src/fxkernel.cpp:414-423): odata += visibilities,
 * odata complex float [nbl][4][nchan], host or device memory.  Synchronises. */
gxc_status gxc_accumulate(gxc_handle *h, float *odata);
/* Copies (not adds) the visibilities into out (host or device), synchronising. */
gxc_status gxc_get_visibilities(gxc_handle *h, float *out);
/* Device pointer of the handle's visibility buffer (valid until the next
 * process() or destroy); complex float [nbl][4][nchan]. */
const float *gxc_device_visibilities(const gxc_handle *h);
/* Per-baseline count of FFTs where both antennas were valid (int32 [nbl], host). */
gxc_status gxc_get_baseline_counts(gxc_handle *h, int32_t *counts);
/* Per-(antenna, FFT) validity flags (uint8 [nant][nfft], host), the reference's antValid. */
gxc_status gxc_get_valid_flags(gxc_handle *h, uint8_t *flags);
/* Text message of the last failing call on this handle ("" if none). */
const char *gxc_last_error(const gxc_handle *h);

/* Test entry for the unpack step: runs process() (device inputs only), then runs
 * the F-stage kernels again with a probe that writes every decoded input sample,
 * as the kernel holds it before the fringe rotation, to `decoded` (host or device):
 * complex float [nant][2 pols][nfft][F].  The kernels are the production
 * templates built with the probe write (the decode is the same code); samples of
 * flagged FFTs stay NaN.  It replaces no reference member: it lets tests compare
 * the GPU decode with the reference's unpack (fxkernel/src/fxkernel.cpp:15-28,
 * :443-487) bit for bit.  Synchronous; allocates its scratch with cudaMalloc. */
gxc_status gxc_probe_unpack(gxc_handle *h, float *decoded);

/* Number of kernel launches the last process() enqueued (for accounting). */
int gxc_last_launch_count(const gxc_handle *h);
/* Effective FFT block (FFTs per F/X pass) chosen for this handle. */
int gxc_fft_block(const gxc_handle *h);
/* F/X passes of the last process(): nfft / fft_block rounded up; when the inputs are on the
   host and the block was chosen, the passes cover 4096, 8192, ... FFTs up to the block (the
   compute starts after a shorter copy), which can add passes. */
int gxc_num_blocks(const gxc_handle *h);
/* F-stage engine this handle runs: GXC_FFT_TENSOR or GXC_FFT_CUDA_CORE (AUTO resolved). */
int gxc_fft_engine(const gxc_handle *h);

/* Stage timing: when enabled, process() records CUDA events around the F-stage
 * and X-stage launches; gxc_stage_times returns the summed milliseconds of the
 * last process() (f_ms, x_ms, other_ms).  Synchronises. */
gxc_status gxc_enable_stage_timing(gxc_handle *h, int enable);
gxc_status gxc_stage_times(gxc_handle *h, float *f_ms, float *x_ms, float *total_ms);

/* Batches of independent jobs of uneven size (antenna counts, channel counts,
 * formats, lengths), launched as one CUDA graph whose parallel branches are the
 * jobs' launch sequences; the GPU overlaps the jobs.  The reference runs one
 * FxKernel per sub-integration and thread (fxkernel/src/bench_fxkernel.cpp:93-139)
 * and has no batch API; this replaces that thread replication on one GPU.
 * inputs are device pointers (16-byte aligned), or pinned host pointers: then each
 * launch copies them host->device at the head of that job's graph branch, so the
 * copies of some jobs overlap the correlation of others.  The input addresses and
 * delays are fixed when the batch is created (the buffers' contents are read at
 * every launch; create a new batch to change addresses or delays).  Creation runs every
 * job once.  Results: gxc_get_visibilities(gxc_batch_job(b, i), out) after the
 * launch's stream has completed. */
typedef struct gxc_job {
  gxc_config cfg;
  const uint8_t *const *inputs; /* [nant] device buffers or pinned host buffers */
  const double *poly;           /* [nant][3] */
  const double *fso;            /* [nant] */
} gxc_job;
typedef struct gxc_batch gxc_batch;
gxc_status gxc_batch_create(const gxc_job *jobs, int njobs, gxc_batch **out);
gxc_status gxc_batch_launch(gxc_batch *b, void *stream);
int gxc_batch_size(const gxc_batch *b);
gxc_handle *gxc_batch_job(gxc_batch *b, int i);
/* Kernel launches one batch launch contains (the sum over its jobs). */
int gxc_batch_launch_count(const gxc_batch *b);
gxc_status gxc_batch_destroy(gxc_batch *b);

/* Streaming ingest of consecutive sub-integrations (one configuration) from host
 * memory.  Replaces the reference GPU driver's copy-then-wait-for-the-previous-
 * stream loop (gcorr/src/testgpukernel.cu:462-486) and the CPU driver's
 * process()+accumulate() per sub-integration (fxkernel/src/testfxkernel.cpp:81-108).
 * The pipeline owns `nslots` (1..8) device input slots, a copy stream and a
 * compute stream: submit() enqueues the host->device copy of sub-integration
 * k into slot k % nslots (after that slot's previous sub-integration finished)
 * and its correlation behind that copy, so copies overlap the previous
 * sub-integration's F and X stages.  submit() returns once the work is
 * enqueued; inputs[a] and vis_out must stay valid and untouched until
 * gxc_pipeline_wait(seq) returns.  Use pinned host memory (cudaHostAlloc /
 * cudaHostRegister) for inputs and vis_out: pageable buffers make the copies
 * synchronous and remove the overlap.  vis_out (optional; host or device) receives
 * this sub-integration's visibilities in GXC_LAYOUT_FXKERNEL.  With integrate != 0
 * every sub-integration's (normalised) visibilities are also added into a
 * device-side compensated FP32 sum: the reference's accumulate() over a long
 * integration (fxkernel/src/fxkernel.cpp:414-423), read by
 * gxc_pipeline_integration (synchronises; reset != 0 clears it).
 *
 * Linear->circular polarisation conversion, the voltage-domain transform of
 * examples/chris/bench/gpubench.cu:145-160 (P1' = g1*P1 - g2*P2,
 * P2' = g1*P1 + g2*P2 per antenna and channel), applied exactly to the
 * visibilities as V' = J_j V J_k^H with J = [[g1, -g2], [g1, g2]].  gains:
 * complex float [nant][2][nchan] (g1 then g2 per antenna), host or device; null =
 * ideal feeds, g1 = 1/sqrt(2), g2 = i/sqrt(2).  gxc_pipeline_set_lin2circ applies it
 * to every later sub-integration before integration and copy-out; gxc_lin2circ
 * converts a device buffer [nbl][4][nchan] in place (gains then device memory or
 * null) on `stream`. */
typedef struct gxc_pipeline gxc_pipeline;
gxc_status gxc_pipeline_create(const gxc_config *cfg, int nslots, int integrate, gxc_pipeline **out);
gxc_status gxc_pipeline_submit(gxc_pipeline *p, const uint8_t *const *inputs, const double *poly, const double *fso,
                               float *vis_out, int64_t *seq);
gxc_status gxc_pipeline_wait(gxc_pipeline *p, int64_t seq);
gxc_status gxc_pipeline_sync(gxc_pipeline *p);
gxc_status gxc_pipeline_integration(gxc_pipeline *p, float *out, int reset, int *nsub);
gxc_status gxc_pipeline_set_lin2circ(gxc_pipeline *p, int enable, const float *gains);
gxc_handle *gxc_pipeline_handle(gxc_pipeline *p);
const char *gxc_pipeline_last_error(const gxc_pipeline *p);
gxc_status gxc_pipeline_destroy(gxc_pipeline *p);
gxc_status gxc_lin2circ(float *vis, const float *gains, int nant, int nchan, int autos, void *stream);

/* Harness file formats (host side).
 * .conf files (fxkernel/src/common.cpp:54-114, parseConfig): keywords NBIT, NPOL,
 * COMPLEX, NCHAN, LO, BANDWIDTH, NUMFFTS, NANT (case-insensitive), then NANT lines
 * "name file p0 p1 p2 fso".  gxc_conf_config copies nant, nchan, nfft, nbit,
 * is_complex, lo and bw into cfg and leaves its other fields alone; it returns
 * GXC_ERR_UNSUPPORTED unless NPOL is 2.  gxc_conf_int takes NBIT, NPOL, COMPLEX,
 * NCHAN, NUMFFTS or NANT (-1 otherwise); gxc_conf_double takes LO or BANDWIDTH.
 * gxc_conf_delays fills poly[nant][3] and fso[nant] (either may be null).
 * Raw files (common.cpp:38-52, readdata): each gxc_reader_read fills bufs[a] with
 * the next bytes_per_read bytes of file a (files read in parallel) and returns
 * GXC_END_OF_DATA when any file ends.
 * gxc_save_visibilities writes vis ([nbl][4][nchan] complex float, host) in the
 * vis.out text format of FxKernel::saveVisibilities (fxkernel/src/fxkernel.cpp:370-412).
 * gxc_host_alloc / gxc_host_free: pinned host buffers, as allocDataHost uses for
 * GPU input (common.cpp:3-36). */
typedef struct gxc_conffile gxc_conffile;
gxc_status gxc_conf_read(const char *path, gxc_conffile **out);
gxc_status gxc_conf_config(const gxc_conffile *cf, gxc_config *cfg);
int gxc_conf_int(const gxc_conffile *cf, const char *key);
double gxc_conf_double(const gxc_conffile *cf, const char *key);
const char *gxc_conf_antenna_name(const gxc_conffile *cf, int a);
const char *gxc_conf_antenna_file(const gxc_conffile *cf, int a);
gxc_status gxc_conf_delays(const gxc_conffile *cf, double *poly, double *fso);
void gxc_conf_free(gxc_conffile *cf);
typedef struct gxc_reader gxc_reader;
gxc_status gxc_reader_open(const char *const *paths, int nant, size_t bytes_per_read, gxc_reader **out);
gxc_status gxc_reader_read(gxc_reader *r, uint8_t *const *bufs);
gxc_status gxc_reader_close(gxc_reader *r);
gxc_status gxc_save_visibilities(const char *path, const float *vis, int nbl, int nchan, double bw_hz);
gxc_status gxc_host_alloc(size_t bytes, void **out);
gxc_status gxc_host_free(void *p);

/* VDIF input.  gxc_vdif_parse_header decodes a 16- or 32-byte VDIF frame header
 * (host memory; the fields the reference reads in examples/mark/dump_vdif.py:40-55).
 * gxc_vdif_depacketize places the frames of one antenna's stream (device memory,
 * nbytes of back-to-back frames of frame_bytes each, header included) into that
 * antenna's engine input buffer `out` (device, nslots*payload_bytes bytes): the
 * frame of second `s` and number `f` goes to slot (s - seconds0)*frames_per_second
 * + f - frame0, as the reference's ingest orders frames (ingest/src/ingest.c:267-330).
 * Frames that are marked invalid, malformed (length field != frame_bytes, payload !=
 * payload_bytes), of another thread (thread_id >= 0) or outside [0, nslots) are
 * skipped; valid[slot] (device, uint8 [nslots]) is 1 for a slot that was filled,
 * and empty slots are set to `fill`.  Two-channel VDIF payloads are the engine's
 * input layout (2-bit: channel = polarisation, codes 0..3 = the fxkernel levels;
 * 8-bit complex: ch0 re, im, ch1 re, im); offset_binary_8bit != 0 converts 8-bit
 * offset-binary samples to int8.  stats (device, optional) accumulates
 * [accepted, skipped outside window / other thread, invalid or malformed].  Pass
 * valid to gxc_set_frame_validity to flag the FFTs that touch empty slots.
 * Asynchronous on `stream`. */
typedef struct gxc_vdif_header {
  int invalid, legacy;
  int64_t seconds;   /* seconds from the reference epoch */
  int ref_epoch;     /* half-years since 2000 */
  int frame;         /* frame number within the second */
  int version, nchan, frame_bytes, is_complex, bits, thread, station, header_bytes;
} gxc_vdif_header;
gxc_status gxc_vdif_parse_header(const uint8_t *header, gxc_vdif_header *out);
gxc_status gxc_vdif_depacketize(const uint8_t *frames, size_t nbytes, int frame_bytes, int payload_bytes,
                                int64_t seconds0, int frame0, int frames_per_second, int thread_id,
                                int offset_binary_8bit, uint8_t fill, uint8_t *out, size_t nslots, uint8_t *valid,
                                unsigned long long *stats, void *stream);

/* PSRDADA streams.  The reference's ingest writes each station's VDIF payloads, headers stripped,
 * into a PSRDADA ring buffer behind an ASCII header ("KEY value  # comment" lines in the first
 * HDR_SIZE bytes, ingest/src/ingest.c:185-330, ingest/src/dada_header_template_atca.txt).  A
 * stream saved from such a ring (header, then data) holds one antenna's samples in this engine's
 * input layout.  gxc_dada_parse_header decodes a header text (absent numbers are -1, absent
 * reals 0, "unset" strings empty); gxc_dada_header_value returns one key's value token.
 * gxc_dada_config copies nbit, is_complex (NDIM 2), bw (|BW|) and lo (FREQ - |BW|/2, the band
 * edge) into cfg and returns GXC_ERR_UNSUPPORTED unless NPOL is 2.  gxc_dada_open opens one stream
 * per antenna and positions each after its header; every gxc_dada_read then fills bufs[a] with the
 * next bytes_per_read bytes of stream a (offset_binary_8bit != 0 converts 8-bit offset-binary
 * samples to two's complement) and returns GXC_END_OF_DATA when any stream ends.  Attaching to a
 * live shared-memory ring needs the psrdada library and is not built. */
typedef struct gxc_dada_header {
  long long hdr_size;                 /* HDR_SIZE (4096 when absent) */
  int nbit, npol, ndim, nchan;        /* NBIT, NPOL, NDIM (1 real, 2 complex), NCHAN */
  double bw_mhz, freq_mhz, tsamp_us;  /* BW, FREQ (band centre), TSAMP */
  long long bytes_per_second, obs_offset, picoseconds;
  double mjd_start;
  char utc_start[32];
  char source[64];
} gxc_dada_header;
typedef struct gxc_dada_reader gxc_dada_reader;
gxc_status gxc_dada_parse_header(const char *text, size_t len, gxc_dada_header *out);
gxc_status gxc_dada_header_value(const char *text, size_t len, const char *key, char *value, size_t value_len);
gxc_status gxc_dada_config(const gxc_dada_header *hdr, gxc_config *cfg);
gxc_status gxc_dada_open(const char *const *paths, int nant, size_t bytes_per_read, int offset_binary_8bit,
                         gxc_dada_reader **out);
gxc_status gxc_dada_header_of(const gxc_dada_reader *r, int a, gxc_dada_header *out);
gxc_status gxc_dada_read(gxc_dada_reader *r, uint8_t *const *bufs);
gxc_status gxc_dada_close(gxc_dada_reader *r);

/* The X-stage alone, on already-channelised data, as the reference GPU X kernels
 * take it (gcorr/src/gxkernel.h:86-88, CrossCorrAccumHoriz/CCAH2/CCAH3;
 * layout gcorr/src/gxkernel.h:30-44): ants is complex float
 * [nant][2 pols][nfft*fftwidth] with sample f*fftwidth + chan (chan < nchan),
 * host or device memory.  accum receives complex float [nbl][4][nchan]
 * (crosses in fxkernel order, then autos when autos != 0), each product
 * summed over the nfft spectra and divided by nfft as CCAH3 does
 * (gcorr/src/gxkernel.cu:574-581).  precision: GXC_PRECISION_FP32 or _FP16
 * (values cast to FP16 unscaled); x_engine: GXC_XENGINE_* (as for gxc_config).  Synchronous on
 * `stream`; allocates its scratch with cudaMalloc. */
gxc_status gxc_xcorr(const float *ants, int nant, int nfft, int nchan, int fftwidth, int precision, int x_engine,
                     int autos, float *accum, void *stream);

/* gxc_xcorr for callers that cannot allocate device memory.  No counterpart in
 * the reference: it exists for code where cudaMalloc is off limits (a host
 * callback or real-time ingest thread that must not block on the allocator,
 * which can synchronise the device; a process whose GPU memory budget belongs
 * to a framework that owns every allocation).  Same arguments and results as
 * gxc_xcorr with the CUDA-core engine, with these differences:
 *   - precision GXC_PRECISION_FP32 or _FP16 only (FP8: GXC_ERR_UNSUPPORTED);
 *   - ants and accum must be device memory of the current device (host buffers,
 *     which gxc_xcorr stages, return GXC_ERR_INVALID_ARGUMENT);
 *   - it only enqueues work on `stream`: synchronise before reading accum.
 * The scratch lives in one fixed array of GXC_XCORR_NOALLOC_SCRATCH_BYTES held
 * by every GPU that loads the library until the process exits.  Problems whose
 * accumulators (nbl*4*nchan complex float, twice) plus one FFT of channelised
 * data do not fit are rejected with GXC_ERR_INVALID_ARGUMENT.  The first call on
 * a device looks up the array's device address and may load the library's device
 * code: make it at initialisation, before any stream capture and outside any
 * thread that must not block.  Calls after a cudaDeviceReset are not supported.
 * All calls share the array: calls that overlap on the GPU (other streams or
 * host threads) race on it, so serialise them on one stream. */
#define GXC_XCORR_NOALLOC_SCRATCH_BYTES (16u << 20)
gxc_status gxc_xcorr_noalloc(const float *ants, int nant, int nfft, int nchan, int fftwidth, int precision,
                             int autos, float *accum, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GXC_H */
