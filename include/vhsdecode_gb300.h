/*
 * vhsdecode_gb300 -- C ABI of the GB300 (sm_103a) RF decode backend.
 *
 * Drop-in for the reference's native `cuda-fast` boundary
 * (src/VHSDecode.CudaFast.Native/include/vhsdecode_cuda_fast.h:26-174 in
 * vhs-decode-dotnet): same status codes, enums, callback shapes, versioned
 * structs that start with `struct_size`, a thread-local last error and a
 * whole-run entry point.  The managed side binds it through P/Invoke exactly
 * as Core/Dsp/CudaFast/CudaFastNativeRuntime.cs:131-185 binds the cuda-fast
 * library (NativeLibrary.Load + GetExport, ABI version check).
 *
 * Beyond the run() handoff it exposes a session API that keeps a capture and
 * every intermediate on the device (used by the serving loop, the parity tests
 * and the benchmark), and a few stage-level entry points used by the tests.
 *
 * All functions are safe to call on a machine without a GPU: they then return
 * VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE (or do host-only work).
 */
#ifndef VHSDECODE_GB300_H
#define VHSDECODE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#  if defined(VHSDECODE_GB300_EXPORTS)
#    define VHSDECODE_GB300_API __declspec(dllexport)
#  else
#    define VHSDECODE_GB300_API __declspec(dllimport)
#  endif
#  define VHSDECODE_GB300_CALL __cdecl
#else
#  define VHSDECODE_GB300_API __attribute__((visibility("default")))
#  define VHSDECODE_GB300_CALL
#endif

#define VHSDECODE_GB300_ABI_VERSION 0x00010005u
#define VHSDECODE_GB300_NAME_CAPACITY 128u

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: values of vhsdecode_cuda_fast_status (vhsdecode_cuda_fast.h:26-36). */
typedef enum vhsdecode_gb300_status {
    VHSDECODE_GB300_STATUS_OK = 0,
    VHSDECODE_GB300_STATUS_NULL_POINTER = -20000,
    VHSDECODE_GB300_STATUS_INVALID_ARGUMENT = -20001,
    VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE = -20002,
    VHSDECODE_GB300_STATUS_INPUT_ERROR = -20003,
    VHSDECODE_GB300_STATUS_OUTPUT_ERROR = -20004,
    VHSDECODE_GB300_STATUS_DECODE_ERROR = -20005,
    VHSDECODE_GB300_STATUS_CANCELLED = -20006,
    VHSDECODE_GB300_STATUS_INTERNAL_ERROR = -20007
} vhsdecode_gb300_status;

/* vhsdecode_cuda_fast_profile (vhsdecode_cuda_fast.h:38-42); PAL_M is rejected. */
typedef enum vhsdecode_gb300_profile {
    VHSDECODE_GB300_PROFILE_NTSC = 0,
    VHSDECODE_GB300_PROFILE_PAL = 1,
    VHSDECODE_GB300_PROFILE_PAL_M = 2
} vhsdecode_gb300_profile;

/* vhsdecode_cuda_fast_tape_speed (:44-48).  LP and EP apply the format's
 * sub-deemphasis to VHS (S-VHS LP/EP equal S-VHS SP). */
typedef enum vhsdecode_gb300_tape_speed {
    VHSDECODE_GB300_TAPE_SPEED_SP = 0,
    VHSDECODE_GB300_TAPE_SPEED_LP = 1,
    VHSDECODE_GB300_TAPE_SPEED_EP = 2
} vhsdecode_gb300_tape_speed;

/* Tape format: the reference's --tape_format values VHS and SVHS (format
 * parameter snapshot cases <system>/VHS/sp and <system>/SVHS/sp).  The
 * reference's cuda-fast ABI has no such field (it decodes VHS only). */
typedef enum vhsdecode_gb300_tape_format {
    VHSDECODE_GB300_TAPE_FORMAT_VHS = 0,
    VHSDECODE_GB300_TAPE_FORMAT_SVHS = 1
} vhsdecode_gb300_tape_format;

/* vhsdecode_cuda_fast_input_sample_format (:50-53), plus FLAC: the read
 * callback delivers the bytes of a FLAC stream of 16-bit mono samples (a .ldf
 * capture), sample_offset and sample_count counting bytes, and the stream is
 * decoded on the device.  The reference decodes .ldf on the managed side
 * through libsndfile or ffmpeg (Core/Rf/RfLoaderFactory.cs:35,136). */
typedef enum vhsdecode_gb300_input_sample_format {
    VHSDECODE_GB300_INPUT_FLOAT32 = 0,
    VHSDECODE_GB300_INPUT_INT16 = 1,
    VHSDECODE_GB300_INPUT_FLAC = 2
} vhsdecode_gb300_input_sample_format;

/* Arithmetic of the block demodulator. */
typedef enum vhsdecode_gb300_precision {
    VHSDECODE_GB300_PRECISION_FP32_FUSED = 0, /* cluster-fused FP32, FP64 sync/TBC */
    VHSDECODE_GB300_PRECISION_FP64_PLAIN = 1  /* one block at a time, FP64 throughout */
} vhsdecode_gb300_precision;

/* Callbacks: shapes of vhsdecode_cuda_fast_read_callback / cancel_callback (:55-62).
 * read: copy up to sample_count samples (int16, or float for input format
 * FLOAT32) starting at sample_offset into destination and return the count; a
 * short count means end of input, 0 means end of input or failure.  Offsets and
 * counts are source samples (before any device decimation). cancel: return
 * nonzero to cancel. */
typedef size_t (VHSDECODE_GB300_CALL *vhsdecode_gb300_read_callback)(
    void* user_data, void* destination, uint64_t sample_offset, size_t sample_count);
typedef int32_t (VHSDECODE_GB300_CALL *vhsdecode_gb300_cancel_callback)(void* user_data);

/* vhsdecode_cuda_fast_runtime_info_v1 (:71-81). */
typedef struct vhsdecode_gb300_runtime_info_v1 {
    uint32_t struct_size;
    uint32_t abi_version;
    int32_t device_id;
    int32_t compute_major;
    int32_t compute_minor;
    int32_t multiprocessor_count;
    uint64_t total_vram_bytes;
    uint64_t free_vram_bytes;
    char device_name[VHSDECODE_GB300_NAME_CAPACITY];
} vhsdecode_gb300_runtime_info_v1;

/* vhsdecode_cuda_fast_config_v1 (:83-98), same fields and order. */
typedef struct vhsdecode_gb300_config_v1 {
    uint32_t struct_size;
    uint32_t profile;
    uint32_t tape_speed;
    int32_t device_id;
    double sample_rate_mhz;     /* decode rate (the source runs at factor x this) */
    uint64_t total_samples;     /* source samples */
    const char* output_base_utf8;
    int32_t overwrite;
    uint32_t input_sample_format;
    uint32_t maximum_output_fields;
    uint32_t device_decimation_factor;  /* 1, or 2: 2:1 half-band FIR on the device */
    vhsdecode_gb300_read_callback read_callback;
    vhsdecode_gb300_cancel_callback cancel_callback;
    void* user_data;
} vhsdecode_gb300_config_v1;

/* config_v1 followed by the tape format and decode flags.  run() takes either
 * struct, told apart by struct_size (config_v1 decodes VHS with neutral
 * chroma, as cuda-fast).  decode_flags: 0, or VHSDECODE_GB300_DECODE_CHROMA to
 * decode the colour-under chroma into _chroma.tbc (the managed decoder's
 * output, whose burst refinement also moves the luma line locations); other
 * bits must be zero. */
typedef struct vhsdecode_gb300_config_v2 {
    uint32_t struct_size;
    uint32_t profile;
    uint32_t tape_speed;
    int32_t device_id;
    double sample_rate_mhz;
    uint64_t total_samples;
    const char* output_base_utf8;
    int32_t overwrite;
    uint32_t input_sample_format;
    uint32_t maximum_output_fields;
    uint32_t device_decimation_factor;
    vhsdecode_gb300_read_callback read_callback;
    vhsdecode_gb300_cancel_callback cancel_callback;
    void* user_data;
    uint32_t tape_format;       /* vhsdecode_gb300_tape_format */
    uint32_t decode_flags;      /* 0 or VHSDECODE_GB300_DECODE_CHROMA */
} vhsdecode_gb300_config_v2;

/* vhsdecode_cuda_fast_result_v1 (:100-106). */
typedef struct vhsdecode_gb300_result_v1 {
    uint32_t struct_size;
    uint32_t fields_written;
    uint32_t output_line_length;
    uint32_t output_field_lines;
    double elapsed_seconds;
} vhsdecode_gb300_result_v1;

/* Session: one device-resident decode context. */
typedef struct vhsdecode_gb300_session vhsdecode_gb300_session;

typedef struct vhsdecode_gb300_session_config_v1 {
    uint32_t struct_size;
    uint32_t profile;
    uint32_t tape_speed;
    int32_t device_id;
    double sample_rate_mhz;
    uint64_t max_samples;       /* capacity of one capture / window */
    uint32_t precision;         /* vhsdecode_gb300_precision */
    uint32_t max_fields;        /* 0 = derived from max_samples */
    uint32_t tape_format;       /* vhsdecode_gb300_tape_format */
    uint32_t decimation;        /* 0 or 1: none.  2: decode's samples are at twice
                                   sample_rate_mhz and pass the device 2:1 half-band
                                   decimator first (config_v1.device_decimation_factor);
                                   max_samples counts them */
} vhsdecode_gb300_session_config_v1;

/* flags for vhsdecode_gb300_session_decode */
#define VHSDECODE_GB300_DECODE_DEVICE_INPUT 0x1u /* rf is a device pointer (16-byte aligned) */
#define VHSDECODE_GB300_DECODE_DEMOD_ONLY   0x2u /* stop after the block demodulator */
#define VHSDECODE_GB300_DECODE_FLOAT_INPUT  0x4u /* rf holds float samples (input format FLOAT32) */
#define VHSDECODE_GB300_DECODE_CHROMA       0x8u /* colour-under chroma as the reference's default
                                                    decode does it: the burst phase refines the line
                                                    locations (so the luma moves too) and each field
                                                    gets a uint16 chroma field (session_copy_chroma);
                                                    without it the decode is the reference's
                                                    --skip_chroma one */

typedef struct vhsdecode_gb300_decode_result_v1 {
    uint32_t struct_size;
    uint32_t fields;            /* fields decoded (TBC rendered) */
    uint32_t output_line_length;
    uint32_t output_field_lines;
    uint64_t blocks;            /* 32768-sample blocks demodulated */
    uint64_t stream_samples;    /* stitched stream length = blocks * 30720 */
    uint32_t repaired_blocks;   /* blocks that took the diff-demod spike repair */
    uint32_t stop_reason;       /* 0 end of data, 1 max fields (failed fields are skipped past) */
    double device_ms;           /* stream time of the whole decode */
    double demod_ms;            /* block demodulator kernel time */
    double field_ms;            /* pulses + hsync + TBC + dropout kernels */
    double host_ms;             /* host control plane */
    uint32_t kernel_launches;   /* device kernels this decode launched */
    uint32_t segments;          /* pipeline segments of the demod (1 for the plain path) */
    uint32_t fft_plan;          /* radix plans the fused demodulator used (tuned per device) */
    uint32_t reserved;
} vhsdecode_gb300_decode_result_v1;

typedef struct vhsdecode_gb300_field_info_v1 {
    uint32_t struct_size;
    int32_t is_first_field;
    int64_t span_start;         /* stitched-stream index of the field span */
    int64_t file_loc;           /* RF sample index of line 0 */
    double line0;               /* span-relative */
    double first_hsync;
    double mean_line_length;
    double next_field_offset;
    uint32_t line_count;        /* line locations available */
    uint32_t dropout_count;
} vhsdecode_gb300_field_info_v1;

/* ---- reference-shaped entry points ---------------------------------- */

/* vhsdecode_cuda_fast_get_abi_version (:145-146) */
VHSDECODE_GB300_API uint32_t VHSDECODE_GB300_CALL vhsdecode_gb300_get_abi_version(void);

/* vhsdecode_cuda_fast_get_runtime_info (:148-151) */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_get_runtime_info(
    int32_t device_id, vhsdecode_gb300_runtime_info_v1* info);

/* vhsdecode_cuda_fast_run (:153-156): whole-run handoff.  Pulls int16 RF through
 * read_callback, decodes every field and writes <base>.tbc (uint16 LE luma,
 * outlinelen x (frame_lines/2+1) per field) and <base>.tbc.json.  `config`
 * may point to a vhsdecode_gb300_config_v2 (struct_size tells). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_run(
    const vhsdecode_gb300_config_v1* config, vhsdecode_gb300_result_v1* result);

/* vhsdecode_cuda_fast_get_last_error (:173-174), thread-local message. */
VHSDECODE_GB300_API const char* VHSDECODE_GB300_CALL vhsdecode_gb300_get_last_error(void);

/* ---- session API ------------------------------------------------------ */

/* Replaces the preview context of vhsdecode_cuda_fast_preview_create (:158-161):
 * a persistent device context for repeated windows. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_create(
    const vhsdecode_gb300_session_config_v1* config, vhsdecode_gb300_session** session);

/* vhsdecode_cuda_fast_preview_destroy (:169-171) */
VHSDECODE_GB300_API void VHSDECODE_GB300_CALL vhsdecode_gb300_session_destroy(
    vhsdecode_gb300_session* session);

/* Use this CUDA stream (cudaStream_t as void*) for all device work; NULL = the
 * session's own stream. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_set_stream(
    vhsdecode_gb300_session* session, void* cuda_stream);

/* Decode one capture/window (counterpart of
 * vhsdecode_cuda_fast_preview_decode_window, :292-295).  rf holds int16
 * samples, or float ones with VHSDECODE_GB300_DECODE_FLOAT_INPUT. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_decode(
    vhsdecode_gb300_session* session, const void* rf, uint64_t sample_count,
    uint32_t max_fields, uint32_t flags, vhsdecode_gb300_decode_result_v1* result);

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_get_field(
    vhsdecode_gb300_session* session, uint32_t index, vhsdecode_gb300_field_info_v1* info);

/* Copy `count` fields of uint16 TBC luma starting at `first` to host memory. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_tbc(
    vhsdecode_gb300_session* session, uint32_t first, uint32_t count, uint16_t* destination);

/* Copy `count` fields of uint16 chroma (the _chroma.tbc payload) starting at
 * `first`; the last decode must have asked for VHSDECODE_GB300_DECODE_CHROMA. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_chroma(
    vhsdecode_gb300_session* session, uint32_t first, uint32_t count, uint16_t* destination);

/* Chroma stages of one field of the last chroma decode, as double (tests):
 * 0 chroma TBC of the output lines, 1 the up-converted chroma after the final
 * band-pass (field samples each), 2 the line-1 chroma TBC at the burst-probe
 * windows (lines x window), 3 the kept burst sequence (lines x phase, offset,
 * magnitude, I, Q, then its rotation index), 4 the phase averages (all, even,
 * odd, mean magnitude), 5 the hsync-refined line locations the burst
 * refinement started from.  *count receives the values written. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_chroma_stage(
    vhsdecode_gb300_session* session, uint32_t field, uint32_t stage, double* destination, uint64_t capacity,
    uint64_t* count);

/* Refined line locations of one field (span-relative samples). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_lines(
    vhsdecode_gb300_session* session, uint32_t field, double* destination, uint32_t capacity);

/* Dropouts of one field mapped to TBC coordinates (field line, start x, end x). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_dropouts(
    vhsdecode_gb300_session* session, uint32_t field, int32_t* line, int32_t* start_x,
    int32_t* end_x, uint32_t capacity, uint32_t* count);

/* Stitched stream channel (0 video Hz, 1 sync reference Hz, 2 envelope, 3 chroma
 * after a VHSDECODE_GB300_DECODE_CHROMA decode) as double. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_copy_stream(
    vhsdecode_gb300_session* session, uint32_t channel, uint64_t start, uint64_t count,
    double* destination);

/* Device pointer of the uint16 TBC buffer (fields x lines x outlinelen). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_session_tbc_device(
    vhsdecode_gb300_session* session, void** device_pointer, uint64_t* bytes);

/* ---- stage-level entry points (tests) ------------------------------ */

/* Filter spectra (bins 0..16384) for a format at a sample rate; host only.
 * video / sync / sub_high are interleaved (re, im); sub_high (may be NULL)
 * receives Video x the sub-deemphasis high-pass, zeros for formats without
 * sub-deemphasis.  env receives the envelope low-pass b0, b1, a1 and, from
 * env[3], the sub-deemphasis amplitude low-pass b0, b1, a1 (zeros without). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_design_filters(
    uint32_t profile, uint32_t tape_speed, uint32_t tape_format, double sample_rate_mhz,
    double* rf_video, double* video, double* sync, double* sub_high, double* env);

/* Chroma filters and tables for a format at a sample rate; host only.
 * rf_sos / final_sos receive 4 x 6 section coefficients (b0 b1 b2 a0 a1 a2) of
 * the RF chroma band-pass and the final / burst-probe band-pass (the
 * reference's IirFilterDesign.ButterworthBandPassSos designs); geometry gets
 * burst start, burst end (output samples), chroma offset roll, RF and final
 * pad lengths, the two chroma_rotation values and the field sample count.
 * heterodyne (4 x field), burst_sin and burst_cos (field) may be NULL. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_design_chroma(
    uint32_t profile, uint32_t tape_speed, uint32_t tape_format, double sample_rate_mhz, double* rf_sos,
    double* final_sos, int32_t* geometry, float* heterodyne, float* burst_sin, float* burst_cos);

/* Host control plane on given raw pulses of one span; host only.
 * state[0] = previous first-field flag (-1 unknown), state[1] = has previous
 * hsync; updated in place.  out[0..4] = first_field, line0, first_hsync,
 * mean line length, next field offset.  locs receives the unrefined line
 * locations.  ref (optional, span_len doubles) feeds the long-hsync rescue. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_field_sync(
    uint32_t profile, double sample_rate_mhz, const int64_t* starts, const int64_t* lengths,
    uint64_t pulse_count, int64_t span_len, const double* ref, int32_t* state, double* out,
    double* locs, uint32_t locs_capacity, uint32_t* locs_count);

/* Device sinc TBC of `source` (double) through the linear line-location plan;
 * output values are float32-rounded, as the reference's ResampleLines. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_tbc_resample_lines(
    const double* source, uint64_t source_length, const double* locations,
    uint32_t location_count, uint32_t first_line, uint32_t line_count,
    uint32_t output_line_length, double nominal_line_length, double level_smoothing,
    double* destination);

/* Device pulse detection over one array (PulseDetection.FindPulses semantics). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_find_pulses(
    const double* reference, uint64_t length, double high, int64_t minimum_length,
    int64_t maximum_length, int64_t* starts, int64_t* lengths, uint64_t capacity,
    uint64_t* count);

/* Device FM demodulation of n float pairs (PortedMath.UnwrapHilbertVhsRustApproximation,
 * Core/Dsp/PortedMath.cs:70-230, 519-551): out[0] = 0, out[i] = wrapped angle
 * difference of samples i and i-1 scaled to Hz at sample_rate_hz. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_vhs_demod(
    const float* real, const float* imaginary, uint64_t n, double sample_rate_hz, float* out);

/* Device ReplaceSpikes (RfDemodulator.ReplaceSpikes, Core/Dsp/RfDemodulator.cs:966-1001)
 * in the block demodulator's parallel form, in place on `demod` (n a multiple of
 * 32, at most 2^20): windows [i-8, i+30) around demod > max_value take `diffed`
 * where max(diffed) < max(demod). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_replace_spikes(
    float* demod, const float* diffed, uint64_t n, float max_value);

/* Device polynomial atan2 (the FM demodulator's angle) for n float pairs. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_vhs_angles(
    const float* real, const float* imaginary, uint64_t n, float* angles);

/* Device 2:1 decimation of a whole host capture (cuda_fast_read_upload_half_rate,
 * src/VHSDecode.CudaFast.Native/include/cuda_fast_decimator.h:27-36, over one
 * window covering the capture): source_count int16 (input_sample_format 1) or
 * float (0) samples in, source_count / 2 float samples out, sample i the
 * half-band FIR centred on source sample 2 i with zeros outside the capture. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_decimate_half_rate(
    const void* source, uint32_t input_sample_format, uint64_t source_count, float* destination);

/* ---------------------------------------------------------------- serving
 * Window server: continuous batching of decode windows from many client
 * streams on one GPU.  Replaces the single-window preview context of
 * vhsdecode_cuda_fast_preview_create / _decode_window (:158-171), which
 * serialises windows behind a mutex: here `workers` windows decode at once,
 * each on a device slot of its format, admitted while the slots' device
 * memory stays inside the budget.  Windows of one stream_id decode in
 * submission order and carry the stream's sync history (field parity, hsync
 * history, next-field continuation) unless `seek` is set.  `samples` and
 * `tbc_out` must stay valid until the window's result has been returned by
 * vhsdecode_gb300_server_wait. */
typedef struct vhsdecode_gb300_server vhsdecode_gb300_server;

typedef struct vhsdecode_gb300_server_config_v1 {
    uint32_t struct_size;
    int32_t device_id;
    uint32_t workers;               /* windows decoded at once (0 = 4) */
    uint32_t max_batch;             /* 0 or 1: each window has its own launches; n > 1: a free
                                       worker takes up to n waiting windows (any streams and
                                       formats, not decimated) and demodulates all their blocks
                                       in one persistent launch */
    uint64_t max_window_samples;    /* longest window accepted; sizes every slot */
    uint64_t memory_budget_bytes;   /* device memory for slots (0 = 80 % of free memory) */
} vhsdecode_gb300_server_config_v1;

typedef struct vhsdecode_gb300_window_v1 {
    uint32_t struct_size;
    uint32_t stream_id;             /* client stream; its windows decode in order */
    uint32_t profile;               /* vhsdecode_gb300_profile */
    uint32_t tape_speed;
    double sample_rate_mhz;
    const int16_t* samples;         /* host RF samples of the window */
    uint64_t sample_count;
    uint64_t source_offset;         /* stream position of samples[0] */
    uint32_t seek;                  /* 1: discontinuity, start without the stream's history */
    uint32_t max_fields;            /* 0 = as many as fit */
    uint16_t* tbc_out;              /* host destination for the fields' TBC, or NULL */
    uint64_t tbc_capacity;          /* uint16 elements at tbc_out */
    uint32_t tape_format;           /* vhsdecode_gb300_tape_format */
    uint32_t decimation;            /* 0 or 1: none; 2: samples run at twice sample_rate_mhz and
                                       pass the device 2:1 decimator (the reference preview's
                                       40 -> 20 MSPS mode); counts and offsets stay source samples */
} vhsdecode_gb300_window_v1;

typedef struct vhsdecode_gb300_window_result_v1 {
    uint32_t struct_size;
    int32_t status;                 /* vhsdecode_gb300_status of this window */
    uint32_t stream_id;
    uint32_t fields;
    uint32_t first_field_is_first;  /* parity of the window's first field */
    uint32_t continued;             /* 1 when the stream's sync history was used */
    uint64_t ticket;
    uint64_t sample_count;
    uint64_t next_source_offset;    /* a window starting at or before this continues the stream;
                                       starting exactly here (on the stream's 983040-sample grid)
                                       reproduces a whole-stream decode bit for bit */
    double queue_ms;                /* submit to start of decode */
    double decode_ms;
    double latency_ms;              /* submit to result */
    uint32_t batched;               /* windows in the launch that demodulated this one */
    uint32_t reserved;
} vhsdecode_gb300_window_result_v1;

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_server_create(
    const vhsdecode_gb300_server_config_v1* config, vhsdecode_gb300_server** server);
/* Queues a window; returns at once with its ticket. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_server_submit(
    vhsdecode_gb300_server* server, const vhsdecode_gb300_window_v1* window, uint64_t* ticket);
/* Blocks until the window is done; returns its status (result->status). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_server_wait(
    vhsdecode_gb300_server* server, uint64_t ticket, vhsdecode_gb300_window_result_v1* result);
/* Finishes the windows being decoded, cancels queued ones, frees the slots. */
VHSDECODE_GB300_API void VHSDECODE_GB300_CALL vhsdecode_gb300_server_destroy(vhsdecode_gb300_server* server);

/* STREAMINFO of a FLAC stream (Core/Rf/RawFlacStreamInfo.cs; the reference's
 * loader accepts a stream only when it starts with "fLaC" and a 34-byte
 * STREAMINFO block, LibsndfilePcm16SampleLoaderTests.cs:1038-1110). */
typedef struct vhsdecode_gb300_flac_info_v1 {
    uint32_t struct_size;
    uint32_t sample_rate;
    uint32_t channels;
    uint32_t bits_per_sample;
    uint32_t min_block;
    uint32_t max_block;
    uint64_t total_samples;
    uint64_t first_frame_offset;   /* bytes */
} vhsdecode_gb300_flac_info_v1;

/* Parses the STREAMINFO of `bytes` bytes of FLAC (host only, no GPU). */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_flac_info(
    const uint8_t* data, uint64_t bytes, vhsdecode_gb300_flac_info_v1* info);

/* Decodes a whole FLAC stream of 16-bit mono samples held in host memory on
 * device `device_id` (frames found and decoded in parallel, each checked
 * against its CRC-16); copies up to `capacity` samples to `out` and returns
 * the stream's sample count in *samples.  Replaces the libsndfile / ffmpeg
 * .ldf loaders (Core/Rf/LibsndfilePcm16SampleLoader.cs,
 * Core/Rf/FfmpegPcm16SampleLoader.cs).  INPUT_ERROR for a corrupt stream. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_flac_decode(
    const uint8_t* data, uint64_t bytes, int16_t* out, uint64_t capacity, uint64_t* samples,
    int32_t device_id);

/* Sync-pulse edge events over `length` float samples already on the device,
 * with no device memory allocated by the call.  No counterpart in the
 * reference: it serves callers that may not allocate while decoding (a thread
 * capturing CUDA graphs, a real-time loop, a fixed memory budget).
 * events[i] = 2 * position + (0 for a pulse start, 1 for a pulse end), in
 * order; *total receives the full count (entries past `capacity` are not
 * written).  `stream` is a cudaStream_t (NULL = legacy default stream).
 * Limit: length <= 16777216 samples, else INVALID_ARGUMENT.  The first call on
 * a device sets up its fixed scratch: make it before capturing a stream.
 * Every call outside a stream capture looks the scratch address up again, so
 * a context recreated after cudaDeviceReset is followed.
 * Calls on one device share that scratch and must not overlap. */
VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_pulse_events_noalloc(
    const float* sync, int64_t length, double high, int64_t* events, int64_t capacity,
    int64_t* total, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VHSDECODE_GB300_H */
