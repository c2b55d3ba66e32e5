// Device FLAC decoding of 16-bit mono RF captures: shared types (flac.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <vector>

namespace vhsd {

struct FlacInfo {
    uint32_t sample_rate, channels, bits_per_sample, min_block, max_block;
    uint64_t total_samples;
    uint64_t first_frame;   // byte offset of the first frame
};

struct FlacFrame {
    int64_t off, end;       // byte range of the frame in the chunk (end: next frame)
    int64_t sample0;        // first output sample, relative to the chunk's first
    int32_t header_len, block;
};

// STREAMINFO and the offset of the first frame; an error status if the stream
// does not start with "fLaC" and a 34-byte STREAMINFO.
int32_t flac_stream_info(const uint8_t* p, uint64_t n, FlacInfo& info);

// Decodes a FLAC stream chunk by chunk: each chunk starts on a frame; all
// frames but the last are decoded (the last too when at_eof), their samples
// appended to `out`; returns the bytes consumed (the caller keeps the rest and
// puts it in front of the next chunk).  Throws Failure(INPUT_ERROR) on a
// corrupt stream.
class FlacStreamDecoder {
public:
    ~FlacStreamDecoder();
    void init(int device);
    size_t decode(const uint8_t* p, size_t n, bool at_eof, std::vector<int16_t>& out);
    // the same, with the chunk's samples copied to dest(count) (null: not copied)
    size_t decode_to(const uint8_t* p, size_t n, bool at_eof, const std::function<int16_t*(size_t)>& dest);
    // starts a new stream (the next chunk begins with its first frame)
    void reset() { next_frame = next_sample = sample_base = decoded_frames = 0; }
    uint64_t decoded_frames = 0;

private:
    void reserve(size_t bytes, size_t samples, size_t frames);
    cudaStream_t stream = nullptr;
    uint8_t* d_bytes = nullptr;
    int64_t* d_cand = nullptr;
    FlacFrame* d_frames = nullptr;
    int* d_work = nullptr;      // frame order of the decode launch
    int16_t* d_out = nullptr;
    int* d_misc = nullptr;
    size_t cap_bytes = 0, cap_cand = 0, cap_frames = 0, cap_work = 0, cap_out = 0;
    uint64_t next_frame = 0, next_sample = 0, sample_base = 0;
};

}  // namespace vhsd
