// VDIF depacketiser: frames of one antenna's VDIF stream (device memory) to
// the engine's contiguous packed input buffer, plus per-frame validity.
//
// Header (VDIF standard, little-endian 32-bit words; fields as the reference's
// examples/mark/dump_vdif.py:40-55 decodes them):
//   w0: bit 31 invalid, bit 30 legacy (16-byte header; else 32 bytes), bits 0-29 seconds from epoch
//   w1: bits 24-29 reference epoch (half-years from 2000), bits 0-23 frame number within the second
//   w2: bits 29-31 version, bits 24-28 log2(channels), bits 0-23 frame length in 8-byte units
//   w3: bit 31 complex, bits 26-30 bits per sample - 1, bits 16-25 thread id, bits 0-15 station id
// The reference's ingest (ingest/src/ingest.c:267-330) places each frame at
// (seconds - seconds0) * frames_per_second + frame - frame0 within a ring-buffer
// block; the same placement is done here on the GPU, one CTA per frame.
//
// Two-channel VDIF payloads are already the engine's input layout: 2-bit
// samples packed LSB first with the channels interleaved per time sample
// (offset-binary codes 0..3 = the levels -3.3359, -1, +1, +3.3359 of
// fxkernel/src/fxkernel.cpp:15-28), and 8-bit complex samples as
// ch0.re ch0.im ch1.re ch1.im; VDIF 8-bit samples are offset binary, so they
// are converted to two's-complement int8 (XOR 0x80) on the way.
#include <stdint.h>

#include "gxc_internal.h"

namespace {

__device__ __forceinline__ uint32_t le32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

struct VdifArgs {
  const uint8_t *frames;
  long long nframes;
  int frame_bytes, payload_bytes;
  long long seconds0;
  int frame0, fps, thread_id, xor80;
  uint8_t *out;
  long long nslots;
  uint8_t *valid;
  unsigned long long *stats;  // [accepted, outside window or other thread, malformed or invalid]
  int vec;                    // 1: 16-byte copies are aligned
};

__global__ void vdif_depacketize_kernel(const VdifArgs a) {
  __shared__ long long s_slot;
  __shared__ int s_hdr;
  const long long f = blockIdx.x;
  const uint8_t *fr = a.frames + f * (long long)a.frame_bytes;
  if (threadIdx.x == 0) {
    const uint32_t w0 = le32(fr), w1 = le32(fr + 4), w2 = le32(fr + 8), w3 = le32(fr + 12);
    const int invalid = (int)(w0 >> 31), legacy = (int)((w0 >> 30) & 1u);
    const long long sec = (long long)(w0 & 0x3fffffffu);
    const int frame = (int)(w1 & 0x00ffffffu);
    const int len = (int)(w2 & 0x00ffffffu) * 8;
    const int thread = (int)((w3 >> 16) & 0x3ffu);
    const int hdr = legacy ? 16 : 32;
    long long slot = -1;
    int why = 2;
    if (!invalid && len == a.frame_bytes && a.frame_bytes - hdr == a.payload_bytes && frame < a.fps) {
      why = 1;
      if (a.thread_id < 0 || thread == a.thread_id) {
        const long long s = (sec - a.seconds0) * a.fps + frame - a.frame0;
        if (s >= 0 && s < a.nslots) {
          slot = s;
          why = 0;
        }
      }
    }
    if (a.stats) atomicAdd(a.stats + why, 1ull);
    s_slot = slot;
    s_hdr = hdr;
  }
  __syncthreads();
  const long long slot = s_slot;
  if (slot < 0) return;
  const uint8_t *src = fr + s_hdr;
  uint8_t *dst = a.out + slot * (long long)a.payload_bytes;
  if (a.vec) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    const uint32_t x = a.xor80 ? 0x80808080u : 0u;
    for (int i = threadIdx.x; i < a.payload_bytes / 16; i += blockDim.x) {
      uint4 v = s4[i];
      v.x ^= x;
      v.y ^= x;
      v.z ^= x;
      v.w ^= x;
      d4[i] = v;
    }
  } else {
    const uint8_t x = a.xor80 ? 0x80 : 0;
    for (int i = threadIdx.x; i < a.payload_bytes; i += blockDim.x) dst[i] = src[i] ^ x;
  }
  if (threadIdx.x == 0) a.valid[slot] = 1;
}

__global__ void vdif_fill_kernel(uint8_t *out, const uint8_t *valid, long long nslots, int payload_bytes,
                                 uint8_t fill) {
  const long long slot = blockIdx.x;
  if (slot >= nslots || valid[slot]) return;
  uint8_t *dst = out + slot * (long long)payload_bytes;
  for (int i = threadIdx.x; i < payload_bytes; i += blockDim.x) dst[i] = fill;
}

}  // namespace

extern "C" {

gxc_status gxc_vdif_parse_header(const uint8_t *h, gxc_vdif_header *out) {
  if (!h || !out) return GXC_ERR_INVALID_ARGUMENT;
  auto w = [&](int i) {
    return (uint32_t)h[4 * i] | ((uint32_t)h[4 * i + 1] << 8) | ((uint32_t)h[4 * i + 2] << 16) |
           ((uint32_t)h[4 * i + 3] << 24);
  };
  const uint32_t w0 = w(0), w1 = w(1), w2 = w(2), w3 = w(3);
  out->invalid = (int)(w0 >> 31);
  out->legacy = (int)((w0 >> 30) & 1u);
  out->seconds = (int64_t)(w0 & 0x3fffffffu);
  out->ref_epoch = (int)((w1 >> 24) & 0x3fu);
  out->frame = (int)(w1 & 0x00ffffffu);
  out->version = (int)(w2 >> 29);
  out->nchan = 1 << ((w2 >> 24) & 0x1fu);
  out->frame_bytes = (int)(w2 & 0x00ffffffu) * 8;
  out->is_complex = (int)(w3 >> 31);
  out->bits = (int)((w3 >> 26) & 0x1fu) + 1;
  out->thread = (int)((w3 >> 16) & 0x3ffu);
  out->station = (int)(w3 & 0xffffu);
  out->header_bytes = out->legacy ? 16 : 32;
  return GXC_OK;
}

gxc_status gxc_vdif_depacketize(const uint8_t *frames, size_t nbytes, int frame_bytes, int payload_bytes,
                                int64_t seconds0, int frame0, int frames_per_second, int thread_id,
                                int offset_binary_8bit, uint8_t fill, uint8_t *out, size_t nslots, uint8_t *valid,
                                unsigned long long *stats, void *stream) {
  if (!frames || !out || !valid || frame_bytes < 32 || payload_bytes < 1 || payload_bytes > frame_bytes - 16 ||
      frames_per_second < 1 || frame0 < 0 || nslots < 1)
    return GXC_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const long long nframes = (long long)(nbytes / (size_t)frame_bytes);
  VdifArgs a;
  a.frames = frames;
  a.nframes = nframes;
  a.frame_bytes = frame_bytes;
  a.payload_bytes = payload_bytes;
  a.seconds0 = seconds0;
  a.frame0 = frame0;
  a.fps = frames_per_second;
  a.thread_id = thread_id;
  a.xor80 = offset_binary_8bit ? 1 : 0;
  a.out = out;
  a.nslots = (long long)nslots;
  a.valid = valid;
  a.stats = stats;
  const int hdr = frame_bytes - payload_bytes;
  a.vec = ((uintptr_t)frames % 16 == 0) && ((uintptr_t)out % 16 == 0) && (frame_bytes % 16 == 0) &&
          (payload_bytes % 16 == 0) && (hdr % 16 == 0);
  if (cudaMemsetAsync(valid, 0, nslots, s) != cudaSuccess) return GXC_ERR_CUDA;
  if (nframes > 0) {
    if (nframes > 0x7fffffffLL) return GXC_ERR_INVALID_ARGUMENT;
    vdif_depacketize_kernel<<<(unsigned)nframes, 256, 0, s>>>(a);
    if (cudaGetLastError() != cudaSuccess) return GXC_ERR_CUDA;
  }
  if ((long long)nslots > 0x7fffffffLL) return GXC_ERR_INVALID_ARGUMENT;
  vdif_fill_kernel<<<(unsigned)nslots, 256, 0, s>>>(out, valid, (long long)nslots, payload_bytes, fill);
  return cudaGetLastError() == cudaSuccess ? GXC_OK : GXC_ERR_CUDA;
}

}  // extern "C"
