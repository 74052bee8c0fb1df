// gpv_hostio.cpp -- host side of the packed Level2 output of gpv_voxelize_to_host.
//
// Over the CPU-GPU link (~192 GB/s device to host on a GB300 machine) a Level2 state byte costs as
// much as any other byte, and a 256^3 / 16^3 voxelization produces 1.2 GB of them: the link,
// not the GPU, then sets the host-to-host time.  The Level2 kernel can instead send each state
// as a 2-bit code (16 cells per 32-bit word, cell k at bits 2k: 0 outside, 1 inside,
// 2 boundary) into page-locked staging, a quarter of the bytes; the host threads here turn the
// codes of every finished z slab into the reference's bytes (0, 127, 254) while the GPU computes
// the next slabs.  The bytes are exactly the ones the kernel would have written.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#if defined(__aarch64__) && defined(__ARM_NEON)
#include <arm_neon.h>
#endif

#include "gpv_hostio.h"

namespace gpv {

namespace {

// Codes of 4 cells (one byte) -> their 4 state bytes, little-endian.
struct Lut4 {
  uint32_t v[256];
  Lut4() {
    for (int b = 0; b < 256; ++b) {
      uint32_t r = 0;
      for (int i = 0; i < 4; ++i) {
        const uint32_t c = (b >> (2 * i)) & 3u;
        r |= (c == 1 ? 127u : c == 2 ? 254u : 0u) << (8 * i);
      }
      v[b] = r;
    }
  }
};
const Lut4 kLut4;

void expand_scalar(const uint32_t *codes, uint8_t *out, size_t words) {
  for (size_t w = 0; w < words; ++w) {
    const uint32_t x = codes[w];
    const uint32_t o[4] = {kLut4.v[x & 255u], kLut4.v[(x >> 8) & 255u], kLut4.v[(x >> 16) & 255u],
                           kLut4.v[x >> 24]};
    std::memcpy(out + 16 * w, o, 16);
  }
}

}  // namespace

void expand_codes(const uint32_t *codes, uint8_t *out, size_t words) {
#if defined(__aarch64__) && defined(__ARM_NEON)
  // 16 cells per word: the word's 4 bytes spread over 16 lanes (byte j/4 to lane j), each lane's
  // 2-bit field shifted down, times 127 (codes 0..2 -> 0, 127, 254; no lane overflows)
  static const uint8_t kIdx[16] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3};
  static const int8_t kSh[16] = {0, -2, -4, -6, 0, -2, -4, -6, 0, -2, -4, -6, 0, -2, -4, -6};
  const uint8x16_t idx = vld1q_u8(kIdx);
  const int8x16_t sh = vld1q_s8(kSh);
  const uint8x16_t three = vdupq_n_u8(3), k127 = vdupq_n_u8(127);
  size_t w = 0;
  for (; w + 4 <= words; w += 4) {
    const uint8x16_t b = vreinterpretq_u8_u32(vld1q_u32(codes + w));
    for (int l = 0; l < 4; ++l) {
      const uint8x16_t s = vqtbl1q_u8(b, vaddq_u8(idx, vdupq_n_u8((uint8_t)(4 * l))));
      vst1q_u8(out + 16 * (w + l), vmulq_u8(vandq_u8(vshlq_u8(s, sh), three), k127));
    }
  }
  expand_scalar(codes + w, out + 16 * w, words - w);
#else
  expand_scalar(codes, out, words);
#endif
}

ExpandPool::ExpandPool(int threads) {
  for (int t = 1; t < threads; ++t) th_.emplace_back([this] { worker(); });
}

ExpandPool::~ExpandPool() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  for (std::thread &t : th_) t.join();
}

// Takes chunks of the current range until none is left; returns the number of chunks done.
size_t ExpandPool::drain() {
  size_t done = 0;
  for (;;) {
    const size_t k = next_.fetch_add(1);
    if (k >= chunks_) return done;
    const size_t w0 = k * kChunkWords, w1 = std::min(words_, w0 + kChunkWords);
    expand_codes(src_ + w0, dst_ + 16 * w0, w1 - w0);
    ++done;
  }
}

void ExpandPool::worker() {
  uint64_t seen = 0;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
    }
    const size_t n = drain();
    if (n) {
      std::lock_guard<std::mutex> lk(mu_);
      finished_ += n;
      if (finished_ == chunks_) cv_done_.notify_all();
    }
  }
}

void ExpandPool::run(const uint32_t *codes, uint8_t *out, size_t words) {
  if (!words) return;
  {
    std::lock_guard<std::mutex> lk(mu_);
    src_ = codes;
    dst_ = out;
    words_ = words;
    chunks_ = (words + kChunkWords - 1) / kChunkWords;
    next_.store(0);
    finished_ = 0;
    ++gen_;
  }
  cv_.notify_all();
  const size_t n = drain();  // the caller works too
  std::unique_lock<std::mutex> lk(mu_);
  finished_ += n;
  cv_done_.wait(lk, [&] { return finished_ == chunks_; });
}

}  // namespace gpv
