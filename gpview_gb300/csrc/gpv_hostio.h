// gpv_hostio.h -- host threads of the packed Level2 output (gpv_hostio.cpp).
#pragma once
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <thread>
#include <vector>

namespace gpv {

// 2-bit Level2 codes (16 cells per word, cell k at bits 2k: 0 outside, 1 inside, 2 boundary)
// -> the reference's state bytes 0, 127, 254 (words * 16 bytes).
void expand_codes(const uint32_t *codes, uint8_t *out, size_t words);

// A fixed set of host threads that expand one range of codes at a time; run() blocks until
// the range is done, with the calling thread working too.
class ExpandPool {
 public:
  explicit ExpandPool(int threads);
  ~ExpandPool();
  ExpandPool(const ExpandPool &) = delete;
  ExpandPool &operator=(const ExpandPool &) = delete;
  void run(const uint32_t *codes, uint8_t *out, size_t words);
  int threads() const { return (int)th_.size() + 1; }

 private:
  static constexpr size_t kChunkWords = size_t(1) << 16;  // 1 MiB of output per chunk
  void worker();
  size_t drain();
  std::mutex mu_;
  std::condition_variable cv_, cv_done_;
  std::vector<std::thread> th_;
  const uint32_t *src_ = nullptr;
  uint8_t *dst_ = nullptr;
  size_t words_ = 0, chunks_ = 0, finished_ = 0;
  std::atomic<size_t> next_{0};
  uint64_t gen_ = 0;
  bool stop_ = false;
};

}  // namespace gpv
