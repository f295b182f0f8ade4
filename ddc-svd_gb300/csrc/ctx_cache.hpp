// ctx_cache.hpp -- a small table of values kept per CUDA context.
//
// The key is the context's unique id (cuCtxGetId), not the CUcontext handle:
// a handle value can be reused after a context is destroyed (for example
// after cudaDeviceReset) and then names a different context, while an id is
// never reused within a process.  A value therefore can never be served to
// a context other than the one it was made in.  Host-only C++ (no CUDA
// types), so the logic is also checked on a machine without a GPU.
#pragma once

#include <mutex>

namespace ddcsvd {

template <int Slots>
class CtxValueCache {
 public:
  // The value cached for `ctx_id`; on a miss `make(void** value)` (returning
  // 0 on success, else a status that is passed through and nothing cached)
  // produces it.  When the table is full the oldest entry makes room.
  template <class Make>
  int get(unsigned long long ctx_id, void** out, Make make) {
    std::lock_guard<std::mutex> g(mu_);
    for (int i = 0; i < used_; i++) {
      if (id_[i] == ctx_id) {
        *out = val_[i];
        return 0;
      }
    }
    void* v = nullptr;
    const int rc = make(&v);
    if (rc != 0) return rc;
    int slot = used_;
    if (used_ < Slots) {
      used_++;
    } else {
      slot = next_;
      next_ = (next_ + 1) % Slots;
    }
    id_[slot] = ctx_id;
    val_[slot] = v;
    *out = v;
    return 0;
  }

  int size() {
    std::lock_guard<std::mutex> g(mu_);
    return used_;
  }

 private:
  std::mutex mu_;
  unsigned long long id_[Slots] = {};
  void* val_[Slots] = {};
  int used_ = 0, next_ = 0;
};

}  // namespace ddcsvd
