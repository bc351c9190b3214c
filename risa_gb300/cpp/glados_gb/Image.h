// Pooled frame buffers, the unit that flows between stages.
//
// Mirrors the reference's glados::Image (glados/Image.h:41-211) and
// glados::MemoryPool (glados/MemoryPool.h:53-138): an Image owns one buffer
// of a memory manager's kind (device or pinned host), carries index / plane /
// device / start-time metadata, is move-only in practice, and returns its
// buffer to the pool it came from when it is destroyed. A default-constructed
// Image is invalid and acts as the end-of-stream sentinel.
#pragma once

#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

namespace glados_gb {

inline void check_cuda(cudaError_t e, const char* what) {
   if (e != cudaSuccess)
      throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Device memory (cudaMalloc), owned through a unique_ptr with cudaFree.
template <class T>
struct DeviceMemoryManager {
   using value_type = T;
   struct Deleter {
      void operator()(T* p) const { if (p) cudaFree(p); }
   };
   using pointer_type = std::unique_ptr<T, Deleter>;
   static pointer_type make_ptr(std::size_t n) {
      T* p = nullptr;
      check_cuda(cudaMalloc(&p, sizeof(T) * n), "cudaMalloc");
      return pointer_type(p);
   }
   static constexpr bool on_device = true;
};

// Page-locked host memory (cudaMallocHost), for the H2D / D2H boundary.
template <class T>
struct HostMemoryManager {
   using value_type = T;
   struct Deleter {
      void operator()(T* p) const { if (p) cudaFreeHost(p); }
   };
   using pointer_type = std::unique_ptr<T, Deleter>;
   static pointer_type make_ptr(std::size_t n) {
      T* p = nullptr;
      check_cuda(cudaMallocHost(&p, sizeof(T) * n), "cudaMallocHost");
      return pointer_type(p);
   }
   static constexpr bool on_device = false;
};

template <class M>
class MemoryPool;

template <class M>
class Image {
 public:
   using value_type = typename M::value_type;
   using pointer_type = typename M::pointer_type;
   using clock = std::chrono::high_resolution_clock;

   Image() noexcept = default;  // invalid: the end-of-stream sentinel
   Image(std::size_t size, pointer_type data, unsigned pool_index)
       : size_{size}, data_{std::move(data)}, pool_index_{pool_index}, valid_{true} {}

   Image(Image&& o) noexcept { *this = std::move(o); }
   Image& operator=(Image&& o) noexcept {
      if (this != &o) {
         release();
         size_ = o.size_;
         index_ = o.index_;
         plane_ = o.plane_;
         device_ = o.device_;
         data_ = std::move(o.data_);
         pool_index_ = o.pool_index_;
         start_ = o.start_;
         valid_ = o.valid_;
         o.valid_ = false;
      }
      return *this;
   }
   Image(const Image&) = delete;
   Image& operator=(const Image&) = delete;
   ~Image() { release(); }

   bool valid() const noexcept { return valid_; }
   std::size_t size() const noexcept { return size_; }
   std::size_t index() const noexcept { return index_; }
   std::size_t plane() const noexcept { return plane_; }
   int device() const noexcept { return device_; }
   unsigned memoryPoolIndex() const noexcept { return pool_index_; }
   clock::time_point start() const noexcept { return start_; }
   value_type* data() const noexcept { return data_.get(); }
   const pointer_type& container() const noexcept { return data_; }

   void setIdx(std::size_t i) { index_ = i; }
   void setPlane(std::size_t p) { plane_ = p; }
   void setDevice(int d) { device_ = d; }
   void setStart(clock::time_point t) { start_ = t; }
   void setMemPoolIdx(unsigned i) { pool_index_ = i; }
   // milliseconds since the frame entered the pipeline (Image.h:97-99)
   double duration() const {
      return std::chrono::duration<double, std::milli>(clock::now() - start_).count();
   }
   // Detach from the pool (used when a pool is torn down).
   void invalidate() { valid_ = false; }

 private:
   void release();

   std::size_t size_ = 0, index_ = 0, plane_ = 0;
   int device_ = 0;
   pointer_type data_{};
   unsigned pool_index_ = 0;
   clock::time_point start_{};
   bool valid_ = false;
};

// One pool per memory-manager type; each registered stage gets its own list
// of pre-allocated buffers. requestMemory blocks until a buffer is free
// (MemoryPool.h:68-79), which is the pipeline's back-pressure.
template <class M>
class MemoryPool {
 public:
   using image_type = Image<M>;

   static MemoryPool* instance() {
      static MemoryPool pool;
      return &pool;
   }

   unsigned registerStage(int count, std::size_t elements) {
      std::lock_guard<std::mutex> lock{mutex_};
      const unsigned idx = (unsigned)pools_.size();
      std::vector<image_type> list;
      list.reserve(count);
      for (int i = 0; i < count; ++i) list.emplace_back(elements, M::make_ptr(elements), idx);
      pools_.push_back(std::move(list));
      return idx;
   }

   image_type requestMemory(unsigned idx) {
      std::unique_lock<std::mutex> lock{mutex_};
      if (idx >= pools_.size()) throw std::runtime_error("MemoryPool: stage is not registered");
      cv_.wait(lock, [&] { return !pools_[idx].empty(); });
      image_type ret = std::move(pools_[idx].back());
      pools_[idx].pop_back();
      return ret;
   }

   void returnMemory(image_type&& img) {
      std::lock_guard<std::mutex> lock{mutex_};
      const unsigned idx = img.memoryPoolIndex();
      if (idx >= pools_.size()) throw std::runtime_error("MemoryPool: stage is not registered");
      if (closed_.size() > idx && closed_[idx]) {
         img.invalidate();  // the stage is gone: let the buffer be freed
         return;
      }
      pools_[idx].push_back(std::move(img));
      cv_.notify_all();
   }

   // Frees the buffers currently in the pool; buffers still in flight are
   // freed when they come back (MemoryPool.h:128-133).
   void freeMemory(unsigned idx) {
      std::vector<image_type> dying;
      {
         std::lock_guard<std::mutex> lock{mutex_};
         if (idx >= pools_.size()) return;
         if (closed_.size() <= idx) closed_.resize(idx + 1, false);
         closed_[idx] = true;
         dying.swap(pools_[idx]);
      }
      for (auto& im : dying) im.invalidate();
   }

   std::size_t available(unsigned idx) {
      std::lock_guard<std::mutex> lock{mutex_};
      return idx < pools_.size() ? pools_[idx].size() : 0;
   }

 private:
   MemoryPool() = default;
   ~MemoryPool() {
      // buffers still pooled at exit are freed without being returned
      for (auto& list : pools_)
         for (auto& im : list) im.invalidate();
   }
   std::vector<std::vector<image_type>> pools_;
   std::vector<bool> closed_;
   std::mutex mutex_;
   std::condition_variable cv_;
};

template <class M>
void Image<M>::release() {
   if (valid_) {
      valid_ = false;
      Image tmp;
      tmp.size_ = size_;
      tmp.data_ = std::move(data_);
      tmp.pool_index_ = pool_index_;
      tmp.valid_ = true;
      MemoryPool<M>::instance()->returnMemory(std::move(tmp));
   }
}

}  // namespace glados_gb
