// Drop-in stages for the reference's reconstruction pipeline.
//
// Each class keeps the reference's stage contract (RISA/risaLib/include/risa/*):
// a constructor taking the path of the libconfig file, process(input_type&&)
// that queues a frame (or, for an invalid frame, drains and forwards the end
// of stream) and wait() -> output_type that hands the next result to the
// following stage. As in the reference, every stage owns one worker thread
// and one CUDA stream per device, pre-allocates its output buffers in a
// MemoryPool, routes a frame by the device it lives on, synchronises the
// stream after each frame and copies index / plane / start time to its
// output. The device work of every stage is one call into the C ABI
// (include/risa_gb300.h).
//
//   reference class                      this header
//   risa::cuda::H2D                      risa_gb::cuda::H2D
//   risa::cuda::Reordering               risa_gb::cuda::Reordering
//   risa::cuda::DetectorInterpolation    risa_gb::cuda::DetectorInterpolation
//   risa::cuda::Attenuation              risa_gb::cuda::Attenuation
//   risa::cuda::Fan2Para                 risa_gb::cuda::Fan2Para
//   risa::cuda::Filter                   risa_gb::cuda::Filter
//   risa::cuda::Backprojection           risa_gb::cuda::Backprojection
//   risa::cuda::Masking                  risa_gb::cuda::Masking
//   risa::cuda::D2H                      risa_gb::cuda::D2H
//   (none)                               risa_gb::cuda::BatchedFBP (whole chain, batched)
#pragma once

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../glados_gb/Image.h"
#include "../glados_gb/Queue.h"
#include "risa_gb300.h"

namespace risa_gb {

// Reads one config file once: geometry, processing options and raw settings.
class Config {
 public:
   explicit Config(const std::string& path) : path_(path) {
      if (risa_gb_config_load(path.c_str(), &geometry, &params) != RISA_GB_OK)
         throw std::runtime_error(std::string("risa_gb: ") + risa_gb_last_error());
   }
   bool has(const std::string& key) const {
      char buf[8];
      const risa_gb_status s = risa_gb_config_lookup(path_.c_str(), key.c_str(), buf, sizeof(buf));
      return s == RISA_GB_OK || s == RISA_GB_EINVAL;  // EINVAL: present, longer than buf
   }
   std::string str(const std::string& key, const std::string& fallback = std::string()) const {
      std::vector<char> buf(1 << 16);
      if (risa_gb_config_lookup(path_.c_str(), key.c_str(), buf.data(), buf.size()) != RISA_GB_OK)
         return fallback;
      return std::string(buf.data());
   }
   long integer(const std::string& key, long fallback) const {
      const std::string s = str(key);
      return s.empty() ? fallback : std::stol(s);
   }
   bool boolean(const std::string& key, bool fallback) const {
      const std::string s = str(key);
      if (s.empty()) return fallback;
      return s == "true" || s == "1";
   }
   const std::string& path() const { return path_; }

   risa_gb_geometry geometry{};
   risa_gb_params params{};

 private:
   std::string path_;
};

inline void check(risa_gb_status s, const char* what) {
   if (s != RISA_GB_OK)
      throw std::runtime_error(std::string("risa_gb ") + what + ": " + risa_gb_last_error());
}

namespace cuda {

using RawHostManager = glados_gb::HostMemoryManager<uint16_t>;
using RawDeviceManager = glados_gb::DeviceMemoryManager<uint16_t>;
using FloatDeviceManager = glados_gb::DeviceMemoryManager<float>;
using FloatHostManager = glados_gb::HostMemoryManager<float>;

// Per-device worker threads, queues and streams shared by every stage.
// Derived classes implement init(dev), step(dev, input) -> output and
// optionally fini(dev); step runs on the device's worker thread.
template <class In, class Out, class Derived>
class DeviceStage {
 public:
   using input_type = glados_gb::Image<In>;
   using output_type = glados_gb::Image<Out>;

   void process(input_type&& img) {
      if (img.valid()) {
         inputs_[img.device()]->push(std::move(img));
         return;
      }
      for (auto& q : inputs_) q.second->push(input_type());
      for (auto& t : workers_) t.join();
      workers_.clear();
      results_.push(output_type());
   }
   output_type wait() { return results_.take(); }

 protected:
   void start(int stream_priority) {
      check_cuda(cudaGetDeviceCount(&devices_), "cudaGetDeviceCount");
      for (int d = 0; d < devices_; ++d) {
         glados_gb::check_cuda(cudaSetDevice(d), "cudaSetDevice");
         cudaStream_t s;
         glados_gb::check_cuda(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, stream_priority),
                               "cudaStreamCreateWithPriority");
         streams_[d] = s;
         inputs_[d].reset(new glados_gb::Queue<input_type>());
         static_cast<Derived*>(this)->init(d);
      }
      for (int d = 0; d < devices_; ++d) workers_.emplace_back(&DeviceStage::worker, this, d);
   }
   void stop() {
      if (!workers_.empty()) {
         for (auto& q : inputs_) q.second->push(input_type());
         for (auto& t : workers_) t.join();
         workers_.clear();
      }
      for (auto& s : streams_) {
         cudaSetDevice(s.first);
         cudaStreamDestroy(s.second);
      }
      streams_.clear();
   }
   static void check_cuda(cudaError_t e, const char* what) { glados_gb::check_cuda(e, what); }
   cudaStream_t stream(int d) { return streams_.at(d); }
   int devices() const { return devices_; }
   void emit(output_type&& out) { results_.push(std::move(out)); }

 private:
   void worker(int d) {
      glados_gb::check_cuda(cudaSetDevice(d), "cudaSetDevice");
      while (true) {
         input_type in = inputs_[d]->take();
         if (!in.valid()) break;
         output_type out = static_cast<Derived*>(this)->step(d, std::move(in));
         if (out.valid()) results_.push(std::move(out));
      }
   }

   int devices_ = 0;
   std::map<int, cudaStream_t> streams_;
   std::map<int, std::unique_ptr<glados_gb::Queue<input_type>>> inputs_;
   glados_gb::Queue<output_type> results_;
   std::vector<std::thread> workers_;
};

template <class Out, class In>
inline void copy_meta(glados_gb::Image<Out>& out, const glados_gb::Image<In>& in, int device) {
   out.setIdx(in.index());
   out.setPlane(in.plane());
   out.setStart(in.start());
   out.setDevice(device);
}

// ---------------------------------------------------------------------------- H2D
// Host raw frames -> device, round-robin over devices (H2D.cu:84-169); counts
// frames lost upstream from gaps in the index sequence and keeps the best /
// worst inter-arrival time.
class H2D : public DeviceStage<RawHostManager, RawDeviceManager, H2D> {
 public:
   explicit H2D(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      elems_ = (size_t)g.n_fan_proj * g.n_fan_det;
      pool_size_ = (int)cfg_.integer("memPoolSize_H2D", 16);
      start(7);
   }
   ~H2D() {
      stop();
      for (auto& p : pools_) glados_gb::MemoryPool<RawDeviceManager>::instance()->freeMemory(p.second);
   }
   void process(input_type&& img) {
      if (img.valid()) {
         const long idx = (long)img.index();
         if (count_ > 0) {
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - last_).count();
            best_ = std::min(best_, dt);
            worst_ = std::max(worst_, dt);
            if (idx > last_index_ + 1) lost_ += idx - last_index_ - 1;
         }
         last_ = std::chrono::steady_clock::now();
         last_index_ = idx;
         ++count_;
         img.setDevice(next_device_);
         next_device_ = (next_device_ + 1) % devices();
      }
      DeviceStage::process(std::move(img));
   }
   long lost() const { return lost_; }
   double best_interarrival() const { return best_; }
   double worst_interarrival() const { return worst_; }

   void init(int d) { pools_[d] = glados_gb::MemoryPool<RawDeviceManager>::instance()->registerStage(pool_size_, elems_); }
   output_type step(int d, input_type&& in) {
      output_type out = glados_gb::MemoryPool<RawDeviceManager>::instance()->requestMemory(pools_[d]);
      check_cuda(cudaMemcpyAsync(out.data(), in.data(), sizeof(uint16_t) * elems_, cudaMemcpyHostToDevice, stream(d)),
                 "H2D copy");
      check_cuda(cudaStreamSynchronize(stream(d)), "H2D sync");
      copy_meta(out, in, d);
      return out;
   }

 private:
   Config cfg_;
   size_t elems_ = 0;
   int pool_size_ = 16;
   std::map<int, unsigned> pools_;
   std::atomic<int> next_device_{0};
   long count_ = 0, lost_ = 0, last_index_ = -1;
   double best_ = std::numeric_limits<double>::max(), worst_ = 0.0;
   std::chrono::steady_clock::time_point last_{};
};

// ---------------------------------------------------------------------------- Reordering
class Reordering : public DeviceStage<RawDeviceManager, RawDeviceManager, Reordering> {
 public:
   explicit Reordering(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      elems_ = (size_t)g.n_fan_proj * g.n_fan_det;
      pool_size_ = (int)cfg_.integer("memPoolSize_Reordering", 16);
      start(6);
   }
   ~Reordering() {
      stop();
      for (auto& p : pools_) glados_gb::MemoryPool<RawDeviceManager>::instance()->freeMemory(p.second);
   }
   void init(int d) { pools_[d] = glados_gb::MemoryPool<RawDeviceManager>::instance()->registerStage(pool_size_, elems_); }
   output_type step(int d, input_type&& in) {
      const auto& g = cfg_.geometry;
      output_type out = glados_gb::MemoryPool<RawDeviceManager>::instance()->requestMemory(pools_[d]);
      check(risa_gb_reorder_enqueue(in.data(), out.data(), g.n_modules, g.n_fan_proj, g.n_fan_det, 1, stream(d)),
            "reorder");
      check_cuda(cudaStreamSynchronize(stream(d)), "Reordering sync");
      copy_meta(out, in, d);
      return out;
   }

 private:
   Config cfg_;
   size_t elems_ = 0;
   int pool_size_ = 16;
   std::map<int, unsigned> pools_;
};

// ---------------------------------------------------------------------------- DetectorInterpolation
// In-place repair of defect detector columns, on the device (the reference
// copies every frame to the host and back for this, DetectorInterpolation.cu:113-139).
class DetectorInterpolation : public DeviceStage<RawDeviceManager, RawDeviceManager, DetectorInterpolation> {
 public:
   explicit DetectorInterpolation(const std::string& config_file) : cfg_(config_file) { start(6); }
   ~DetectorInterpolation() {
      stop();
      for (auto& h : handles_) risa_gb_defects_destroy(h.second);
      for (auto& w : ws_) cudaFree(w.second);
   }
   void init(int d) {
      risa_gb_defects* h = nullptr;
      check(risa_gb_defects_create(&cfg_.geometry, &cfg_.params, 1, &h), "defects_create");
      handles_[d] = h;
      void* w = nullptr;
      check_cuda(cudaMalloc(&w, risa_gb_defects_workspace_bytes(h, 1)), "cudaMalloc");
      ws_[d] = w;
   }
   output_type step(int d, input_type&& in) {
      check(risa_gb_defects_enqueue(handles_[d], in.data(), 1, nullptr, ws_[d], stream(d)), "defects_enqueue");
      check_cuda(cudaStreamSynchronize(stream(d)), "DetectorInterpolation sync");
      return std::move(in);
   }

 private:
   Config cfg_;
   std::map<int, risa_gb_defects*> handles_;
   std::map<int, void*> ws_;
};

// Reads the reference's per-module raw files (OfflineLoader.cu:56-95 for
// data, Attenuation.cu:274-325 for reference and dark measurements): module
// file i (1-based) holds consecutive frames of n_proj x (n_det / n_modules)
// uint16 values, frame f of plane k at block f * n_planes + k.
// Returns frames in the order [frame][plane][proj][det], detector-major.
inline std::vector<uint16_t> read_module_files(const std::string& prefix, const std::string& ending,
                                               int n_modules, int n_frames, int n_planes, int n_proj,
                                               int n_det) {
   const int w = n_det / n_modules;
   const size_t block = (size_t)n_proj * w;
   std::vector<uint16_t> out((size_t)n_frames * n_planes * n_proj * n_det);
   std::vector<uint16_t> buf(block);
   for (int m = 0; m < n_modules; ++m) {
      const std::string path = prefix + std::to_string(m + 1) + ending;
      FILE* f = std::fopen(path.c_str(), "rb");
      if (!f) throw std::runtime_error("risa_gb: cannot open " + path);
      for (int fr = 0; fr < n_frames * n_planes; ++fr) {
         if (std::fread(buf.data(), sizeof(uint16_t), block, f) != block) {
            std::fclose(f);
            throw std::runtime_error("risa_gb: short read in " + path);
         }
         uint16_t* dst = out.data() + (size_t)fr * n_proj * n_det;
         for (int p = 0; p < n_proj; ++p)
            for (int d = 0; d < w; ++d) dst[(size_t)p * n_det + m * w + d] = buf[(size_t)p * w + d];
      }
      std::fclose(f);
   }
   return out;
}

inline std::string with_slash(std::string s) {
   if (!s.empty() && s.back() != '/') s += '/';
   return s;
}

// ---------------------------------------------------------------------------- Attenuation
// uint16 raw -> float attenuation. The constructor reads, repairs and averages
// the reference and dark measurements from the reference's module files
// (referenceInputPath + "ref_empty_tomograph_repaired_DetModNr_<i>.fx",
// darkInputPath + "dark_192.168.100_DetModNr_<i>.fx", Attenuation.cu:185-205);
// tests may pass the measurements directly instead.
class Attenuation : public DeviceStage<RawDeviceManager, FloatDeviceManager, Attenuation> {
 public:
   explicit Attenuation(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      n_ref_ = (int)cfg_.integer("numberOfReferenceFrames", 1);
      n_dark_ = (int)cfg_.integer("numberOfDarkFrames", 1);
      ref_ = read_module_files(with_slash(cfg_.str("referenceInputPath")) + "ref_empty_tomograph_repaired_DetModNr_",
                               ".fx", g.n_modules, n_ref_, g.n_planes, g.n_fan_proj, g.n_fan_det);
      const std::string dark_dir = cfg_.str("darkInputPath");
      if (!dark_dir.empty())
         dark_ = read_module_files(with_slash(dark_dir) + "dark_192.168.100_DetModNr_", ".fx", g.n_modules,
                                   n_dark_, g.n_planes, g.n_fan_proj, g.n_fan_det);
      else
         n_dark_ = 0;
      setup();
   }
   Attenuation(const std::string& config_file, std::vector<uint16_t> ref, int n_ref, std::vector<uint16_t> dark,
               int n_dark)
       : cfg_(config_file), ref_(std::move(ref)), dark_(std::move(dark)), n_ref_(n_ref), n_dark_(n_dark) {
      setup();
   }
   ~Attenuation() {
      stop();
      for (auto& h : handles_) risa_gb_attenuation_destroy(h.second);
      for (auto& p : pools_) glados_gb::MemoryPool<FloatDeviceManager>::instance()->freeMemory(p.second);
   }
   void init(int d) {
      risa_gb_attenuation* h = nullptr;
      check(risa_gb_attenuation_create(&cfg_.geometry, &cfg_.params, ref_.data(), n_ref_,
                                       n_dark_ ? dark_.data() : nullptr, n_dark_, &h),
            "attenuation_create");
      handles_[d] = h;
      pools_[d] = glados_gb::MemoryPool<FloatDeviceManager>::instance()->registerStage(pool_size_, elems_);
   }
   output_type step(int d, input_type&& in) {
      output_type out = glados_gb::MemoryPool<FloatDeviceManager>::instance()->requestMemory(pools_[d]);
      check(risa_gb_attenuation_enqueue(handles_[d], in.data(), out.data(), (int)in.plane(), 1, stream(d)),
            "attenuation_enqueue");
      check_cuda(cudaStreamSynchronize(stream(d)), "Attenuation sync");
      copy_meta(out, in, d);
      return out;
   }

 private:
   void setup() {
      const auto& g = cfg_.geometry;
      elems_ = (size_t)g.n_fan_proj * g.n_fan_det;
      pool_size_ = (int)cfg_.integer("memPoolSize_attenuation", 16);
      start(5);
   }
   Config cfg_;
   std::vector<uint16_t> ref_, dark_;
   int n_ref_ = 1, n_dark_ = 0;
   size_t elems_ = 0;
   int pool_size_ = 16;
   std::map<int, risa_gb_attenuation*> handles_;
   std::map<int, unsigned> pools_;
};

// ---------------------------------------------------------------------------- Fan2Para
class Fan2Para : public DeviceStage<FloatDeviceManager, FloatDeviceManager, Fan2Para> {
 public:
   explicit Fan2Para(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      elems_ = (size_t)g.n_par_proj * g.n_par_det;
      pool_size_ = (int)cfg_.integer("memPoolSize_fan2Para", 16);
      start(4);
   }
   ~Fan2Para() {
      stop();
      for (auto& h : handles_) risa_gb_fan2para_destroy(h.second);
      for (auto& p : pools_) glados_gb::MemoryPool<FloatDeviceManager>::instance()->freeMemory(p.second);
   }
   void init(int d) {
      risa_gb_fan2para* h = nullptr;
      check(risa_gb_fan2para_create(&cfg_.geometry, &cfg_.params, &h), "fan2para_create");
      handles_[d] = h;
      pools_[d] = glados_gb::MemoryPool<FloatDeviceManager>::instance()->registerStage(pool_size_, elems_);
   }
   output_type step(int d, input_type&& in) {
      output_type out = glados_gb::MemoryPool<FloatDeviceManager>::instance()->requestMemory(pools_[d]);
      check(risa_gb_fan2para_enqueue(handles_[d], in.data(), out.data(), (int)in.plane(), 1, stream(d)),
            "fan2para_enqueue");
      check_cuda(cudaStreamSynchronize(stream(d)), "Fan2Para sync");
      copy_meta(out, in, d);
      return out;
   }

 private:
   Config cfg_;
   size_t elems_ = 0;
   int pool_size_ = 16;
   std::map<int, risa_gb_fan2para*> handles_;
   std::map<int, unsigned> pools_;
};

// ---------------------------------------------------------------------------- Filter (in place)
class Filter : public DeviceStage<FloatDeviceManager, FloatDeviceManager, Filter> {
 public:
   explicit Filter(const std::string& config_file) : cfg_(config_file) { start(3); }
   ~Filter() {
      stop();
      for (auto& h : handles_) risa_gb_filter_destroy(h.second);
   }
   void init(int d) {
      risa_gb_filter* h = nullptr;
      check(risa_gb_filter_create(&cfg_.geometry, &cfg_.params, &h), "filter_create");
      handles_[d] = h;
   }
   output_type step(int d, input_type&& in) {
      check(risa_gb_filter_enqueue(handles_[d], in.data(), 1, stream(d)), "filter_enqueue");
      check_cuda(cudaStreamSynchronize(stream(d)), "Filter sync");
      return std::move(in);
   }

 private:
   Config cfg_;
   std::map<int, risa_gb_filter*> handles_;
};

// ---------------------------------------------------------------------------- Backprojection
class Backprojection : public DeviceStage<FloatDeviceManager, FloatDeviceManager, Backprojection> {
 public:
   explicit Backprojection(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      elems_ = (size_t)g.n_pixels * g.n_pixels;
      pool_size_ = (int)cfg_.integer("memPoolSize_backProjection", 16);
      start(2);
   }
   ~Backprojection() {
      stop();
      for (auto& h : handles_) risa_gb_backprojection_destroy(h.second);
      for (auto& p : pools_) glados_gb::MemoryPool<FloatDeviceManager>::instance()->freeMemory(p.second);
   }
   void init(int d) {
      risa_gb_backprojection* h = nullptr;
      check(risa_gb_backprojection_create(&cfg_.geometry, &cfg_.params, &h), "backprojection_create");
      handles_[d] = h;
      pools_[d] = glados_gb::MemoryPool<FloatDeviceManager>::instance()->registerStage(pool_size_, elems_);
   }
   output_type step(int d, input_type&& in) {
      output_type out = glados_gb::MemoryPool<FloatDeviceManager>::instance()->requestMemory(pools_[d]);
      check(risa_gb_backprojection_enqueue(handles_[d], in.data(), out.data(), 1, stream(d)),
            "backprojection_enqueue");
      check_cuda(cudaStreamSynchronize(stream(d)), "Backprojection sync");
      copy_meta(out, in, d);
      return out;
   }

 private:
   Config cfg_;
   size_t elems_ = 0;
   int pool_size_ = 16;
   std::map<int, risa_gb_backprojection*> handles_;
   std::map<int, unsigned> pools_;
};

// ---------------------------------------------------------------------------- Masking (in place)
class Masking : public DeviceStage<FloatDeviceManager, FloatDeviceManager, Masking> {
 public:
   explicit Masking(const std::string& config_file) : cfg_(config_file) { start(1); }
   ~Masking() {
      stop();
      for (auto& h : handles_) risa_gb_masking_destroy(h.second);
      for (auto& w : ws_) cudaFree(w.second);
   }
   void init(int d) {
      risa_gb_masking* h = nullptr;
      check(risa_gb_masking_create(&cfg_.geometry, &cfg_.params, &h), "masking_create");
      handles_[d] = h;
      void* w = nullptr;
      check_cuda(cudaMalloc(&w, risa_gb_masking_workspace_bytes(h, 1)), "cudaMalloc");
      ws_[d] = w;
   }
   output_type step(int d, input_type&& in) {
      check(risa_gb_masking_enqueue(handles_[d], in.data(), 1, ws_[d], stream(d)), "masking_enqueue");
      check_cuda(cudaStreamSynchronize(stream(d)), "Masking sync");
      return std::move(in);
   }

 private:
   Config cfg_;
   std::map<int, risa_gb_masking*> handles_;
   std::map<int, void*> ws_;
};

// ---------------------------------------------------------------------------- D2H
// Device images -> pinned host images (D2H.cu:119-148); keeps an images/s rate.
class D2H : public DeviceStage<FloatDeviceManager, FloatHostManager, D2H> {
 public:
   explicit D2H(const std::string& config_file) : cfg_(config_file) {
      const auto& g = cfg_.geometry;
      elems_ = (size_t)g.n_pixels * g.n_pixels;
      pool_size_ = (int)cfg_.integer("memPoolSize_D2H", 16);
      pool_ = glados_gb::MemoryPool<FloatHostManager>::instance()->registerStage(pool_size_, elems_);
      t0_ = std::chrono::steady_clock::now();
      start(0);
   }
   ~D2H() {
      stop();
      glados_gb::MemoryPool<FloatHostManager>::instance()->freeMemory(pool_);
   }
   double images_per_second() const {
      const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
      return s > 0 ? (double)count_ / s : 0.0;
   }
   void init(int) {}
   output_type step(int d, input_type&& in) {
      output_type out = glados_gb::MemoryPool<FloatHostManager>::instance()->requestMemory(pool_);
      check_cuda(cudaMemcpyAsync(out.data(), in.data(), sizeof(float) * elems_, cudaMemcpyDeviceToHost, stream(d)),
                 "D2H copy");
      check_cuda(cudaStreamSynchronize(stream(d)), "D2H sync");
      copy_meta(out, in, d);
      ++count_;
      return out;
   }

 private:
   Config cfg_;
   size_t elems_ = 0;
   int pool_size_ = 16;
   unsigned pool_ = 0;
   std::atomic<long> count_{0};
   std::chrono::steady_clock::time_point t0_;
};

}  // namespace cuda
}  // namespace risa_gb
