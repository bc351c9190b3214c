// Online input: the detector modules' packet format and frame assembly.
//
// Reference: each detector module streams its projections to its own port
// (ReceiverModule.cpp:56-116). A packet is
//    [uint64 frame index][uint16 part][proj_per_packet x det_per_module uint16]
// (native byte order, no padding: the payload starts at byte 10); part p holds
// projections p*proj_per_packet .. of that module. The reference copies every
// packet into a per-module ring of inputBufferSize frames, announces a frame of
// a module when its last part arrives, and hands out the newest frame every
// module has announced (OnlineReceiverNotification.h:53-79); the frame is then
// gathered module by module into a [module][projection][detector] image
// (Receiver.cpp:71-86).
//
// Here packets land directly in a caller-owned ring of whole frames in that
// module-major layout -- the layout the engine's module_major mode reads, so a
// frame goes to the device with one copy and no reordering. Two completion
// rules (Completion):
//   exact (default): a frame is complete when every part of every module has
//     arrived (a lost packet is detected, not overwritten silently); frames are
//     handed out in index order, and an incomplete frame is given up once a
//     frame skip_lag newer is complete (counted as skipped);
//   last_part: the reference's rule -- a module announces a frame when the
//     frame's last part arrives (ReceiverModule.cpp:85-86,111-112) and the
//     frame handed out is the newest one every module has announced, provided
//     it is newer than the last one handed out (OnlineReceiverNotification.h:
//     53-79, whose last index starts at 0, so frame 0 is never handed out).
//     Parts lost before the last one leave what the slot held before, and the
//     frames between two hand-outs are skipped.
// Unlike the reference's receiver, a slot whose frame has not been released
// is never overwritten (the sender gets ring_full and retries). Sockets are
// not part of this file: any transport calls ingest() with the packet bytes.
#pragma once
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <vector>

namespace risa_gb {

struct PacketLayout {
   int modules = 0;          // numberOfDetectorModules
   int det_per_module = 0;   // numberOfDetectorsPerModule
   int proj = 0;             // projections per frame (samplingRate * 1e6 / scanRate)
   int proj_per_packet = 0;  // numberOfProjectionsPerPacket
   int ring = 0;             // inputBufferSize: frames the ring holds
   static constexpr size_t kHeaderBytes = sizeof(uint64_t) + sizeof(uint16_t);

   int parts() const { return proj / proj_per_packet; }
   size_t payload_values() const { return (size_t)proj_per_packet * det_per_module; }
   size_t packet_bytes() const { return kHeaderBytes + sizeof(uint16_t) * payload_values(); }
   size_t module_values() const { return (size_t)proj * det_per_module; }
   size_t frame_values() const { return (size_t)modules * module_values(); }
   bool valid() const {
      return modules > 0 && det_per_module > 0 && proj_per_packet > 0 && proj % proj_per_packet == 0 &&
             parts() <= 65536 && ring > 0;
   }
};

// Writes one packet (senders, tests): out holds layout.packet_bytes() bytes.
inline void encode_packet(const PacketLayout& L, uint64_t index, uint16_t part, const uint16_t* payload,
                          uint8_t* out) {
   std::memcpy(out, &index, sizeof(index));
   std::memcpy(out + sizeof(index), &part, sizeof(part));
   std::memcpy(out + PacketLayout::kHeaderBytes, payload, sizeof(uint16_t) * L.payload_values());
}

// Outcome of FrameAssembler::ingest.
enum class Ingest { accepted, duplicate, malformed, stale, ring_full };

// When a frame may be handed out (see the top of this file).
enum class Completion { exact, last_part };

// Assembles packets of all modules into whole frames in a ring of layout.ring
// frames [ring][module][projection][detector] (caller-owned, e.g. pinned host
// memory). Thread-safe: one thread per module may call ingest() concurrently
// with a consumer calling next()/release(). The payload copy is done under
// the lock, so a slot is never reused while a packet is being written to it.
class FrameAssembler {
  public:
   // skip_lag (exact rule): an incomplete frame is given up once a frame that
   // many indices newer is complete (default: half the ring; must be below the
   // ring size so that frame has a slot of its own)
   FrameAssembler(const PacketLayout& layout, uint16_t* frames, int skip_lag = 0,
                  Completion rule = Completion::exact)
       : L_(layout), frames_(frames), slots_(layout.ring),
         lag_(skip_lag > 0 ? skip_lag : (layout.ring / 2 > 0 ? layout.ring / 2 : 1)), rule_(rule) {
      if (!L_.valid() || !frames_ || lag_ >= std::max(2, L_.ring))
         throw std::invalid_argument("FrameAssembler: inconsistent packet layout or skip lag");
      for (auto& s : slots_) s.have.assign((size_t)L_.modules * L_.parts(), 0);
      if (rule_ == Completion::last_part) {
         // the reference's notification starts with every module at index 0
         // and its last handed-out index at 0
         announced_.assign(L_.modules, 0);
         delivered_any_ = true;
         last_delivered_ = 0;
      }
   }

   Completion rule() const { return rule_; }

   const PacketLayout& layout() const { return L_; }

   Ingest ingest(int module, const uint8_t* packet, size_t bytes) {
      if (module < 0 || module >= L_.modules || !packet || bytes != L_.packet_bytes()) return Ingest::malformed;
      uint64_t index = 0;
      uint16_t part = 0;
      std::memcpy(&index, packet, sizeof(index));
      std::memcpy(&part, packet + sizeof(index), sizeof(part));
      if ((int)part >= L_.parts()) return Ingest::malformed;
      std::lock_guard<std::mutex> lk(m_);
      if (delivered_any_ && index <= last_delivered_) return Ingest::stale;
      const size_t slot_no = (size_t)(index % (uint64_t)L_.ring);
      Slot& s = slots_[slot_no];
      if (!s.used || s.index != index) {
         if (s.used && index < s.index) return Ingest::stale;
         // The slot's frame is taken over only once the consumer released it,
         // or -- never handed out -- once a newer frame was delivered past it
         // (it was skipped). Otherwise the sender is ahead by a whole ring: it
         // retries.
         const bool skipped = s.used && !s.delivered && delivered_any_ && s.index < last_delivered_;
         if (s.used && !s.released && !skipped) return Ingest::ring_full;
         if (skipped) ++abandoned_;
         s.used = true;
         s.index = index;
         s.count = 0;
         s.complete = s.delivered = s.released = false;
         std::fill(s.have.begin(), s.have.end(), (uint8_t)0);
      }
      const size_t bit = (size_t)module * L_.parts() + part;
      if (s.have[bit]) {
         ++duplicates_;
         return Ingest::duplicate;
      }
      uint16_t* dst = frames_ + slot_no * L_.frame_values() + (size_t)module * L_.module_values() +
                      (size_t)part * L_.payload_values();
      std::memcpy(dst, packet + PacketLayout::kHeaderBytes, sizeof(uint16_t) * L_.payload_values());
      s.have[bit] = 1;
      if (++s.count == L_.modules * L_.parts()) {
         s.complete = true;
         if (rule_ == Completion::exact) cv_.notify_all();
      }
      if (rule_ == Completion::last_part && (int)part == L_.parts() - 1) {
         if (announced_[module] < index) announced_[module] = index;
         cv_.notify_all();
      }
      return Ingest::accepted;
   }

   // Waits (up to timeout_s) for the next complete frame in index order and
   // returns its index and ring memory; false on timeout, or when finish() was
   // called and no complete frame is left. Older incomplete frames are skipped.
   bool next(uint64_t* index, const uint16_t** frame, double timeout_s) {
      std::unique_lock<std::mutex> lk(m_);
      const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
      if (rule_ == Completion::last_part) return next_last_part(lk, deadline, index, frame);
      for (;;) {
         Slot* best = nullptr;
         uint64_t newest_complete = 0;
         for (auto& s : slots_) {
            if (!s.used || s.delivered || (delivered_any_ && s.index <= last_delivered_)) continue;
            if (s.complete) {
               if (!best || s.index < best->index) best = &s;
               newest_complete = std::max(newest_complete, s.index);
            }
         }
         // every older frame still arriving is waited for until a frame
         // skip_lag newer than it is complete (or the stream finished)
         if (best && !finished_) {
            bool open_below = false;
            uint64_t newest_open = 0;
            for (auto& s : slots_)
               if (s.used && !s.complete && (!delivered_any_ || s.index > last_delivered_) && s.index < best->index) {
                  open_below = true;
                  newest_open = std::max(newest_open, s.index);
               }
            if (open_below && newest_complete < newest_open + (uint64_t)lag_) best = nullptr;
         }
         if (best) {
            if (delivered_any_) skipped_ += best->index - last_delivered_ - 1;
            best->delivered = true;
            last_delivered_ = best->index;
            delivered_any_ = true;
            *index = best->index;
            *frame = frames_ + (size_t)(best - slots_.data()) * L_.frame_values();
            return true;
         }
         if (finished_) return false;
         if (cv_.wait_until(lk, deadline) == std::cv_status::timeout) return false;
      }
   }

   // The consumer is done with frame `index` (its slot may be reused).
   void release(uint64_t index) {
      std::lock_guard<std::mutex> lk(m_);
      Slot& s = slots_[(size_t)(index % (uint64_t)L_.ring)];
      if (s.used && s.index == index) s.released = true;
   }

   // No more packets: next() drains the complete frames, then returns false.
   void finish() {
      std::lock_guard<std::mutex> lk(m_);
      finished_ = true;
      cv_.notify_all();
   }

   uint64_t skipped() const { std::lock_guard<std::mutex> lk(m_); return skipped_; }
   uint64_t abandoned() const { std::lock_guard<std::mutex> lk(m_); return abandoned_; }
   uint64_t duplicates() const { std::lock_guard<std::mutex> lk(m_); return duplicates_; }

  private:
   // The reference's fetch(): the smallest of the modules' newest announced
   // indices, once it exceeds the last index handed out.
   template <class Deadline>
   bool next_last_part(std::unique_lock<std::mutex>& lk, const Deadline& deadline, uint64_t* index,
                       const uint16_t** frame) {
      for (;;) {
         const uint64_t m = *std::min_element(announced_.begin(), announced_.end());
         if (m > last_delivered_) {
            Slot& s = slots_[(size_t)(m % (uint64_t)L_.ring)];
            skipped_ += m - last_delivered_ - 1;
            last_delivered_ = m;
            if (s.used && s.index == m) {  // always so: an unreleased slot is never taken over
               s.delivered = true;
               *index = m;
               *frame = frames_ + (size_t)(&s - slots_.data()) * L_.frame_values();
               return true;
            }
            ++skipped_;
            continue;
         }
         if (finished_) return false;
         if (cv_.wait_until(lk, deadline) == std::cv_status::timeout) return false;
      }
   }

   struct Slot {
      bool used = false, complete = false, delivered = false, released = false;
      uint64_t index = 0;
      int count = 0;
      std::vector<uint8_t> have;  // [module][part]
   };
   PacketLayout L_;
   uint16_t* frames_;
   std::vector<Slot> slots_;
   int lag_;
   Completion rule_;
   std::vector<uint64_t> announced_;  // last_part rule: newest announced index per module
   mutable std::mutex m_;
   std::condition_variable cv_;
   bool delivered_any_ = false, finished_ = false;
   uint64_t last_delivered_ = 0, skipped_ = 0, abandoned_ = 0, duplicates_ = 0;
};

}  // namespace risa_gb
