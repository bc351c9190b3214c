// FrameAssembler on the CPU: module packets in any order, concurrent module
// threads, lost / duplicate / malformed / stale packets, ring back-pressure.
#include <algorithm>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

#include "risa_gb/Packets.h"

using namespace risa_gb;

static int failures = 0;
#define EXPECT(c)                                                          \
   do {                                                                    \
      if (!(c)) {                                                          \
         std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);          \
         ++failures;                                                       \
      }                                                                    \
   } while (0)

static uint16_t value(uint64_t f, int m, int p, int d) { return (uint16_t)(f * 7919u + m * 131u + p * 17u + d); }

struct Stream {
   PacketLayout L;
   std::vector<uint8_t> bytes;
   explicit Stream(const PacketLayout& l) : L(l), bytes(l.packet_bytes()) {}
   const uint8_t* packet(uint64_t f, int m, int part) {
      std::vector<uint16_t> pay(L.payload_values());
      for (int pp = 0; pp < L.proj_per_packet; ++pp)
         for (int d = 0; d < L.det_per_module; ++d)
            pay[(size_t)pp * L.det_per_module + d] = value(f, m, part * L.proj_per_packet + pp, d);
      encode_packet(L, f, (uint16_t)part, pay.data(), bytes.data());
      return bytes.data();
   }
};

static bool frame_ok(const PacketLayout& L, uint64_t f, const uint16_t* fr) {
   for (int m = 0; m < L.modules; ++m)
      for (int p = 0; p < L.proj; ++p)
         for (int d = 0; d < L.det_per_module; ++d)
            if (fr[((size_t)m * L.proj + p) * L.det_per_module + d] != value(f, m, p, d)) return false;
   return true;
}

int main() {
   PacketLayout L;
   L.modules = 4;
   L.det_per_module = 16;
   L.proj = 100;
   L.proj_per_packet = 10;
   L.ring = 4;
   EXPECT(L.valid() && L.parts() == 10 && L.packet_bytes() == 10 + 2 * 160);

   // 1. frames 0..11, packets of two consecutive frames interleaved at random,
   //    one consumer thread reading and releasing; one packet of frame 5 lost,
   //    one duplicate, malformed packets
   {
      std::vector<uint16_t> ring(L.ring * L.frame_values());
      FrameAssembler fa(L, ring.data());
      std::vector<uint64_t> got;
      int bad = 0;
      std::thread consumer([&] {
         uint64_t idx;
         const uint16_t* fr;
         while (fa.next(&idx, &fr, 5.0)) {
            if (!frame_ok(L, idx, fr)) ++bad;
            got.push_back(idx);
            fa.release(idx);
         }
      });
      Stream st(L);
      std::mt19937 rng(7);
      for (uint64_t f0 = 0; f0 < 12; f0 += 2) {
         std::vector<std::tuple<uint64_t, int, int>> order;
         for (uint64_t f = f0; f < f0 + 2; ++f)
            for (int m = 0; m < L.modules; ++m)
               for (int p = 0; p < L.parts(); ++p)
                  if (!(f == 5 && m == 2 && p == 3)) order.emplace_back(f, m, p);
         std::shuffle(order.begin(), order.end(), rng);
         for (auto& [f, m, p] : order) {
            Ingest r;
            do {  // a full ring makes the sender retry once the consumer released a frame
               r = fa.ingest(m, st.packet(f, m, p), L.packet_bytes());
               if (r == Ingest::ring_full) std::this_thread::sleep_for(std::chrono::milliseconds(1));
            } while (r == Ingest::ring_full);
            EXPECT(r == Ingest::accepted);
         }
         if (f0 == 0) {
            EXPECT(fa.ingest(1, st.packet(1, 1, 1), L.packet_bytes()) == Ingest::duplicate ||
                   fa.ingest(1, st.packet(1, 1, 1), L.packet_bytes()) == Ingest::stale);
            EXPECT(fa.ingest(1, st.packet(1, 1, 1), L.packet_bytes() - 2) == Ingest::malformed);
            EXPECT(fa.ingest(9, st.packet(1, 1, 1), L.packet_bytes()) == Ingest::malformed);
         }
      }
      fa.finish();
      consumer.join();
      EXPECT(bad == 0);
      const std::vector<uint64_t> want = {0, 1, 2, 3, 4, 6, 7, 8, 9, 10, 11};
      EXPECT(got == want);
      EXPECT(fa.skipped() == 1);
      // a packet of an already delivered frame is stale
      EXPECT(fa.ingest(0, st.packet(3, 0, 0), L.packet_bytes()) == Ingest::stale);
   }

   // 2. one thread per module, frames 0..39, consumer releases promptly
   {
      std::vector<uint16_t> ring(L.ring * L.frame_values());
      FrameAssembler fa(L, ring.data());
      const uint64_t F = 40;
      std::vector<std::thread> producers;
      for (int m = 0; m < L.modules; ++m)
         producers.emplace_back([&, m] {
            Stream st(L);
            for (uint64_t f = 0; f < F; ++f)
               for (int p = L.parts() - 1; p >= 0; --p) {  // parts in reverse order
                  Ingest r;
                  do {
                     r = fa.ingest(m, st.packet(f, m, p), L.packet_bytes());
                     if (r == Ingest::ring_full) std::this_thread::yield();
                  } while (r == Ingest::ring_full);
               }
         });
      uint64_t n = 0, expect = 0, idx;
      const uint16_t* fr;
      int bad = 0;
      while (n < F && fa.next(&idx, &fr, 5.0)) {
         if (idx != expect || !frame_ok(L, idx, fr)) ++bad;
         ++expect;
         ++n;
         fa.release(idx);
      }
      for (auto& t : producers) t.join();
      EXPECT(n == F && bad == 0 && fa.skipped() == 0 && fa.abandoned() == 0);
   }

   // 3. without releases the ring refuses to overwrite complete unread frames
   {
      std::vector<uint16_t> ring(L.ring * L.frame_values());
      FrameAssembler fa(L, ring.data());
      Stream st(L);
      for (uint64_t f = 0; f < (uint64_t)L.ring; ++f)
         for (int m = 0; m < L.modules; ++m)
            for (int p = 0; p < L.parts(); ++p) fa.ingest(m, st.packet(f, m, p), L.packet_bytes());
      EXPECT(fa.ingest(0, st.packet(L.ring, 0, 0), L.packet_bytes()) == Ingest::ring_full);
      uint64_t idx;
      const uint16_t* fr;
      EXPECT(fa.next(&idx, &fr, 1.0) && idx == 0 && frame_ok(L, 0, fr));
      fa.release(0);
      EXPECT(fa.ingest(0, st.packet(L.ring, 0, 0), L.packet_bytes()) == Ingest::accepted);
   }

   // 4. the reference's rule (Completion::last_part): a module announces a frame
   //    with its last part; the newest frame all modules announced is handed
   //    out; frame 0 never is; a lost middle part leaves the slot's old values;
   //    frames between two hand-outs are skipped
   {
      std::vector<uint16_t> ring(L.ring * L.frame_values(), 0);
      FrameAssembler fa(L, ring.data(), 0, Completion::last_part);
      Stream st(L);
      uint64_t idx;
      const uint16_t* fr;
      auto send = [&](uint64_t f, bool lose) {
         for (int m = 0; m < L.modules; ++m)
            for (int p = 0; p < L.parts(); ++p)
               if (!(lose && m == 1 && p == 3)) {
                  const Ingest r = fa.ingest(m, st.packet(f, m, p), L.packet_bytes());
                  EXPECT(r == (f == 0 ? Ingest::stale : Ingest::accepted));
               }
      };
      send(0, false);
      EXPECT(!fa.next(&idx, &fr, 0.05));  // the reference's fetch never returns index 0
      for (uint64_t f = 1; f < 10; ++f) {
         // every module's last part but one: not yet announced by all
         for (int m = 0; m < L.modules; ++m)
            for (int p = 0; p < L.parts(); ++p)
               if (!(f == 4 && m == 1 && p == 3) && !(m == L.modules - 1 && p == L.parts() - 1))
                  EXPECT(fa.ingest(m, st.packet(f, m, p), L.packet_bytes()) == Ingest::accepted);
         EXPECT(!fa.next(&idx, &fr, 0.01));
         EXPECT(fa.ingest(L.modules - 1, st.packet(f, L.modules - 1, L.parts() - 1), L.packet_bytes()) ==
                Ingest::accepted);
         EXPECT(fa.next(&idx, &fr, 1.0) && idx == f);
         if (f == 4) {
            // slot 0 held nothing before (frame 0 was stale): the lost part reads 0
            bool lost_zero = true, rest_ok = true;
            for (int m = 0; m < L.modules; ++m)
               for (int p = 0; p < L.proj; ++p)
                  for (int d = 0; d < L.det_per_module; ++d) {
                     const uint16_t v = fr[((size_t)m * L.proj + p) * L.det_per_module + d];
                     if (m == 1 && p / L.proj_per_packet == 3) lost_zero &= v == 0;
                     else rest_ok &= v == value(f, m, p, d);
                  }
            EXPECT(lost_zero && rest_ok);
         } else {
            EXPECT(frame_ok(L, f, fr));
         }
         fa.release(idx);
      }
      send(10, false);
      send(11, false);
      EXPECT(fa.next(&idx, &fr, 1.0) && idx == 11 && frame_ok(L, 11, fr));
      EXPECT(fa.skipped() == 1);
      fa.release(11);
      fa.finish();
      EXPECT(!fa.next(&idx, &fr, 1.0));
      send(14, false);  // frame 10's slot (never handed out) is taken over
      EXPECT(fa.abandoned() == 1);
   }

   std::printf("packets: failures=%d\n", failures);
   return failures ? 1 : 0;
}
