// Uneven sweep: many independent parallel-beam reconstructions of different
// shapes (image side, angles, rays, filter) in ONE persistent launch.
//
// Per instance: uint16 counts [Pp][Dp] -> repair of known defective detector
// columns (the run rule of interpolateDefectDetectors,
// interpolationFunctions.h:73-97, NONE-mode rounding) -> attenuation
// -log((raw - dark) / (ref - dark)) with a flat field -> ramp-family filter
// (radix-16 register FFT, zero padded to a power of two >= 2 Dp) -> linear
// backprojection (staged windows, NONE-mode sampling) with the circular mask.
//
// Work items (host-built, dependency-ordered): row groups of an instance
// (two rows per LEN/16 threads, 8192/LEN rows per item) and 32 x 32 image
// tiles. A CTA takes the next item from a global counter; a tile waits
// (bounded) until every row group of its instance has been written. Row
// groups of instance i+1 are queued before the tiles of instance i, row
// groups never wait, and every awaited item was taken earlier by a running
// CTA, so the wait always ends without co-residency of the grid.
#pragma once
#include <vector>
#include <cuda_runtime.h>

#include <cstdint>

namespace risa_gb {

// Repair rule of one detector column: len 0 = good column; otherwise the
// column is element m of a run of len defective columns between the good
// columns left and right.
struct SweepRepair {
   uint16_t left, right, m, len;
};

struct SweepInst {
   int N, Pp, Dp, len;          // image side, angles, rays, FFT length (512 .. 4096)
   int row_items, tiles_x, tiles;
   int win_lo, win_len;         // pair-sinogram padding: bin k at u = k + win_lo, u < win_len (both even)
   int wlen2;                   // staged window length in bins (even)
   int masking;
   float norm, mask_value;
   float dark, logden;          // flat field: dark level, log(max(ref - dark, 1e-5))
   size_t raw_off, img_off, pair_off;  // element offsets: uint16, float, float2 (pair_off even)
   const float* a;              // [Pp] per-angle ray-coordinate steps (FP32)
   const float* b;
   const double* ad;            // [Pp] FP64 copies and the offset of the tile origin
   const double* bd;
   const double* t0;
   const float2* h;             // [len] frequency response, 1/len included
   const SweepRepair* repair;   // [Dp] or nullptr
   const int2* tile_win;        // [tile][angle] (even window start, bits of the float origin coordinate),
                                // sweep_tile_windows; nullptr: computed in FP64 by the tile
};

enum SweepKind { kSweepRows = 0, kSweepTile = 1 };
struct SweepItem {
   int inst, kind, index;
};

struct SweepArgs {
   const SweepInst* inst;
   const SweepItem* items;
   int n_items;
   const uint16_t* raw;
   float* img;
   float2* pairs;
   const float2* twp[4];          // radix-16 pass twiddles for len 512, 1024, 2048, 4096
   int* next;                     // work counter, zero at launch
   int* rows_done;                // [instances] row items finished
   int* tiles_done;               // [instances] tiles finished
   unsigned long long* t_first;   // [instances] start of the first row item (%globaltimer ns), ~0 at launch
   unsigned long long* t_done;    // [instances] end of the last tile, 0 at launch
   unsigned long long* t_launch;  // [1] earliest CTA start, ~0 at launch
   int* err;                      // nonzero: a bounded wait gave up (the CTA stopped)
   int ach;                       // angles per staged chunk, <= kSweepACH (set by launch_sweep)
};

// Angles per staged chunk of a tile (one CTA barrier per chunk): 64, or 32
// where 64 windows of the widest instance do not fit in shared memory.
constexpr int kSweepACH = 64;

// Staged window length (bins, even) for a given bins-per-pixel scale.
int sweep_window_len(float scale);
// Padding of an instance's pair sinogram (mirrors the tile kernel's arithmetic).
void sweep_window_extent(const float* a, const float* b, const double* ad, const double* bd, const double* t0,
                         int Pp, int N, int wlen2, bool masking, int* win_lo, int* win_len);
// The tile kernel's window start and window-relative origin of every 32 x 32
// tile and angle of an instance ([tile][angle]), in the same rounded FP64
// steps, appended to `out`.
void sweep_tile_windows(const float* a, const float* b, const double* ad, const double* bd, const double* t0,
                        int Pp, int N, std::vector<int2>& out);
size_t sweep_smem_bytes(int max_wlen2, int ach = kSweepACH);
cudaError_t launch_sweep(const SweepArgs& a, int max_wlen2, cudaStream_t st, int* grid_out);

}  // namespace risa_gb
