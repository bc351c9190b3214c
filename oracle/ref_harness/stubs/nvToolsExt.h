// Stand-in for the legacy NVTX header (CUDA 13 ships only nvtx3); unused by the harness.
#pragma once
