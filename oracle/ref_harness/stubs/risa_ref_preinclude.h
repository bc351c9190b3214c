// cuFFT result codes that CUDA 13 removed but the reference's error helper still names.
// Distinct values outside cuFFT's range; they are never returned.
#pragma once
#include <cufft.h>
#include <numeric>
#define CUFFT_INCOMPLETE_PARAMETER_LIST ((cufftResult)1001)
#define CUFFT_PARSE_ERROR ((cufftResult)1002)
#define CUFFT_LICENSE_ERROR ((cufftResult)1003)
