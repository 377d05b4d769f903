// Compile-time configuration of the GPU.cuh drop-in: the same macro names and
// derived values as the reference's src/config.h, with the reference's
// defaults, each overridable with -D (the reference's header cannot be).
#pragma once
#include <stdint.h>

#include <vector>

#ifndef KMER_SIZE
#define KMER_SIZE 5
#endif
#ifndef HV_DIM
#define HV_DIM 10000
#endif
#ifndef SEQUENCE_LENGTH
#define SEQUENCE_LENGTH 125
#endif
#ifndef SIM_STEP
#define SIM_STEP 10
#endif

#define HV_WORDS ((HV_DIM + 63) / 64)
#define KMER_BITS (2 * KMER_SIZE)
#define KMER_COUNT (1 << KMER_BITS)
#define KMER_MASK (KMER_COUNT - 1)

using HV = std::vector<uint64_t>;
using HV_16 = std::vector<int16_t>;
