// Drop-in replacement for the reference's src/GPU.cuh: the same two
// functions, implemented by libhdc_gb300 on sm_103a (gpu_dropin.cpp).
#pragma once
#include <string>
#include <unordered_map>

#include "config.h"

// src/GPU.cuh:6.  Per sequence, its window hypervectors: windows of
// SEQUENCE_LENGTH bases starting every SIM_STEP, (len - L) / step + 1 of them
// (none when the sequence is shorter than one window), each equal to the
// reference CPU encoder's HVCache::compute of the window.  kmer_map is
// accepted for signature compatibility and not read: binders are derived from
// the base hypervectors, which is what a correctly built table holds.
std::vector<std::vector<HV_16>> encode(const std::vector<int16_t>& kmer_map, const std::vector<std::string>& sequences);

// src/GPU.cuh:8-11.  For every input, its k best database entries
// (k clamped to db.size()), descending, keyed by input pointer.  Scores are
// cosines (the scale of the reference GPU search) computed exactly; ties go
// to the lower database index.  Define HDC_DROPIN_NORM_SCORE to rank and
// report on the reference CPU cosine() scale instead (2*(cos - 0.5)).
std::unordered_map<HV_16*, std::vector<std::pair<float, HV_16*>>> cosine_search(const std::vector<HV_16*>& inputs,
                                                                                const std::vector<HV_16*>& db,
                                                                                int k = 1);
