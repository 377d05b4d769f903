/*
 * Forced include for building the reference's targets/identify.cpp with
 * compute-semantics windows.  TEST INFRASTRUCTURE ONLY.
 *
 * identify calls cache.precompute(ref) (targets/identify.cpp:150) before
 * similarity(); precompute fills the cache with sliding-window updates whose
 * added k-mers are offset by one position (src/encoder.cpp:176), so every
 * window after the first differs from HVCache::compute of the same window.
 * With the call turned into a no-op, similarity() computes each window
 * directly (src/encoder.cpp:208 -> get -> compute), which is the behaviour the
 * GPU path reproduces.  This header is included into identify.cpp only: it
 * pulls in encoder.h first (so the class declaration is untouched), then
 * rewrites the one call expression.
 */
#include "encoder.h"
#define precompute(seq) kmers.size()
