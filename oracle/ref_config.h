/*
 * Compile-time configuration override for building the reference's CPU
 * sources (src/HV.cpp, src/encoder.cpp, targets/propogate-children.cpp,
 * src/hierarchy.cpp of benlaflen/bacterial-classification) at other sizes.
 *
 * The reference fixes its sizes in src/config.h:5-8 with plain #defines and
 * no #ifndef guards, so -D cannot change them.  The build recipe force-
 * includes the reference's own config.h first and this header second; the
 * reference's "#pragma once" then skips config.h when HV.h includes it, and
 * the values below win.  The derived macros (HV_WORDS, KMER_COUNT, K, ...)
 * are defined in terms of these and follow automatically.
 */
#ifndef REF_HV_DIM
#error "define REF_HV_DIM, REF_KMER, REF_WINDOW, REF_STEP"
#endif
#undef KMER_SIZE
#undef HV_DIM
#undef SEQUENCE_LENGTH
#undef SIM_STEP
#define KMER_SIZE REF_KMER
#define HV_DIM REF_HV_DIM
#define SEQUENCE_LENGTH REF_WINDOW
#define SIM_STEP REF_STEP
