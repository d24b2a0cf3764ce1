/*
 * TEST INFRASTRUCTURE ONLY -- stand-in for <boost/align/assume_aligned.hpp> (used by the
 * reference's CPU loops, e.g. DNKG_FPUT_Toda/cpu-implementation/DNKG_FPUT_Toda.cpp:110-111).
 */
#pragma once
#define BOOST_ALIGN_ASSUME_ALIGNED(p, n) ((p) = static_cast<__typeof__(p)>(__builtin_assume_aligned((p), (n))))
