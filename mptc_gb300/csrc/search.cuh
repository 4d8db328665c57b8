// The index-block search of DXTImage::Reencode (codec/dxt_image.cpp:652-957).
//
// For a block and a candidate index word (the interp of a block in the search
// window) the reference assigns the candidate's indices, refits both endpoints
// by least squares in float, snaps them with ToFiveBits/ToSixBits, and keeps
// the candidate only if Pack565(ep1) > Pack565(ep2); the candidate's error is
// floor(SSE/48) against the block's own pixels, compared with the block's stb
// error (orig_err) (candidate_eval.cuh). Positions are scanned row by row; a
// candidate replaces the running minimum when err_diff < min; the first
// err_diff <= 0 pins min to 0 and ends that ROW only, so a later row can still
// replace the selection with a strictly negative err_diff. The kernels apply
// that rule in closed form over the window's positions (selection.cuh).
//
// The inter search reads the previous frame only and runs fully parallel
// (inter_search.cuh). The intra search reads this frame's blocks as already
// final in raster order, so on an intra frame it runs as a dataflow over
// blocks in wavefront order, each block waiting (bounded) on the completion
// words of its causal window (completion.cuh); on an inter frame it iterates
// fixed-point sweeps over the few blocks the inter pass left open
// (intra_search.cuh). scan.cuh holds the ordered compactions of a frame.
#pragma once

#include "candidate_eval.cuh"
#include "selection.cuh"
#include "completion.cuh"
#include "inter_search.cuh"
#include "intra_search.cuh"
#include "scan.cuh"
