// Test infrastructure only: pre-included when the reference's own sources are
// compiled into the CPU oracle binary (oracle/_ref/fsm).
//
// The reference's mining recursion (gspan.cu:1118-1169, `mine`) calls
// `support_gpu(g, dfs_code, layered_embeddings)` with a `const CSRGraph&` and two
// NON-const lvalues.  The reference defines `support_gpu` with const references
// (gspan.cu:200).  Declaring an overload that takes the last two arguments by
// non-const reference makes it the better overload-resolution match for that one
// call site, so the reference's recursion, extension, canonical check and report
// run unmodified while support is computed on the CPU by `ref_support.cc`, with
// the same set semantics as the reference's CUDA kernel (gspan.cu:165-190,
// 255-260, 282-287).  No reference source file is copied or edited.
#pragma once
#include "graph.h"
#include "gspan.h"

int support_gpu(const CSRGraph& g, DFSCode& dfs_code, LayeredEmbeddings& layered_embeddings);
