// scan.cuh — internal entry points of the scan / sort / compaction units.
#pragma once
#include "common.cuh"

size_t fl_scan_scratch_bytes(size_t n);
// Exclusive scan using caller-provided scratch (fl_scan_scratch_bytes(n) bytes).
int fl_scan_u32_with(fl_ctx* ctx, const uint32_t* in, uint32_t* out, size_t n, uint32_t* total, void* scratch);
int fl_launch_fill_u32(fl_ctx* ctx, uint32_t* p, uint32_t v, size_t n);
size_t fl_sort_scratch_bytes(size_t n, int passes);
// Sort using caller-provided scratch (fl_sort_scratch_bytes(n, passes) bytes).
int fl_sort_pairs_with(fl_ctx* ctx, uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                       void* scratch);
