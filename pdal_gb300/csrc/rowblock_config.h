/*
 * rowblock_config.h -- sizes shared by the row-block planner (host) and the
 * row-block kernels (device).
 */
#pragma once

namespace pdal {
constexpr int kThreads = 256;          /* threads per row block */
constexpr int kMaxRowsPerBlock = 512;  /* rows in one STREAM block */
constexpr int kLongStride = 4;         /* partial slots per long-row piece */
} // namespace pdal
