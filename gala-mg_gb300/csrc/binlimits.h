// binlimits.h - upper degrees of the tunable phase-1 degree bins (shared by
// host and device code).
#pragma once

namespace gala {

// Upper degrees of bins 4, 5 and 6; each at most its table limit (256 / 2048 /
// 8192) and not below the previous one.  Bins 0-3 are fixed by their lane-group
// sizes (4 / 8 / 16 / 32).
struct BinLimits {
    int m4 = 256, m5 = 2048, m6 = 8192;
};
constexpr int kMaxWarpDeg = 256, kMaxCta5Deg = 2048, kMaxCta6Deg = 8192;

}  // namespace gala
