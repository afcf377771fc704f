// Window widths of the MSM per (log2 n, curve), measured on NVIDIA GB300 by bend-groth16_gb300/tune_msm.py
// and committed; 0 = not measured, the size rule of msm_pick_c / msm_pick_c_table applies.
// Rows: [0] G1, [1] G2; columns: floor(log2 n) = kTuneMinLog2 .. kTuneMaxLog2.
#pragma once

namespace bg {

constexpr int kTuneMinLog2 = 10;
constexpr int kTuneMaxLog2 = 22;
// one bucket set per window (standalone MSMs, one-shot proofs)
constexpr signed char kTuneSets[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    {8, 8, 9, 9, 9, 10, 11, 12, 15, 15, 15, 15, 17},
    {8, 9, 9, 9, 9, 10, 11, 12, 15, 15, 15, 0, 0}};
// window tables of resident keys (one shared bucket set)
constexpr signed char kTuneTables[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    {9, 0, 11, 0, 13, 0, 15, 0, 17, 0, 19, 0, 0},
    {10, 0, 11, 0, 14, 0, 15, 0, 17, 0, 17, 0, 0}};

}  // namespace bg
