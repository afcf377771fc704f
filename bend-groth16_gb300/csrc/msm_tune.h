// Window widths of the MSM per (log2 n, curve), measured on NVIDIA GB300 by bend-groth16_gb300/tune_msm.py
// and committed; 0 = not measured, the size rule of msm_pick_c / msm_pick_c_table applies
// (msm_pick_c_proof: the bucket-set-per-window entry).
// Rows: [0] G1, [1] G2; columns: floor(log2 n) = kTuneMinLog2 .. kTuneMaxLog2.
#pragma once

namespace bg {

constexpr int kTuneMinLog2 = 10;
constexpr int kTuneMaxLog2 = 22;
// one bucket set per window (standalone MSMs)
constexpr signed char kTuneSets[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    {8, 8, 9, 9, 9, 10, 11, 12, 15, 15, 15, 15, 17},
    {8, 9, 9, 9, 9, 10, 11, 12, 15, 15, 15, 0, 0}};
// window tables of resident keys (one shared bucket set)
constexpr signed char kTuneTables[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    {9, 0, 11, 0, 14, 0, 15, 0, 17, 0, 17, 0, 0},
    {11, 0, 11, 0, 13, 0, 15, 0, 18, 0, 17, 0, 0}};
// one bucket set per window inside a proof (one-shot proofs): the MSMs share the GPU with
// each other's reductions and the QAP, which moves the best width from the standalone one
constexpr signed char kTuneProofSets[2][kTuneMaxLog2 - kTuneMinLog2 + 1] = {
    {10, 0, 11, 0, 10, 0, 12, 0, 13, 0, 15, 0, 0},
    {8, 0, 9, 0, 9, 0, 12, 0, 14, 0, 15, 0, 0}};

}  // namespace bg
