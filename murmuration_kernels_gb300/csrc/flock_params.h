// Model constants of the starling-flock step, shared by the CUDA kernels and
// the host library. Values follow the reference's crates/flock-ref/src/params.rs:5-58
// (and cuda/params.cuh:6-33): every constant is an f32 and every derived
// constant is folded in f32, left to right, as rustc folds it.
#pragma once

#include <stdint.h>

namespace flk {

constexpr float DT = 0.005f;                 // integration step [s]
constexpr float DU = 0.05f;                  // reaction time: a decision is held this long [s]
constexpr float V0 = 10.0f;                  // cruise speed [m/s]
constexpr float MASS = 0.08f;                // [kg]
constexpr float CL_CD = 3.3f;                // lift-to-drag ratio
constexpr float G = 9.81f;                   // [m/s^2]
constexpr float L0 = MASS * G;               // default lift [N]
constexpr float D0 = L0 / CL_CD;             // default drag = thrust [N]
constexpr float TAU = 1.0f;                  // speed relaxation [s]
constexpr float TAU_ROLL = 0.15f;            // roll response [s]
constexpr float MAX_ROLL_RATE = 6.0f;        // [rad/s]
constexpr float MAX_BANK = 80.0f * 3.14159265358979323846f / 180.0f;
constexpr float V_MIN = 0.5f * V0;
constexpr float V_MAX = 2.0f * V0;
constexpr float N_C = 6.5f;                  // topological range
constexpr float R_MAX = 100.0f;              // max perception radius [m]
constexpr float RADIUS_LERP = 0.1f;
constexpr float R_H = 0.2f;                  // radius of maximal separation [m]
constexpr float SIGMA = 1.37f;               // separation Gaussian sd [m]
constexpr float W_SEP = 1.0f;
constexpr float W_ALIGN = 0.5f;
constexpr float W_COH = 0.65f;
constexpr float BLIND_COS = -0.70710678118654752440f;
constexpr float W_ROOST_V = 0.2f;
constexpr float H_ROOST_V = 40.0f;
constexpr float Z0 = 100.0f;                 // preferred height [m]
constexpr float GRID_CELL = 4.0f;            // hash cell edge [m]
constexpr float RADIUS_EXP = RADIUS_LERP / 3.0f;
constexpr float TWO_SIGMA2 = 2.0f * SIGMA * SIGMA;
constexpr float INV_CELL = 1.0f / GRID_CELL;

// Generator constants (crates/flock-ref/src/state.rs:52-54).
constexpr float DENSITY = 0.5f;
constexpr float START_RADIUS = 1.5f;

// Words per bird in a .flk record (state.rs:16).
constexpr int WORDS = 15;

// The adaptive-radius factor (N_C / n)^(RADIUS_EXP) is tabulated for
// n = 0 .. RADIUS_TABLE-1 from the host libm, the function the CPU oracle
// calls, so the new radius agrees with it bit for bit; larger n use powf.
constexpr int RADIUS_TABLE = 1 << 16;

}  // namespace flk
