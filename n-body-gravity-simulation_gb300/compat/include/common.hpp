// common.hpp -- constants of the reference's CUDA host API (CUDA/include/common.hpp:29-46),
// for code written against that API and linked with libnbody_compat.so.
// Units: AU, solar masses, years, so G = 4 pi^2.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace constant {
constexpr double PI = 3.14159265358979323846;
constexpr double G = 4.0 * PI * PI;
constexpr double AU = 1.495978707e11;             // m
constexpr double SOLAR_MASS = 1.98847e30;         // kg
constexpr double SOLAR_YEAR = 365.25 * 24 * 3600; // s

// Kept for source compatibility.  The engine sizes its tree per call and
// honours the leaf capacity given to BarnesHutForceCalculator.
constexpr int MAX_NODES = 1000000;
constexpr int MAX_PARTICLES = 1000000;
constexpr int LEAF_CAPACITY = 8;
constexpr int MAX_DEPTH = 10;
constexpr double EPSILON = 1e-9;
constexpr int BLOCK_SIZE = 256;
constexpr int TILE_SIZE = BLOCK_SIZE;
} // namespace constant
