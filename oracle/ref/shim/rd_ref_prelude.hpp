/* Force-included before every translation unit of the headless reference build.
 * utils.h:138-154 uses std::unordered_map, std::array and assert without
 * including them, and assigns high_resolution_clock::now() to a steady_clock
 * time_point, which only compiles where the two clocks are the same type
 * (MSVC).  <chrono> is included first so that the macro below renames only the
 * reference's uses. */
#pragma once
#include <array>
#include <cassert>
#include <chrono>
#include <sstream>
#include <string>
#include <unordered_map>
#define high_resolution_clock steady_clock
