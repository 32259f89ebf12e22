/* Replaces the CMake-generated configuration header for the oracle build:
 * MPI on (single-rank stand-in), CUDA off, double precision. */
#pragma once
#include <vector>
#include <iostream>
#include <sstream>
#include <fstream>
#include <string>
#define ALSVINN_HAS_CONFIG 1
#define ALSVINN_MAJOR_VERSION 0
#define ALSVINN_MINOR_VERSION 0
#define ALSVINN_PATCH_VERSION 0
#define ALSVINN_USE_MPI 1
namespace alsutils {
std::string getAlsvinnVersion();
void dumpInformationToLog();
}
