/*
 * Forced-include shim for compiling the reference's CPU sources unmodified
 * (oracle/Makefile, target "ref").  TEST INFRASTRUCTURE ONLY.
 *
 * The reference's util/utility.h pulls in argparse (fetched from the network
 * by its CMake, absent here) and CUDA timers.  Defining its include guard
 * skips it; this header supplies what the CPU sources actually use from it:
 * the standard headers, config.h, log.h and the uint/ull typedefs
 * (util/utility.h:23-53).  <cstdint> is needed by cpu_bitruss.cpp:44
 * (UINT32_MAX).
 */
#pragma once
#define GPU_PLEX_UTILITY_H
#include <algorithm>
#include <atomic>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>
#include "util/config.h"
#include "util/log.h"
typedef unsigned int uint;
typedef unsigned long long int ull;
