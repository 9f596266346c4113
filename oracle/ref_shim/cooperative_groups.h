/* Compile-only stand-in for a host build: the FC kernels only name the namespace
 * (emulator/device/device_table_FC.cuh:17-18). TEST INFRASTRUCTURE ONLY. */
#pragma once
namespace cooperative_groups {}
