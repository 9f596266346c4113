/* Compile-only stand-in: the reference includes "H5Cpp.h" (emulator/include/sim_parameters_types.h:37);
 * no HDF5 name is used by the headers on the gate path. TEST INFRASTRUCTURE ONLY. */
#pragma once
