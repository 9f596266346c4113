/* Compile-only stand-in: the reference includes <mpi.h> (emulator/include/sim_parameters_types.h:34)
 * but its gate path never calls MPI. TEST INFRASTRUCTURE ONLY. */
#pragma once
