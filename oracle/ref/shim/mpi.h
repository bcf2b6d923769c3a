/* Stand-in for mpi.h: dmrg_su2.cpp:2 includes it but makes no MPI call. */
#pragma once
