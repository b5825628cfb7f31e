// Single-rank stand-in for the two MPI names the reference touches. Oracle build only.
#pragma once
typedef int MPI_Datatype;
#define MPI_DOUBLE_COMPLEX 0
