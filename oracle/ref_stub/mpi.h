/* Empty stand-in for <mpi.h>. The reference's include/common.h:12 includes
 * <mpi.h> unconditionally, but its serial and OpenMP sources call no MPI
 * function, so an empty header is enough to compile them. Oracle use only. */
#pragma once
