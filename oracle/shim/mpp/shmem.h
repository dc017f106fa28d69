/* Single-PE OpenSHMEM stand-in (test infrastructure only): the reference also includes <mpp/shmem.h>. */
#include "../shmem.h"
