/*
 * Empty conveyor header -- TEST INFRASTRUCTURE ONLY.
 * The reference headers include <convey.h>; the conveyor library is not
 * built for the oracle (it needs autotools code generation), and none of
 * the functions the oracle compiles use a conveyor type.
 */
#ifndef BALE_ORACLE_SHIM_CONVEY_H
#define BALE_ORACLE_SHIM_CONVEY_H
/* the real convey.h pulls these in, and spmat.h relies on them */
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#endif
