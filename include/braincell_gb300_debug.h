/*
 * braincell_gb300 -- tuning diagnostics.  Not part of the stable C ABI of
 * braincell_gb300.h: these entry points exist for kernel tuning, may change
 * between versions, and a drop-in integration should not bind them.
 */
#ifndef BRAINCELL_GB300_DEBUG_H
#define BRAINCELL_GB300_DEBUG_H

#include "braincell_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Cycles summed over CTAs (as seen by each CTA's first thread) in forward
 * elimination, back-substitution, node update and probes/pulses.  Only a library
 * compiled with -DBC_PHASE_TIMERS records them; otherwise all zero.  reset != 0
 * clears the counters after reading them. */
bc_status bc_debug_phase_cycles(bc_plan_t plan, uint64_t* out4, int32_t reset);

#ifdef __cplusplus
}
#endif
#endif /* BRAINCELL_GB300_DEBUG_H */
