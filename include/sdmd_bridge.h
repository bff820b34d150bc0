/*
 * sdmd_bridge.h -- glue that hands the reference sDMD's own state to the engine
 * and back.  sdmd_gb300/bridge/sdmd_ref_bridge.c is compiled INTO the reference
 * (with its src/ on the include path): it reads and writes the reference's
 * globals (atom[], celllist, connectionMap, the potential tables, the counters,
 * glibc's rand() state) directly.  A maintainer calls sdmd_bridge_fill where
 * ThreadProcess() (src/ToolFunctions.c:12-20) would start the event loop, runs
 * the engine (include/sdmd_gpu.h), and calls sdmd_bridge_readback before the
 * reference's own writers (SaveData, src/DataSave.c:105-160) run.
 */
#ifndef SDMD_BRIDGE_H
#define SDMD_BRIDGE_H

#include "sdmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sdmd_bridge sdmd_bridge;   /* owns the arrays of one filled sdmd_system */

/* Fill *out from the reference's globals: the state after InputData() and
 * Prepare()'s set-up (SDEnergyMin, PBC, LinkList; src/SGThread.c:21-46), or any
 * later state of its loop.  Static data (masses, topology, the dense
 * connection map's BOND/CONSTRAINT bits as sparse rows, the pair tables) and the
 * dynamic state (positions, velocities, cells, types, HB state, events, the cell
 * list, the clock, counters and glibc's rand() state) are copied into arrays
 * owned by *owner.  Returns SDMD_OK, or SDMD_EUNSUPPORTED for a configuration the
 * engine does not cover (constraint atoms "_CONS", non-smooth walls). */
int  sdmd_bridge_fill(sdmd_system *out, sdmd_bridge **owner);

/* Write the dynamic state of s (positions, velocities, cells, types, HB and
 * HB-neighbour state with the connection map's HB / NEIGHBOR bits, events, the
 * cell list, the clock, the counters and the rand() state) back into the
 * reference's globals, for its writers or for its own loop to continue (continue
 * mode rebuilds the event tree, src/SGThread.c:54-62). */
int  sdmd_bridge_readback(const sdmd_system *s);

void sdmd_bridge_free(sdmd_bridge *b);

/* glibc's rand() state as the engine's sdmd_rng, and back (through
 * initstate()/setstate(), which share rand()'s generator). */
int  sdmd_bridge_get_rand(sdmd_rng *r);
int  sdmd_bridge_set_rand(const sdmd_rng *r);

#ifdef __cplusplus
}
#endif
#endif
