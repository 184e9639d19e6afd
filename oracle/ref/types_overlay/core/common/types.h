// Overlay of the reference's core/common/types.h used only when the
// reference's kernel is compiled for the CPU oracle (TEST INFRASTRUCTURE).
// Same constants as the reference (core/common/types.h:6-16) except the
// candidate cap, which becomes a runtime value so that the oracle can size the
// buffer and never truncate (the reference abandons a thread's remaining rows
// once 65,536 candidates are reached, global_func.cuh:172-173).
#ifndef HYPERBLOCKER_CORE_COMMON_TYPES_H_
#define HYPERBLOCKER_CORE_COMMON_TYPES_H_

#include <climits>

#define EQUALITIES 'e'
#define SIM 's'

extern int hbref_candidate_capacity;
#define MAX_CANDIDATE_COUNT (hbref_candidate_capacity)
#define MAX_EID_COL_SIZE 64

#define CHECK_POINT INT_MAX
#define CHECK_POINT_CHAR ' '

#define MAX_HASH_TIMES 1

#endif  // HYPERBLOCKER_CORE_COMMON_TYPES_H_
