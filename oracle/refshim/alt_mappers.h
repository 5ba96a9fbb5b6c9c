// alt_mappers.h -- stand-in for the runtime header of the same name that
// apps/circuit/circuit.cc includes.  circuit.cc defines its own mappers and
// uses nothing from this header beyond legion.h.  TEST INFRASTRUCTURE ONLY.
#ifndef CKT_REFSHIM_ALT_MAPPERS_H
#define CKT_REFSHIM_ALT_MAPPERS_H
#include "legion.h"
#endif
