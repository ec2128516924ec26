/*
 * Stand-in for the presolve library's PSLP_API.h (PSLP v0.0.4, fetched by the
 * reference's CMake and absent here).  LP/CP_AL/internal/presolve.h:4 includes
 * it for three names only: the Presolver and Settings handles, held as
 * pointers, and the status enumeration.  Presolve is never run by the
 * reference-solver build (ref_presolve_stub.c; every reference benchmark
 * passes --no_presolve), so opaque declarations suffice.
 */
#pragma once
typedef struct Presolver Presolver;
typedef struct Settings Settings;
enum PresolveStatus_ { PDAL_PRESOLVE_STUB_UNCHANGED = 0 };
