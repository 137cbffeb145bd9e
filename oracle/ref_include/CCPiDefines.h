// Project-written replacement for the header the reference's CMake generates
// from Core/CCPiDefines.h.in. TEST INFRASTRUCTURE ONLY (oracle build).
#pragma once
#define CCPI_EXPORT
#define EXPIMP_TEMPLATE
#define VERSION "reference-oracle"
#define REV_DATE "unknown"
