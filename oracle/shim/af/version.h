/* Version macros for compiling the reference's CPU kernel headers in place.
 * The reference generates this header at configure time; the values below
 * name the reference release the oracle was built against (v3.10.0). */
#pragma once
#define AF_VERSION "3.10.0"
#define AF_VERSION_MAJOR 3
#define AF_VERSION_MINOR 10
#define AF_VERSION_PATCH 0
#define AF_API_VERSION_CURRENT 310
