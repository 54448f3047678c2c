/* Stand-in for the Win32 header the reference's COMMON_DEFINITION.h includes.
   The headless oracle build uses nothing from it. */
#pragma once
