// Stand-in for the CMake-generated export header of libNeonCore (static build: no attributes).
#pragma once
#define LIBNEONCORE_EXPORT
