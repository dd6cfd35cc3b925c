// Stand-in for the CMake-generated export header of libNeonSys (static build: no attributes).
#pragma once
#define LIBNEONSYS_EXPORT
