/*
 * Stand-in for <TH/TH.h>, which Layers/FullAtomModel/cPDBLoader.h includes and which
 * torch 2.x no longer ships.  cPDBLoader.cpp uses nothing of TH itself, only
 * std::numeric_limits, which the real header brought in transitively.  Test
 * infrastructure only (oracle/Makefile, target "ref").
 */
#pragma once
#include <limits>
