/*
 * Stand-in for the reference's Math/nUtil.h when its kinematics sources are
 * compiled for the oracle (oracle/Makefile, target "ref").  The reference header
 * pulls in torch; the kinematics code (cConformation.cpp) and the PDB reader
 * (cPDBLoader.cpp) only need the helpers declared here, which
 * oracle/ref_wrap.cpp implements.  Test
 * infrastructure only.
 */
#pragma once
#include <string>
#include <sys/types.h>

namespace StringUtil {
std::string string_format(const std::string fmt, ...);
std::string trim(const std::string &s);
}
namespace ProtUtil {
std::string convertRes1to3(char resName);
bool isHeavyAtom(std::string &atom_name);
}
