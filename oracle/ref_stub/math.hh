// Test infrastructure (oracle). Stand-in for the reference's src/core/math.hh:
// the FMM sources only call multipole_components (math.cc:99), defined in
// ref_glue.cc.
#pragma once
namespace libcppe {
int multipole_components(int k);
}
