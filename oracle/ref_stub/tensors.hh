// Test infrastructure (oracle). Stand-in for the reference's src/core/tensors.hh;
// calculate.cc includes it but uses nothing from it.
#pragma once
namespace libcppe {}
