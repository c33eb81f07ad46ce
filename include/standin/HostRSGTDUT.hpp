/*
 * Stand-in for modules/HostSolver/include/HostRSGTDUT.hpp.
 *
 * Put include/standin ahead of the reference's HostSolver include directory
 * (and include/ on the path) and code that names HostSolver::HostRSGTDUT --
 * e.g. applications/source/CaseRunners/TransducerModel.cpp:99-105 -- builds
 * the GB300 solver instead, without a source change.  The constructors,
 * makeShared, solve() and getStates() keep the reference's signatures
 * (include/DeviceSolver.hpp).
 */
#pragma once
#include "DeviceSolver.hpp"

namespace HostSolver {
using HostRSGTDUT = DeviceSolver::DeviceRSGTDUT;
}
