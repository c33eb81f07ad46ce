/*
 * Stand-in for modules/HostSolver/include/HostUTModel.hpp.
 *
 * Put include/standin ahead of the reference's HostSolver include directory
 * (and include/ on the path) and code that names HostSolver::HostUTModel --
 * e.g. applications/source/CaseRunners/WaterColumnModel.cpp:127-135 -- builds
 * the GB300 solver instead, without a source change (include/DeviceSolver.hpp).
 */
#pragma once
#include "DeviceSolver.hpp"

namespace HostSolver {
using HostUTModel = DeviceSolver::DeviceUTModel;
}
