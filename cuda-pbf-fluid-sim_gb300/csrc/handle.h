// handle.h - the opaque pbf_sim handle of the C ABI (shared by the
// translation units that implement pbf_* functions on it).
#pragma once

#include "../../include/pbf/simulator.h"

struct pbf_sim {
    sim::Simulator sim;
};
