// kernel_dispatcher.h - the plugin API of the step pipeline.
//
// Same types and lookup rule as the reference (sim/kernel_dispatcher.h:11-36,
// sim/phase_pipeline.h:12): launchers are registered per (PhaseType,
// halfPos, halfVel, compact) and looked up with the fallback halfVel ->
// halfPos.  Unlike the reference, where InitializeKernelDispatcher
// (sim/kernel_dispatcher.cpp:77) is never called, the dispatcher is live:
// every phase of sim::Simulator fetches its launcher from it, so a
// registered launcher replaces the built-in GB300 kernel for that phase.
#pragma once

#include <cstddef>
#include <unordered_map>

#include "device_buffers.h"
#include "parameters.h"

namespace sim {

enum class PhaseType { Integrate, GridBuild, SortPairs, CellRanges, SolveIterations, Velocity, Post };

struct KernelVariant {
    bool halfPos = false;
    bool halfVel = false;
    bool compact = false;
};

using KernelLaunchFn = void (*)(DeviceBuffers&, GridBuffers&, const SimParams&, cudaStream_t);

struct KernelKey {
    PhaseType phase;
    bool halfPos;
    bool halfVel;
    bool compact;
    bool operator==(const KernelKey& o) const {
        return phase == o.phase && halfPos == o.halfPos && halfVel == o.halfVel && compact == o.compact;
    }
};

struct KernelKeyHash {
    size_t operator()(const KernelKey& k) const {
        return (size_t(k.phase) * 131u) ^ (k.halfPos ? 0x1u : 0u) ^ (k.halfVel ? 0x2u : 0u) ^ (k.compact ? 0x4u : 0u);
    }
};

class KernelDispatcher {
public:
    void registerKernel(PhaseType ph, bool halfPos, bool halfVel, bool compact, KernelLaunchFn fn) {
        m_map[{ph, halfPos, halfVel, compact}] = fn;
    }
    KernelLaunchFn find(const KernelVariant& v, PhaseType ph) const {
        auto it = m_map.find(KernelKey{ph, v.halfPos, v.halfVel, v.compact});
        if (it != m_map.end()) return it->second;
        it = m_map.find(KernelKey{ph, v.halfPos, false, v.compact});
        if (it != m_map.end()) return it->second;
        it = m_map.find(KernelKey{ph, false, false, v.compact});
        if (it != m_map.end()) return it->second;
        return nullptr;
    }

private:
    std::unordered_map<KernelKey, KernelLaunchFn, KernelKeyHash> m_map;
};

// Registers the fused GB300 launchers for every phase, dense and compact.
void InitializeKernelDispatcher(KernelDispatcher& kd);

}  // namespace sim
