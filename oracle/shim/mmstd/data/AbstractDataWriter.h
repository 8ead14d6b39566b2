// Minimal stand-in for MegaMol's AbstractDataWriter (plugins/mmstd/include/mmstd/data/AbstractDataWriter.h),
// oracle build only: a module whose pure virtual run() writes the data; Run() lets the harness trigger it,
// as the writer's "manualRun" button or a frontend job would.
#pragma once

#include "mmcore/Module.h"

namespace megamol::core {

class AbstractDataWriter : public Module {
public:
    bool Run() {
        return run();
    }

protected:
    virtual bool run() = 0;
};

} // namespace megamol::core
