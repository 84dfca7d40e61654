// tsph_system.h -- the handle behind tsph_system* (shared by the API units).
#pragma once

#include <memory>

#include "../../include/tsph.h"
#include "tsph_engine.h"

struct tsph_system {
    tsph::HostSetup hs;
    int precision = TSPH_PREC_FP32;
    void *stream = nullptr;
    std::unique_ptr<tsph::EngineBase> eng;
    bool divided = false;
    bool stale_engine = true;  // host particle list changed since the engine was built
    bool profiling = false;
};
