// The opaque handles of include/sparqc.h.
#pragma once
#include "sqc_batch.h"
#include "sqc_engine.h"
#include "sqc_part.h"
#include "sqc_serve.h"

struct sqc_state {
    sqc::Engine eng;
};

struct sqc_batch {
    sqc::Batch b;
};

struct sqc_server {
    sqc::Server s;
};

struct sqc_part_state {
    sqc::PartState p;
};
