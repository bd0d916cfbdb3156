// Handle types behind the opaque pointers of include/sus2g.h (shared by the C ABI translation units).
#pragma once
#include <memory>

#include "engine.h"
#include "model.h"

struct sus2g_model_s {
  sus2g::Model model;
};
struct sus2g_engine_s {
  std::unique_ptr<sus2g::Engine> engine;
  int launches = 0;
};

// Sets the thread's message returned by sus2g_last_error (library-internal, not exported in the ABI header).
void sus2g_set_last_error(const char* message);
