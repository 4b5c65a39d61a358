// The `-b cuda` backend: a plugin for the reference compiler's backend
// interface (src/backend/Backend.hpp:33-36, registered by name like the
// entries of src/main.cpp:133-141).
#pragma once

#include "backend/Backend.hpp"

namespace OpenABL {

struct CudaBackend : public Backend {
  void generate(AST::Script &script, const BackendContext &ctx);
};

}
