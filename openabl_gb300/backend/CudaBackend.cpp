#include "CudaBackend.hpp"

namespace OpenABL {

void CudaBackend::generate(AST::Script &, const BackendContext &) {
  throw BackendError("The cuda backend is not implemented yet");
}

}
