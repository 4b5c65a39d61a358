// `-b cuda`: writes <model>.cu (kernels, model descriptor and the host
// main()), the device runtime, build.sh and run.sh into the output directory,
// the same layout the `c` backend produces (src/backend/CBackend.cpp:29-45).
//
// Configuration (-C name=value):
//   use_float=true         abl_float is float (as LIBABL_USE_FLOAT for `c`)
//   cuda.model=NAME        identifier of the model inside the runtime (default "model")
//   cuda.device_init=true  main()'s add() loops run as kernels (CudaPrinter::findDeviceInit)
//   cuda.seed=N            key of the counter-based random() stream in steps (default 0)
//   cuda.near_mode=M       how ordered near loops gather neighbours: auto, runs, rows,
//                          lists or block (abl_set_near_mode; results are identical)
//   cuda.near_cache=B      keep neighbour lists of agents that never move (default true)
//   cuda.balance=B         hand a block's agents to threads by neighbour count (default true)
//   cuda.precision=P       double (default): the reference's arithmetic, bit for bit;
//                          mixed: near-loop sums of neighbour members in FP32, the
//                          rest FP64 (CudaPrinter::findMixedAccs)
#include "CudaBackend.hpp"

#include <cctype>
#include <sstream>

#include "CudaPrinter.hpp"
#include "FileUtil.hpp"

#ifndef ABL_CUDA_RUNTIME_DIR
#define ABL_CUDA_RUNTIME_DIR ""
#endif
#ifndef ABL_CUDA_INCLUDE_DIR
#define ABL_CUDA_INCLUDE_DIR ""
#endif

namespace OpenABL {

static const char *kRuntimeFiles[] = {
  "abl_runtime.cu", "abl_host.cpp", "abl_host.h", "abl_model.h", "abl_device.cuh",
  "abl_math.cuh", "abl_gen.cuh", "abl_bin.cuh", "abl_persist.cuh",
};

static std::string runtimeDir(const BackendContext &ctx) {
  // The runtime ships as asset/cuda in an OpenABL tree; a build of this
  // plugin outside such a tree points at its own copy.
  std::string assetCuda = ctx.assetDir + "/cuda";
  if (fileExists(assetCuda + "/abl_runtime.cu")) return assetCuda;
  return ABL_CUDA_RUNTIME_DIR;
}

// The folded globals as the printers emit them (literals printed with the
// stream's default six significant digits, src/backend/GenericPrinter.cpp:39-58),
// so that hosts driving the runtime directly can reproduce a configuration.
static std::string literalText(const AST::Expression &e) {
  std::ostringstream s;
  if (auto *f = dynamic_cast<const AST::FloatLiteral *>(&e)) {
    s << f->value;
  } else if (auto *i = dynamic_cast<const AST::IntLiteral *>(&e)) {
    s << i->value;
  } else if (auto *b = dynamic_cast<const AST::BoolLiteral *>(&e)) {
    s << (b->value ? "true" : "false");
  } else if (auto *c = dynamic_cast<const AST::CallExpression *>(&e)) {
    s << "[";
    for (size_t k = 0; k < c->args->size(); k++) {
      s << (k ? ", " : "") << literalText(*(*c->args)[k]);
    }
    s << "]";
  } else {
    s << "null";
  }
  return s.str();
}

static std::string globalsManifest(const AST::Script &script, const std::string &model) {
  std::ostringstream s;
  s << "{\"model\": \"" << model << "\", \"globals\": {";
  bool first = true;
  for (const AST::ConstDeclaration *decl : script.consts) {
    if (decl->isArray) continue;
    s << (first ? "" : ", ") << "\"" << decl->var->name << "\": " << literalText(*decl->expr);
    first = false;
  }
  s << "}}\n";
  return s.str();
}

void CudaBackend::generate(AST::Script &script, const BackendContext &ctx) {
  bool useFloat = ctx.config.getBool("use_float", false);
  std::string model = "model";
  auto it = ctx.config.config.find("cuda.model");
  if (it != ctx.config.config.end()) model = it->second;
  for (char ch : model) {
    if (!(std::isalnum((unsigned char) ch) || ch == '_')) {
      throw BackendError("cuda.model must be an identifier");
    }
  }

  CudaPrinter printer(script, useFloat, model, ctx.config.getBool("cuda.device_init", false),
                      ctx.config.getInt("cuda.seed", 0));
  auto mode = ctx.config.config.find("cuda.near_mode");
  if (mode != ctx.config.config.end()) {
    static const char *const kModes[] = {"auto", "runs", "rows", "lists", "block"};
    for (int k = 0; k < 5; k++)
      if (mode->second == kModes[k]) printer.nearMode = k;
    if (printer.nearMode < 0)
      throw BackendError("cuda.near_mode must be auto, runs, rows, lists or block");
  }
  if (ctx.config.config.count("cuda.near_cache"))
    printer.nearCache = ctx.config.getBool("cuda.near_cache", true) ? 1 : 0;
  if (ctx.config.config.count("cuda.balance"))
    printer.balance = ctx.config.getBool("cuda.balance", true) ? 1 : 0;
  auto prec = ctx.config.config.find("cuda.precision");
  if (prec != ctx.config.config.end()) {
    if (prec->second == "mixed") {
      if (useFloat) throw BackendError("cuda.precision=mixed needs the FP64 build (use_float=false)");
      printer.mixed = true;
    } else if (prec->second != "double") {
      throw BackendError("cuda.precision must be double or mixed");
    }
  }
  printer.print(script);
  writeToFile(ctx.outputDir + "/" + model + ".cu", printer.extractStr());
  writeToFile(ctx.outputDir + "/" + model + ".globals.json", globalsManifest(script, model));

  std::string rt = runtimeDir(ctx);
  for (const char *f : kRuntimeFiles) {
    std::string src = rt + "/" + f;
    if (!fileExists(src)) throw std::runtime_error("cuda runtime file missing: " + src);
    copyFile(src, ctx.outputDir + "/" + f);
  }
  for (const char *h : {"openabl_cuda.h", "openabl_cuda_diag.h"}) {
    std::string header = fileExists(rt + "/" + h) ? rt + "/" + h
                                                  : std::string(ABL_CUDA_INCLUDE_DIR) + "/" + h;
    copyFile(header, ctx.outputDir + "/" + h);
  }
  // The model file is compiled twice: once for its per-phase kernels, host
  // code and main(), once with ABL_PERSIST for its persistent ensemble
  // kernel (plain loads instead of read-only ones, abl_device.cuh).
  const std::string nvcc = "nvcc -gencode arch=compute_103a,code=sm_103a -O3 -fmad=false "
                           "-Xcompiler -ffp-contract=off -std=c++17 -diag-suppress 177 -I. ";
  writeToFile(ctx.outputDir + "/build.sh",
              nvcc + "-DABL_PERSIST -x cu -c " + model + ".cu -o " + model + ".persist.o && \\\n" +
              nvcc + "-DABL_STANDALONE_MAIN " + model + ".cu abl_runtime.cu abl_host.cpp " +
              model + ".persist.o -o main\n");
  writeToFile(ctx.outputDir + "/run.sh", "./main\n");
  makeFileExecutable(ctx.outputDir + "/build.sh");
  makeFileExecutable(ctx.outputDir + "/run.sh");
}

}  // namespace OpenABL
