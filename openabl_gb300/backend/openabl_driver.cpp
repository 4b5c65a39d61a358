// Compiler driver that adds the `cuda` backend to OpenABL.
//
// The reference driver (src/main.cpp) keeps its backend registry in
// getBackends() (src/main.cpp:133-141).  Registering a new backend there is a
// one-line change in the reference tree; this driver makes the same
// addition without editing the reference sources: the reference main.cpp is
// compiled with its `main` renamed to `openabl_reference_main`, every
// non-`cuda` invocation is handed to it unchanged, and `-b cuda` runs the same
// pipeline (src/main.cpp:170-316: parse main + lib, register builtins,
// analyse, generate, optionally build/run and print "Execution time: Xs")
// with CudaBackend.
#include <chrono>
#include <cstring>
#include <iostream>

#include "Cli.hpp"
#include "ParserContext.hpp"
#include "Analysis.hpp"
#include "AnalysisVisitor.hpp"
#include "FileUtil.hpp"
#include "backend/Backend.hpp"
#include "CudaBackend.hpp"

int openabl_reference_main(int argc, char **argv);

namespace OpenABL {
void registerBuiltinFunctions(FunctionList &funcs);
}

using namespace OpenABL;

static bool wantsCuda(int argc, char **argv) {
  for (int i = 1; i + 1 < argc; i++) {
    if ((!std::strcmp(argv[i], "-b") || !std::strcmp(argv[i], "--backend"))
        && !std::strcmp(argv[i + 1], "cuda")) {
      return true;
    }
  }
  return false;
}

static int runCuda(int argc, char **argv) {
  Cli::Options options;
  try {
    options = Cli::parseOptions(argc, argv);
  } catch (const Cli::OptionError &e) {
    std::cerr << "\nERROR: " << e.what() << std::endl;
    return 1;
  }

  FILE *mainFile = fopen(options.fileName.c_str(), "r");
  if (!mainFile) {
    std::cerr << "File \"" << options.fileName << "\" could not be opened." << std::endl;
    return 1;
  }
  if (!directoryExists(options.assetDir)) {
    std::cerr << "Asset directory \"" << options.assetDir << "\" does not exist "
              << "(override with -A or --asset-dir)" << std::endl;
    return 1;
  }
  std::string libFileName = options.assetDir + "/lib.abl";
  FILE *libFile = fopen(libFileName.c_str(), "r");
  if (!libFile) {
    std::cerr << "Library file \"" << libFileName << "\" could not be opened." << std::endl;
    return 1;
  }

  ParserContext mainCtx(mainFile);
  ParserContext libCtx(libFile);
  if (!mainCtx.parse() || !libCtx.parse()) {
    return 1;
  }

  int numErrors = 0;
  ErrorStream err([&numErrors](const Error &e) {
    std::cerr << e.msg << " on line " << e.loc.begin.line << std::endl;
    numErrors++;
  });

  FunctionList funcs;
  registerBuiltinFunctions(funcs);
  AnalysisVisitor visitor(*mainCtx.script, options.params, err, funcs, options.backend);
  visitor.handleLibScript(*libCtx.script);
  visitor.handleMainScript(*mainCtx.script);
  if (numErrors > 0) return 1;
  if (options.lintOnly) return 0;

  if (!options.outputDir.empty()) {
    createDirectory(options.outputDir);
  } else if (options.build || options.run) {
    options.outputDir = createTemporaryDirectory();
    std::cout << "Writing to directory " << options.outputDir << std::endl;
  } else {
    std::cerr << "Missing output directory (-o or --output-dir)" << std::endl;
    return 1;
  }
  options.depsDir = getAbsolutePath(options.depsDir);

  CudaBackend backend;
  BackendContext ctx = {
    options.outputDir, options.assetDir, options.depsDir, Config { options.config }
  };
  try {
    backend.generate(*mainCtx.script, ctx);
  } catch (const BackendError &e) {
    std::cerr << e.what() << std::endl;
    return 2;
  } catch (const std::runtime_error &e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }

  if (options.build || options.run) {
    changeWorkingDirectory(options.outputDir);
    backend.initEnv(ctx);
    if (!executeCommand("./build.sh")) {
      std::cerr << "Build failed" << std::endl;
      return 1;
    }
    if (options.run) {
      auto start = std::chrono::high_resolution_clock::now();
      if (!executeCommand("./run.sh")) {
        std::cerr << "Run failed" << std::endl;
        return 1;
      }
      auto end = std::chrono::high_resolution_clock::now();
      auto msecs = std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count();
      std::cout << "Execution time: " << msecs / 1000.0 << "s" << std::endl;
    }
  }
  fclose(mainFile);
  return 0;
}

int main(int argc, char **argv) {
  if (wantsCuda(argc, argv)) return runCuda(argc, argv);
  return openabl_reference_main(argc, argv);
}
