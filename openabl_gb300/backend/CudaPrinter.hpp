// Printer of the `-b cuda` backend.
//
// Derives from the reference `c` backend's printer (src/backend/CPrinter.hpp)
// so that every expression and statement is printed by the reference's own
// rules -- operator forms, vector operation names, literal precision, casts --
// and therefore evaluates with the same C semantics on the device.  It
// overrides only what changes on the GPU:
//   * globals are fields of a struct `G` handed to kernels and functions
//     (instead of C globals);
//   * a step function becomes a __device__ body plus a kernel over agents;
//     its `near` loop walks the runtime's binned grid (abl_device.cuh) instead
//     of every agent (CPrinter.cpp:148-173);
//   * `simulate` hands the population to the device runtime
//     (instead of CPrinter.cpp:189-233);
//   * the generated file also carries the model descriptor of
//     openabl_gb300/csrc/abl_model.h.
#pragma once

#include <map>
#include <set>
#include <string>
#include <vector>

#include "CPrinter.hpp"

namespace OpenABL {

struct CudaPrinter : public CPrinter {
  using CPrinter::print;

  CudaPrinter(AST::Script &script, bool useFloat, const std::string &modelName,
              bool deviceInit = false, long seed = 0)
    : CPrinter(script, useFloat), script(script), useFloat(useFloat), modelName(modelName),
      deviceInit(deviceInit), seed(seed) {}

  void print(const AST::VarExpression &) override;
  void print(const AST::CallExpression &) override;
  void print(const AST::AgentCreationExpression &) override;
  void print(const AST::ForStatement &) override;
  void print(const AST::IfStatement &) override;
  void print(const AST::WhileStatement &) override;
  void print(const AST::BreakStatement &) override;
  void print(const AST::SimulateStatement &) override;
  void print(const AST::VarDeclarationStatement &) override;
  void print(const AST::AssignOpStatement &) override;
  void print(const AST::MemberAccessExpression &) override;
  void print(const AST::FunctionDeclaration &) override;
  void print(const AST::Script &) override;

private:
  AST::Script &script;
  bool useFloat;
  std::string modelName;
  bool deviceInit;
  long seed;  // -C cuda.seed: key of random() in steps (abl_set_seed)

public:
  // Runtime settings the generated main() applies before simulating
  // (-C cuda.near_mode, cuda.near_cache, cuda.balance); -1: the default.
  int nearMode = -1, nearCache = -1, balance = -1;
  // -C cuda.precision=mixed: near-loop sums of neighbour members in FP32,
  // everything else in FP64 (an FP64 build only).
  bool mixed = false;

private:

  // Device initialisation: main()'s add() loops run as kernels.
  struct DevInit {
    const AST::ForStatement *loop = nullptr;
    const AST::AgentCreationExpression *create = nullptr;
    int agentType = -1;
  };
  std::vector<DevInit> devInit;
  void findDeviceInit(const AST::FunctionDeclaration &mainDecl);
  void printDeviceInit();
  std::map<const AST::FunctionDeclaration *, bool> hostOnlyMemo;
  bool hostOnlyFunction(const AST::FunctionDeclaration *f, int depth);

  // Near-loop printing state.
  int nearCounter = 0;
  int nearLoopDepth = -1;        // loop depth inside the current near body
  bool nearNeedsEnd = false;     // a `break` left the current near body
  std::string nearEndLabel;
  // Distances in the current near body that are only compared with
  // loop-invariant values (printed as abl::lazy_dist).
  std::set<const AST::VarDeclarationStatement *> lazyDecls;
  std::string nearQuery, nearSlot;
  // Conditional blocks of the current near body run in a second pass over
  // each chunk, and the per-chunk mask that records where their condition held.
  std::map<const AST::IfStatement *, std::string> deferredMasks;
  // Printing the second pass: declarations are printed with their exact value.
  bool deferredPass = false;
  // Mixed precision: the current near body's accumulations `acc += nx.m`
  // that run in FP32, by statement, with the name of their FP32 accumulator.
  struct MixedAcc {
    const AST::AssignOpStatement *stmt = nullptr;
    std::string acc;     // the FP32 accumulator (abl::facc)
    int member = -1;     // index of the neighbour member
    bool isPos = false;  // summed as offsets from the querying position
    int comps = 1;
  };
  std::map<const AST::AssignOpStatement *, MixedAcc> mixedAccs;
  std::string mixedAnchor;
  // Neighbour members read from their column where used instead of loaded
  // ahead (member -> column), for the loop variable `nearVar`.
  std::map<std::string, int> columnOnly;
  VarId nearVar;
  std::vector<MixedAcc> findMixedAccs(const AST::ForStatement &loop,
                                      const AST::AgentDeclaration &nearAgent);

  // Kind of function being printed (decides how builtins are lowered).
  enum class FnKind { HOST, STEP, USER, SEQ } fnKind = FnKind::HOST;
  // `out` starts as a copy of `in` in models with runtime add/remove.
  bool copyOut() const { return script.usesRuntimeRemoval || script.usesRuntimeAddition; }

  // Per step function, filled while printing it.
  struct StepInfo {
    const AST::FunctionDeclaration *decl = nullptr;
    int agentType = -1;
    int nearType = -1;
    bool ordered = true;
    unsigned nearMembers = 0;
    unsigned outMaybe = 0;
    unsigned outAlways = 0;
    unsigned outChanged = 0;   // members written with anything but `out.m = in.m`
    bool nearCacheable = false;  // one near loop, centred on the step's own agent
    const AST::ForStatement *nearLoop = nullptr;
    // The near radius names a step-local variable declared at the top of the
    // step with an initialiser of globals and never assigned: its value.
    const AST::VarDeclarationStatement *radiusLocal = nullptr;
    bool usesRemove = false;
    int addType = -1;
    bool usesRng = false;
    // Mixed precision: neighbour members summed from float copies, and
    // whether position offsets are summed (the position's low part).
    unsigned nearMembersF32 = 0;
    bool nearPosLo = false;
    // The step's only near loop is ordered and iterates around the step's own
    // agent: the kernel gathers and sorts neighbour lists per block.
    bool presorted = false;
  };
  std::vector<StepInfo> steps;

  bool isGlobal(const AST::Var &var) const;
  int agentIndex(const AST::AgentDeclaration *decl) const;
  std::string cType(Type t);
  void printGlobals();
  void printStepFunction(const AST::FunctionDeclaration &decl);
  void printKernel(const StepInfo &info);
  void printNearRadius(const StepInfo &info);
  void printPresortPhase(const StepInfo &info, const std::string &view, const std::string &pos);
  void printDescriptor();
  bool ensembleStep(const StepInfo &s) const;
  bool ensembleModel() const;
  void printPersistentKernel();
  void printHostSimulate();
  void printUserFunction(const AST::FunctionDeclaration &decl);
  void printSeqStep(const AST::FunctionDeclaration &decl);
  int memberIndex(const AST::AgentDeclaration *agent, const AST::AgentMember *member) const;
  // Calls whose arguments draw random numbers are printed with a fixed
  // (last to first) argument evaluation order.
  bool mayDraw(const AST::Node &e);
  bool printSequencedCall(const AST::CallExpression &expr);
  std::map<const AST::FunctionDeclaration *, bool> drawsMemo;
  int sequencedCounter = 0;
  const AST::FunctionDeclaration *seqStep = nullptr;
};

}  // namespace OpenABL
