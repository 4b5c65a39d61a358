#include "CudaPrinter.hpp"

#include <functional>
#include <map>
#include <sstream>

#include "ASTVisitor.hpp"
#include "backend/Backend.hpp"

namespace OpenABL {

namespace {

// Root variable of an assignment target (`x`, `x.m`, `x.m.c`, `x[i]`).
const AST::VarExpression *targetRoot(const AST::Expression &e) {
  if (auto *v = dynamic_cast<const AST::VarExpression *>(&e)) return v;
  if (auto *m = dynamic_cast<const AST::MemberAccessExpression *>(&e)) return targetRoot(*m->expr);
  if (auto *a = dynamic_cast<const AST::ArrayAccessExpression *>(&e)) return targetRoot(*a->arrayExpr);
  return nullptr;
}

// Member of `var` named by an assignment target `var.m[...]`, or "" for the
// whole variable.
std::string targetMember(const AST::Expression &e) {
  const AST::Expression *cur = &e;
  std::string last;
  while (true) {
    if (auto *m = dynamic_cast<const AST::MemberAccessExpression *>(cur)) {
      last = m->member;
      cur = &*m->expr;
    } else if (auto *a = dynamic_cast<const AST::ArrayAccessExpression *>(cur)) {
      cur = &*a->arrayExpr;
    } else {
      return last;
    }
  }
}

bool isHostOnlyBuiltin(const std::string &name) {
  return name == "random" || name == "randomInt" || name == "add" || name == "save"
      || name == "removeCurrent" || name == "count" || name == "sum" || name == "log_csv"
      || name == "getLastExecTime";
}

// Collects calls, loops and assignments below a node.
struct Collector : public AST::Visitor {
  std::vector<const AST::CallExpression *> calls;
  std::vector<const AST::ForStatement *> nearLoops;
  std::vector<const AST::AssignStatement *> assigns;
  std::vector<const AST::AssignOpStatement *> assignOps;
  std::vector<const AST::VarExpression *> varExprs;
  std::vector<const AST::VarDeclarationStatement *> decls;
  std::vector<const AST::ForStatement *> fors;
  std::vector<const AST::MemberAccessExpression *> members;
  int breaks = 0, returns = 0, continues = 0, whiles = 0;

  void enter(AST::CallExpression &e) override { calls.push_back(&e); }
  void enter(AST::ForStatement &s) override {
    fors.push_back(&s);
    if (s.isNear()) nearLoops.push_back(&s);
  }
  void enter(AST::AssignStatement &s) override { assigns.push_back(&s); }
  void enter(AST::AssignOpStatement &s) override { assignOps.push_back(&s); }
  void enter(AST::VarExpression &e) override { varExprs.push_back(&e); }
  void enter(AST::VarDeclarationStatement &s) override { decls.push_back(&s); }
  void enter(AST::MemberAccessExpression &e) override { members.push_back(&e); }
  void enter(AST::BreakStatement &) override { breaks++; }
  void enter(AST::ReturnStatement &) override { returns++; }
  void enter(AST::ContinueStatement &) override { continues++; }
  void enter(AST::WhileStatement &) override { whiles++; }
};

template <typename N>
Collector collect(N &node) {
  Collector c;
  const_cast<typename std::remove_const<N>::type &>(node).accept(c);
  return c;
}

// Whether the result of a near body can depend on the order in which
// neighbours are visited.  Order-free bodies only accumulate integers into
// variables declared outside the loop with +=, -=, |=, &=, ^= and never read
// those variables otherwise; everything else is treated as order-dependent.
// `orderFree` lists further accumulations whose order does not matter (the
// mixed form's FP32 sums, which are not bit-exact to the reference in any
// order).
bool nearBodyIsOrdered(const AST::ForStatement &loop,
                       const std::set<const AST::AssignOpStatement *> *orderFree = nullptr) {
  Collector c = collect(*loop.stmt);
  if (c.breaks || c.returns) return true;
  std::set<VarId> inner;
  inner.insert(loop.var->id);
  for (auto *d : c.decls) inner.insert(d->var->id);
  for (auto *f : c.fors) inner.insert(f->var->id);
  for (auto *call : c.calls) {
    if (call->isBuiltin() && isHostOnlyBuiltin(call->name)) return true;
    if (call->kind == AST::CallExpression::Kind::USER) return true;
  }
  for (auto *a : c.assigns) {
    const AST::VarExpression *root = targetRoot(*a->left);
    if (!root || !inner.count(root->var->id)) return true;
  }
  std::map<VarId, int> accTargets;
  for (auto *a : c.assignOps) {
    const AST::VarExpression *root = targetRoot(*a->left);
    if (!root) return true;
    if (inner.count(root->var->id)) continue;
    if (orderFree && orderFree->count(a)) {
      accTargets[root->var->id]++;
      continue;
    }
    auto *plain = dynamic_cast<const AST::VarExpression *>(&*a->left);
    if (!plain) return true;
    Type t = a->left->type;
    bool okOp = a->op == AST::BinaryOp::ADD || a->op == AST::BinaryOp::SUB
             || a->op == AST::BinaryOp::BITWISE_OR || a->op == AST::BinaryOp::BITWISE_AND
             || a->op == AST::BinaryOp::BITWISE_XOR;
    if (!okOp || !(t.isInt() || t.isBool())) return true;
    accTargets[root->var->id]++;
  }
  std::map<VarId, int> uses;
  for (auto *v : c.varExprs) uses[v->var->id]++;
  for (auto &kv : accTargets) {
    if (uses[kv.first] != kv.second) return true;  // read somewhere besides its own update
  }
  return false;
}

// Whether every variable in `e` is a global and every call a builtin or a
// type constructor, i.e. `e` has one value for the whole near loop.
bool isLoopInvariant(const AST::Script &script, const AST::Expression &e) {
  Collector c = collect(*const_cast<AST::Expression *>(&e));
  for (auto *v : c.varExprs) {
    if (!script.scope.has(v->var->id) || !script.scope.get(v->var->id).isGlobal) return false;
  }
  for (auto *call : c.calls) {
    if (call->kind == AST::CallExpression::Kind::USER) return false;
    if (call->isBuiltin() && isHostOnlyBuiltin(call->name)) return false;
  }
  return true;
}

// `X.pos` for the given variable and position member.
bool isPosOf(const AST::Expression &e, VarId var, const std::string &pos) {
  auto *m = dynamic_cast<const AST::MemberAccessExpression *>(&e);
  if (!m || m->member != pos) return false;
  auto *v = dynamic_cast<const AST::VarExpression *>(&*m->expr);
  return v && v->var->id == var;
}

struct ComparisonCollector : public AST::Visitor {
  std::vector<const AST::BinaryOpExpression *> cmps;
  void enter(AST::BinaryOpExpression &e) override {
    switch (e.op) {
      case AST::BinaryOp::SMALLER: case AST::BinaryOp::SMALLER_EQUALS:
      case AST::BinaryOp::GREATER: case AST::BinaryOp::GREATER_EQUALS:
      case AST::BinaryOp::EQUALS: case AST::BinaryOp::NOT_EQUALS:
        cmps.push_back(&e);
        break;
      default:
        break;
    }
  }
};

// A conditional block of a near body run in a second pass over each chunk,
// with the body's declarations it reads, recomputed there.
struct DeferredIf {
  const AST::IfStatement *ifs = nullptr;
  std::vector<const AST::VarDeclarationStatement *> recompute;
};

// Declarations `float d = dist(q.pos, nx.pos)` (or length(q.pos - nx.pos),
// either order) inside a near body whose every use is a comparison with a
// loop-invariant value.
std::set<const AST::VarDeclarationStatement *> findLazyDistances(
    const AST::Script &script, const AST::ForStatement &loop,
    const std::vector<const AST::Statement *> &excluded) {
  std::set<const AST::VarDeclarationStatement *> out;
  auto *q = dynamic_cast<const AST::VarExpression *>(&loop.getNearAgent());
  if (!q) return out;
  VarId qid = q->var->id, nid = loop.var->id;
  const AST::AgentDeclaration *agent = loop.type->resolved.getAgentDecl();
  std::string pos = agent->getPositionMember()->name;
  Collector c = collect(*loop.stmt);
  ComparisonCollector cc;
  const_cast<AST::Statement &>(*loop.stmt).accept(cc);
  for (auto *d : c.decls) {
    if (!d->initializer || !d->type->resolved.isFloat()) continue;
    auto *call = dynamic_cast<const AST::CallExpression *>(&*d->initializer);
    if (!call || !call->isBuiltin()) continue;
    const std::string &fn = call->calledSig.name;
    const AST::Expression *a = nullptr, *b = nullptr;
    if ((fn == "dist_float2" || fn == "dist_float3") && call->args->size() == 2) {
      a = &*(*call->args)[0];
      b = &*(*call->args)[1];
    } else if ((fn == "length_float2" || fn == "length_float3") && call->args->size() == 1) {
      auto *sub = dynamic_cast<const AST::BinaryOpExpression *>(&*(*call->args)[0]);
      if (!sub || sub->op != AST::BinaryOp::SUB) continue;
      a = &*sub->left;
      b = &*sub->right;
    } else {
      continue;
    }
    bool pair = (isPosOf(*a, qid, pos) && isPosOf(*b, nid, pos))
             || (isPosOf(*a, nid, pos) && isPosOf(*b, qid, pos));
    if (!pair) continue;
    VarId id = d->var->id;
    int uses = 0, cmpUses = 0;
    auto count = [&](const Collector &cl, const ComparisonCollector &cmpc, int sign) {
      for (auto *v : cl.varExprs) uses += sign * (v->var->id == id);
      for (auto *cmp : cmpc.cmps) {
        auto *l = dynamic_cast<const AST::VarExpression *>(&*cmp->left);
        auto *r = dynamic_cast<const AST::VarExpression *>(&*cmp->right);
        if (l && l->var->id == id && isLoopInvariant(script, *cmp->right)) cmpUses += sign;
        else if (r && r->var->id == id && isLoopInvariant(script, *cmp->left)) cmpUses += sign;
      }
    };
    count(c, cc, 1);
    // Blocks run in the second pass recompute the value exactly; their uses
    // do not count here.
    for (const AST::Statement *e : excluded) {
      ComparisonCollector ec;
      const_cast<AST::Statement &>(*e).accept(ec);
      count(collect(*const_cast<AST::Statement *>(e)), ec, -1);
    }
    if (uses > 0 && uses == cmpUses) out.insert(d);
  }
  return out;
}

// Conditional accumulations that a near loop can run in a second pass.
//
// A top-level statement `if (C) B` (no else) of a near body qualifies when B
// only updates variables declared before the loop ("its accumulators") that
// nothing else in the body mentions, reads nothing but the neighbour, globals,
// its own locals and accumulators, and variables the body never writes, and
// has no calls other than pure builtins, no loops and no jumps; the body as a
// whole has no break or return.  Then running B for the iterations where C
// held, in the same ascending neighbour order but after the rest of the
// body's iterations over the same chunk, performs every accumulator's updates
// in the same order on the same values, so the results are identical.  The
// gain: B's instructions issue once per neighbour where C held in some lane,
// instead of once per neighbour where C held in any lane of the warp (e.g.
// boids2d's collision sum, which every lane hits at its own agent).  Only
// blocks that update floating-point accumulators are moved.
std::vector<DeferredIf> findDeferredIfs(const AST::Script &script,
                                        const AST::FunctionDeclaration *step,
                                        const AST::ForStatement &loop) {
  std::vector<DeferredIf> out;
  auto *block = dynamic_cast<const AST::BlockStatement *>(&*loop.stmt);
  if (!block || !step) return out;
  Collector body = collect(*loop.stmt);
  if (body.breaks || body.returns) return out;
  std::set<VarId> inner;  // declared inside the body, or the loop variable
  inner.insert(loop.var->id);
  for (auto *d : body.decls) inner.insert(d->var->id);
  for (auto *f : body.fors) inner.insert(f->var->id);
  std::set<VarId> params;
  for (const AST::ParamPtr &p : *step->params) params.insert(p->var->id);
  if (step->isParallelStep()) params.insert(step->stepParam().outVar->id);
  auto isGlobalVar = [&](VarId id) {
    return script.scope.has(id) && script.scope.get(id).isGlobal;
  };
  std::map<VarId, int> bodyRefs;
  for (auto *v : body.varExprs) bodyRefs[v->var->id]++;
  std::set<VarId> bodyWritten;
  for (auto *a : body.assigns) {
    if (auto *r = targetRoot(*a->left)) bodyWritten.insert(r->var->id);
  }
  for (auto *a : body.assignOps) {
    if (auto *r = targetRoot(*a->left)) bodyWritten.insert(r->var->id);
  }
  // Top-level declarations of the body whose value the second pass can
  // recompute: never assigned, initialised from the neighbour, globals,
  // variables the body never writes and earlier such declarations only,
  // through pure builtins.
  std::map<VarId, const AST::VarDeclarationStatement *> recomputable;
  std::map<VarId, std::set<VarId>> recomputeDeps;
  for (const AST::StatementPtr &st : *block->stmts) {
    auto *d = dynamic_cast<const AST::VarDeclarationStatement *>(&*st);
    if (!d || !d->initializer || bodyWritten.count(d->var->id)) continue;
    Collector ic = collect(*d->initializer);
    bool pure = true;
    std::set<VarId> deps;
    for (auto *call : ic.calls) {
      if (call->kind == AST::CallExpression::Kind::USER) pure = false;
      if (call->isBuiltin() && isHostOnlyBuiltin(call->name)) pure = false;
    }
    for (auto *v : ic.varExprs) {
      VarId id = v->var->id;
      if (id == loop.var->id || isGlobalVar(id)) continue;
      if (recomputable.count(id)) {
        deps.insert(id);
        deps.insert(recomputeDeps[id].begin(), recomputeDeps[id].end());
        continue;
      }
      if (inner.count(id) || bodyWritten.count(id) || id == step->stepParam().outVar->id)
        pure = false;
    }
    if (!pure) continue;
    recomputable[d->var->id] = d;
    recomputeDeps[d->var->id] = deps;
  }
  for (const AST::StatementPtr &st : *block->stmts) {
    auto *ifs = dynamic_cast<const AST::IfStatement *>(&*st);
    if (!ifs || ifs->elseStmt) continue;
    Collector b = collect(*ifs->ifStmt);
    if (b.breaks || b.returns || b.continues || b.whiles || !b.fors.empty()) continue;
    bool ok = true, floatTarget = false;
    for (auto *call : b.calls) {
      if (call->kind == AST::CallExpression::Kind::USER) ok = false;
      if (call->isBuiltin() && isHostOnlyBuiltin(call->name)) ok = false;
    }
    std::set<VarId> local, targets;
    for (auto *d : b.decls) local.insert(d->var->id);
    auto noteTarget = [&](const AST::Expression &left) {
      const AST::VarExpression *r = targetRoot(left);
      if (!r) {
        ok = false;
        return;
      }
      VarId id = r->var->id;
      if (local.count(id)) return;
      if (inner.count(id) || params.count(id) || isGlobalVar(id) || left.type.isAgent()) {
        ok = false;
        return;
      }
      targets.insert(id);
      if (left.type.isFloat() || left.type.isVec()) floatTarget = true;
    };
    for (auto *a : b.assigns) noteTarget(*a->left);
    for (auto *a : b.assignOps) noteTarget(*a->left);
    if (!ok || targets.empty() || !floatTarget) continue;
    std::map<VarId, int> refs;
    for (auto *v : b.varExprs) refs[v->var->id]++;
    std::set<VarId> need;
    for (auto &kv : refs) {
      VarId id = kv.first;
      if (targets.count(id)) {
        if (bodyRefs[id] != kv.second) ok = false;  // mentioned elsewhere in the body
      } else if (id == loop.var->id || local.count(id) || isGlobalVar(id)) {
        // the neighbour, B's own locals, globals
      } else if (recomputable.count(id)) {
        need.insert(id);  // a per-iteration value the second pass recomputes
        need.insert(recomputeDeps[id].begin(), recomputeDeps[id].end());
      } else if (inner.count(id) || bodyWritten.count(id)) {
        ok = false;  // a per-iteration value of the rest of the body
      }
    }
    if (!ok) continue;
    DeferredIf di;
    di.ifs = ifs;
    // Recomputed declarations in body order; each must precede the if.
    for (const AST::StatementPtr &st2 : *block->stmts) {
      if (&*st2 == ifs) break;
      auto *d = dynamic_cast<const AST::VarDeclarationStatement *>(&*st2);
      if (d && need.count(d->var->id)) {
        di.recompute.push_back(d);
        need.erase(d->var->id);
      }
    }
    if (need.empty()) out.push_back(di);
  }
  return out;
}

}  // namespace

void CudaPrinter::print(const AST::VarDeclarationStatement &stmt) {
  if (lazyDecls.count(&stmt) && !deferredPass) {
    *this << "const auto " << *stmt.var << " = abl::make_lazy_dist(" << nearQuery
          << ", abl_NB, " << nearSlot << ", [&]() -> abl_float { return " << *stmt.initializer
          << "; });";
    return;
  }
  CPrinter::print(stmt);
}

bool CudaPrinter::isGlobal(const AST::Var &var) const {
  return script.scope.has(var.id) && script.scope.get(var.id).isGlobal;
}

int CudaPrinter::agentIndex(const AST::AgentDeclaration *decl) const {
  for (size_t k = 0; k < script.agents.size(); k++) {
    if (script.agents[k] == decl) return (int) k;
  }
  return -1;
}

std::string CudaPrinter::cType(Type t) {
  switch (t.getTypeId()) {
    case Type::BOOL: return "bool";
    case Type::INT32: return "int";
    case Type::FLOAT: return useFloat ? "float" : "double";
    case Type::VEC2: return "float2";
    case Type::VEC3: return "float3";
    default:
      throw BackendError("The cuda backend does not support agent members of this type");
  }
}

static const char *ablTypeId(Type t) {
  switch (t.getTypeId()) {
    case Type::BOOL: return "ABL_T_BOOL";
    case Type::INT32: return "ABL_T_INT";
    case Type::FLOAT: return "ABL_T_FLOAT";
    case Type::VEC2: return "ABL_T_FLOAT2";
    case Type::VEC3: return "ABL_T_FLOAT3";
    default: return "0";
  }
}

void CudaPrinter::print(const AST::VarExpression &expr) {
  if (isGlobal(*expr.var)) {
    *this << "abl_G." << expr.var->name;
    return;
  }
  CPrinter::print(expr);
}

int CudaPrinter::memberIndex(const AST::AgentDeclaration *agent,
                             const AST::AgentMember *member) const {
  for (size_t k = 0; k < agent->members->size(); k++) {
    if (&*(*agent->members)[k] == member) return (int) k;
  }
  return -1;
}

// Whether evaluating `e` can draw random numbers: a random()/randomInt() call
// in it, or a call of a user function that draws (directly or further down).
bool CudaPrinter::mayDraw(const AST::Node &e) {
  Collector c = collect(const_cast<AST::Node &>(e));
  for (auto *call : c.calls) {
    if (call->isBuiltin() && (call->name == "random" || call->name == "randomInt")) return true;
    if (call->kind != AST::CallExpression::Kind::USER || !call->calledFunc) continue;
    auto it = drawsMemo.find(call->calledFunc);
    if (it == drawsMemo.end()) {
      drawsMemo[call->calledFunc] = false;  // a recursive call draws nothing by itself
      bool d = mayDraw(*call->calledFunc);
      drawsMemo[call->calledFunc] = d;
      if (d) return true;
    } else if (it->second) {
      return true;
    }
  }
  return false;
}

// C leaves the evaluation order of function arguments unspecified, so a call
// like float2_create(random_float(..), random_float(..)) -- the expansion of
// random(float2 lo, float2 hi), asset/lib.abl -- draws its components in an
// order the C compiler picks.  The reference programs built with gcc on
// x86-64 evaluate arguments from last to first (the y component is drawn
// before x); the generated code fixes that order whenever two or more
// arguments can draw, so results do not depend on the host compiler or CPU.
bool CudaPrinter::printSequencedCall(const AST::CallExpression &expr) {
  const size_t n = expr.args->size();
  if (n < 2) return false;
  if (expr.isBuiltin() && (isHostOnlyBuiltin(expr.name) && expr.name != "random"
                           && expr.name != "randomInt")) {
    return false;
  }
  if (expr.isCtor() && !expr.type.isVec()) return false;
  int drawing = 0;
  for (const AST::ExpressionPtr &arg : *expr.args) drawing += mayDraw(*arg) ? 1 : 0;
  if (drawing < 2) return false;
  const std::string tmp = "abl_e" + std::to_string(++sequencedCounter) + "_";
  *this << "([&]() { ";
  for (size_t k = n; k-- > 0;) *this << "const auto " << tmp << k << " = " << *(*expr.args)[k] << "; ";
  *this << "return ";
  if (expr.isCtor()) {
    *this << "float" << expr.type.getVecLen() << "_create(";
  } else if (expr.kind == AST::CallExpression::Kind::USER) {
    *this << expr.calledSig.name << "(abl_G, abl_R, ";
  } else if (expr.name == "random" || expr.name == "randomInt") {
    *this << (expr.name == "random" ? "abl_random(abl_R, " : "abl_random_int(abl_R, ");
  } else {
    *this << expr.calledSig.name << "(";
  }
  for (size_t k = 0; k < n; k++) *this << (k ? ", " : "") << tmp << k;
  *this << "); }())";
  return true;
}

void CudaPrinter::print(const AST::CallExpression &expr) {
  if (printSequencedCall(expr)) return;
  if (expr.kind == AST::CallExpression::Kind::USER) {
    *this << expr.calledSig.name << "(abl_G, abl_R";
    for (const AST::ExpressionPtr &arg : *expr.args) *this << ", " << *arg;
    *this << ")";
    return;
  }
  if (expr.isBuiltin()) {
    const std::string &n = expr.name;
    if (n == "random" || n == "randomInt") {
      // Host: the reference's sequential stream; device: abl::rng.
      *this << (n == "random" ? "abl_random(abl_R" : "abl_random_int(abl_R");
      for (const AST::ExpressionPtr &arg : *expr.args) *this << ", " << *arg;
      *this << ")";
      return;
    }
    if (n == "removeCurrent") {
      // FlameGPU lowers it to a flag as well (FlameGPUPrinter.cpp:171-173).
      *this << "abl_K.remove()";
      return;
    }
    if (n == "add" && fnKind == FnKind::STEP) {
      const AST::AgentDeclaration *a = expr.calledSig.paramTypes[0].getAgentDecl();
      *this << "abl_add_" << a->name << "(abl_K, " << expr.getArg(0) << ")";
      return;
    }
    if (n == "count") {
      Type t = expr.getArg(0).type;
      const AST::AgentDeclaration *a = t.getAgentDecl();
      if (expr.getNumArgs() == 2) {
        const AST::AgentMember *m = t.getAgentMember();
        *this << "abl_seq_count_eq(abl_C, " << agentIndex(a) << ", " << memberIndex(a, m)
              << ", (" << cType(m->type->resolved) << ") " << expr.getArg(1) << ")";
      } else {
        *this << "abl_seq_count(abl_C, " << agentIndex(a) << ")";
      }
      return;
    }
    if (n == "sum") {
      Type t = expr.getArg(0).type;
      const AST::AgentDeclaration *a = t.getAgentDecl();
      const AST::AgentMember *m = t.getAgentMember();
      Type mt = m->type->resolved;
      std::string rt = mt.isBool() ? "int" : cType(mt);
      *this << "abl_seq_sum<" << rt << ">(abl_C, " << agentIndex(a) << ", " << memberIndex(a, m)
            << ")";
      return;
    }
    if (n == "getLastExecTime") {
      *this << "abl_seq_exec_time(abl_C)";
      return;
    }
    if (n == "log_csv") {
      // "%d" / "%f" per argument, comma separated (FlameGPUPrinter.cpp:226-245).
      std::string fmt;
      for (size_t k = 0; k < expr.args->size(); k++) {
        fmt += (k ? "," : "");
        fmt += (*expr.args)[k]->type.isInt() ? "%d" : "%f";
      }
      *this << "abl_log_csv(abl_C, \"" << fmt << "\\n\"";
      for (const AST::ExpressionPtr &arg : *expr.args) *this << ", " << *arg;
      *this << ")";
      return;
    }
  }
  CPrinter::print(expr);
}

// `Agent { m: e, ... }`: members are evaluated in the written order (as gcc
// does for the reference's compound literal, CPrinter.cpp:87-90).
void CudaPrinter::print(const AST::AgentCreationExpression &expr) {
  *this << "([&]() { " << expr.name << " abl_a; ";
  for (const AST::MemberInitEntryPtr &m : *expr.members) {
    *this << "abl_a." << m->name << " = " << *m->expr << "; ";
  }
  *this << "return abl_a; }())";
}

void CudaPrinter::print(const AST::IfStatement &stmt) {
  auto it = deferredMasks.find(&stmt);
  if (it != deferredMasks.end()) {
    *this << "if (" << *stmt.condExpr << ") " << it->second << " |= 1ull << abl_k;";
    return;
  }
  CPrinter::print(stmt);
}

void CudaPrinter::print(const AST::WhileStatement &stmt) {
  if (nearLoopDepth >= 0) nearLoopDepth++;
  CPrinter::print(stmt);
  if (nearLoopDepth >= 0) nearLoopDepth--;
}

void CudaPrinter::print(const AST::BreakStatement &stmt) {
  if (nearLoopDepth == 0) {
    *this << "goto " << nearEndLabel << ";";
    nearNeedsEnd = true;
    return;
  }
  CPrinter::print(stmt);
}

// Mixed precision (-C cuda.precision=mixed): the accumulations of a near
// body that run in FP32.  A statement `acc += nx.m` qualifies when acc is a
// float, float2 or float3 variable declared outside the loop, mentioned
// nowhere else in the body, and m a member of the loop's agent of the same
// type.  Only the sum changes precision: which neighbours are visited, the
// order, the radius test and every other expression stay the reference's
// FP64 ones.
std::vector<CudaPrinter::MixedAcc> CudaPrinter::findMixedAccs(
    const AST::ForStatement &loop, const AST::AgentDeclaration &nearAgent) {
  std::vector<MixedAcc> out;
  if (!mixed) return out;
  Collector c = collect(*loop.stmt);
  std::set<VarId> inner;
  for (auto *d : c.decls) inner.insert(d->var->id);
  for (auto *f : c.fors) inner.insert(f->var->id);
  std::map<VarId, int> uses;
  for (auto *v : c.varExprs) uses[v->var->id]++;
  for (auto *a : c.assignOps) {
    if (a->op != AST::BinaryOp::ADD) continue;
    auto *lv = dynamic_cast<const AST::VarExpression *>(&*a->left);
    auto *rm = dynamic_cast<const AST::MemberAccessExpression *>(&*a->right);
    if (!lv || !rm || inner.count(lv->var->id) || isGlobal(*lv->var)) continue;
    auto *rv = dynamic_cast<const AST::VarExpression *>(&*rm->expr);
    if (!rv || rv->var->id != loop.var->id || uses[lv->var->id] != 1) continue;
    for (size_t k = 0; k < nearAgent.members->size(); k++) {
      const AST::AgentMember &m = *(*nearAgent.members)[k];
      if (m.name != rm->member) continue;
      Type t = m.type->resolved;
      if (!(t == Type::FLOAT || t.isVec()) || !(a->left->type == t)) break;
      MixedAcc acc;
      acc.stmt = a;
      acc.member = (int) k;
      acc.isPos = m.isPosition;
      acc.comps = t.isVec() ? t.getVecLen() : 1;
      out.push_back(acc);
      break;
    }
  }
  return out;
}

// A member of the near loop's neighbour that is not loaded ahead (mixed
// form, read only by lazy distances) is read from its column at the current
// slot.
void CudaPrinter::print(const AST::MemberAccessExpression &expr) {
  auto *v = dynamic_cast<const AST::VarExpression *>(&*expr.expr);
  auto it = columnOnly.find(expr.member);
  if (v && it != columnOnly.end() && v->var->id == nearVar) {
    *this << "((const " << cType(expr.type) << " *) abl_NB.cols[" << it->second << "])["
          << nearSlot << "]";
    return;
  }
  CPrinter::print(expr);
}

void CudaPrinter::print(const AST::AssignOpStatement &stmt) {
  auto it = mixedAccs.find(&stmt);
  if (it == mixedAccs.end()) {
    CPrinter::print(stmt);
    return;
  }
  const MixedAcc &m = it->second;
  if (m.isPos) {
    *this << m.acc << ".add_offset(abl_NB, " << nearSlot << ", " << mixedAnchor << ");";
  } else {
    *this << m.acc << ".add_member(abl_NB, " << m.member << ", " << nearSlot << ");";
  }
}

// The near loop (reference: CPrinter.cpp:148-173).  Candidates come from the
// runtime's grid; the reference's own radius test decides the rare
// candidates that the float prefilter cannot.
void CudaPrinter::print(const AST::ForStatement &stmt) {
  for (size_t k = 0; k < devInit.size(); k++) {
    if (devInit[k].loop == &stmt && fnKind == FnKind::HOST) {
      auto range = stmt.getRange();
      *this << "abl_devinit_record(" << (int) k << ", " << range.first << ", " << range.second
            << ");";
      return;
    }
  }
  if (!stmt.isNear()) {
    if (nearLoopDepth >= 0) nearLoopDepth++;
    CPrinter::print(stmt);
    if (nearLoopDepth >= 0) nearLoopDepth--;
    return;
  }
  if (nearLoopDepth >= 0) throw BackendError("Nested near loops are not supported");
  const AST::Expression &agentExpr = stmt.getNearAgent();
  const AST::Expression &radiusExpr = stmt.getNearRadius();
  AST::AgentDeclaration *agentDecl = stmt.type->resolved.getAgentDecl();
  AST::AgentMember *posMember = agentDecl->getPositionMember();
  bool is3 = posMember->type->resolved == Type::VEC3;
  const char *distFn = is3 ? "dist_float3" : "dist_float2";
  int dim = is3 ? 3 : 2;
  int id = ++nearCounter;
  std::string sid = std::to_string(id);
  std::string q = "abl_q" + sid, c = "abl_c" + sid, ex = "abl_exact" + sid;
  std::string nxs = "abl_nx" + sid, slot = "abl_slot" + sid;

  int posIdx = -1;
  for (size_t k = 0; k < agentDecl->members->size(); k++) {
    if (&*(*agentDecl->members)[k] == posMember) posIdx = (int) k;
  }
  std::string posCol = "((const " + cType(posMember->type->resolved) + " *) abl_NB.cols["
                     + std::to_string(posIdx) + "])";

  const bool presorted = fnKind == FnKind::STEP && !steps.empty() && steps.back().presorted;

  // The querying agent's index, when the loop is centred on the step's own
  // agent: its cell then comes from the binning.
  const AST::FunctionDeclaration *stepDecl =
      fnKind == FnKind::STEP && !steps.empty() ? steps.back().decl : nullptr;
  auto *centerVar = dynamic_cast<const AST::VarExpression *>(&agentExpr);
  const bool centredOnSelf = stepDecl && centerVar
                          && centerVar->var->id == stepDecl->stepParam().var->id;
  *this << "{" << indent << nl
        << "const abl::near_query<" << dim << "> " << q << "(abl_NB, (double) " << agentExpr
        << "->" << posMember->name << ".x, (double) " << agentExpr << "->" << posMember->name
        << ".y, " << (is3 ? "(double) " : "0.0");
  if (is3) *this << agentExpr << "->" << posMember->name << ".z";
  *this << (centredOnSelf ? ", abl_K.self" : "") << ");" << nl;
  if (presorted) {
    *this << "abl::near_list_cursor<" << dim << "> " << c << "(abl_NB, " << q << ", abl_K);";
  } else {
    *this << "abl::near_cursor<" << dim << "> " << c << "(abl_NB, " << q << ");";
  }
  std::vector<MixedAcc> maccs = fnKind == FnKind::STEP ? findMixedAccs(stmt, *agentDecl)
                                                       : std::vector<MixedAcc>();
  auto savedMixed = mixedAccs;
  std::string savedAnchor = mixedAnchor;
  mixedAccs.clear();
  if (!maccs.empty()) {
    mixedAnchor = "abl_ma" + sid;
    *this << nl << "const abl::mixed_anchor<" << dim << "> " << mixedAnchor << "((double) "
          << agentExpr << "->" << posMember->name << ".x, (double) " << agentExpr << "->"
          << posMember->name << ".y, " << (is3 ? "(double) " : "0.0");
    if (is3) *this << agentExpr << "->" << posMember->name << ".z";
    *this << ");";
    for (size_t j = 0; j < maccs.size(); j++) {
      maccs[j].acc = "abl_fa" + sid + "_" + std::to_string(j);
      mixedAccs[maccs[j].stmt] = maccs[j];
      *this << nl << "abl::facc<" << maccs[j].comps << "> " << maccs[j].acc << ";";
    }
  }
  *this << nl
        << "auto " << ex << " = [&](int abl_s) -> bool {" << indent << nl
        << "const " << cType(posMember->type->resolved) << " abl_p = " << posCol << "[abl_s];"
        << nl << "return !(" << distFn << "(abl_p, " << agentExpr << "->" << posMember->name
        << ") > " << radiusExpr << ");" << outdent << nl << "};" << nl
        << "while (" << c << ".fill(" << q << ", " << ex << ")) {" << indent;
  // Load the members the loop reads (AnalysisVisitor collects them,
  // src/AnalysisVisitor.cpp:1101-1105).  The next neighbour's members are
  // loaded while the body runs on the current one.
  const AST::FunctionDeclaration *cur = steps.empty() ? nullptr : steps.back().decl;
  std::string pslot = "abl_pslot" + sid, pnx = "abl_pnx" + sid;
  // Members the FP32 sums read from float copies need no FP64 load unless
  // the body reads them elsewhere too.
  // The same for members read only inside lazy distances, whose reference
  // expression runs for the few candidates the FP32 band leaves undecided:
  // those members are read from their column where used (`columnOnly`).
  std::map<std::string, int> fp64Reads;
  std::vector<DeferredIf> deferred;
  if (fnKind == FnKind::STEP) deferred = findDeferredIfs(script, stepDecl, stmt);
  auto savedColumnOnly = columnOnly;
  const VarId savedNearVar = nearVar;
  columnOnly.clear();
  if (!maccs.empty()) {
    std::vector<const AST::Statement *> bodies;
    for (const DeferredIf &d : deferred) bodies.push_back(&*d.ifs->ifStmt);
    std::set<const AST::MemberAccessExpression *> inLazy;
    for (const AST::VarDeclarationStatement *d : findLazyDistances(script, stmt, bodies))
      for (auto *ma : collect(*const_cast<AST::Expression *>(&*d->initializer)).members)
        inLazy.insert(ma);
    std::map<std::string, int> lazyReads;
    Collector bc = collect(*stmt.stmt);
    for (auto *ma : bc.members) {
      auto *v = dynamic_cast<const AST::VarExpression *>(&*ma->expr);
      if (!v || v->var->id != stmt.var->id) continue;
      if (inLazy.count(ma)) lazyReads[ma->member]++;
      else fp64Reads[ma->member]++;
    }
    for (const MixedAcc &m : maccs)
      fp64Reads[(*agentDecl->members)[m.member]->name]--;
    for (size_t k = 0; k < agentDecl->members->size(); k++) {
      const std::string &nm = (*agentDecl->members)[k]->name;
      if (fp64Reads[nm] <= 0 && lazyReads[nm] > 0) columnOnly[nm] = (int) k;
    }
    nearVar = stmt.var->id;
  }
  auto loadMembers = [&](const std::string &var, const std::string &at) {
    for (size_t k = 0; k < agentDecl->members->size(); k++) {
      const AST::AgentMember &m = *(*agentDecl->members)[k];
      bool used = cur && cur->accessedMembers.count(m.name);
      if (!used) continue;
      if (!maccs.empty() && fp64Reads[m.name] <= 0) continue;
      *this << nl << var << "." << m.name << " = ((const " << cType(m.type->resolved)
            << " *) abl_NB.cols[" << (int) k << "])[" << at << "];";
    }
  };
  *this << nl << "int " << pslot << " = " << c << ".slot(0);" << nl << agentDecl->name << " "
        << pnx << ";";
  loadMembers(pnx, pslot);
  std::map<const AST::IfStatement *, std::string> savedMasks = deferredMasks;
  deferredMasks.clear();
  for (size_t j = 0; j < deferred.size(); j++) {
    std::string mask = "abl_dm" + sid + "_" + std::to_string(j);
    deferredMasks[deferred[j].ifs] = mask;
    *this << nl << "unsigned long long " << mask << " = 0ull;";
  }
  *this << nl << "for (int abl_k = 0; abl_k < " << c << ".cnt; ++abl_k) {" << indent << nl
        << "const int " << slot << " = " << pslot << ";" << nl
        << agentDecl->name << " " << nxs << " = " << pnx << ";" << nl
        << "if (abl_k + 1 < " << c << ".cnt) {" << indent << nl
        << pslot << " = " << c << ".slot(abl_k + 1);";
  loadMembers(pnx, pslot);
  *this << outdent << nl << "}";
  *this << nl << agentDecl->name << "* " << *stmt.var << " = &" << nxs << ";" << nl;

  std::string savedLabel = nearEndLabel;
  bool savedNeeds = nearNeedsEnd;
  std::vector<const AST::Statement *> deferredBodies;
  for (const DeferredIf &d : deferred) deferredBodies.push_back(&*d.ifs->ifStmt);
  lazyDecls = findLazyDistances(script, stmt, deferredBodies);
  nearQuery = q;
  nearSlot = slot;
  nearEndLabel = "abl_near_end" + sid;
  nearNeedsEnd = false;
  nearLoopDepth = 0;
  *this << *stmt.stmt;
  lazyDecls.clear();
  *this << outdent << nl << "}";
  // Second pass over the chunk: the deferred conditional blocks, each over
  // the neighbours where its condition held, in ascending order.
  deferredPass = true;
  for (size_t j = 0; j < deferred.size(); j++) {
    const std::string &mask = deferredMasks[deferred[j].ifs];
    *this << nl << "for (unsigned long long abl_m = " << mask << "; abl_m; abl_m &= abl_m - 1ull) {"
          << indent << nl << "const int " << slot << " = " << c
          << ".slot(__ffsll((long long) abl_m) - 1);" << nl << agentDecl->name << " " << nxs << ";";
    loadMembers(nxs, slot);
    *this << nl << agentDecl->name << "* " << *stmt.var << " = &" << nxs << ";";
    for (const AST::VarDeclarationStatement *d : deferred[j].recompute) *this << nl << *d;
    *this << nl << *deferred[j].ifs->ifStmt << outdent << nl << "}";
  }
  deferredPass = false;
  deferredMasks = savedMasks;
  nearLoopDepth = -1;
  *this << outdent << nl << "}";
  // Mixed precision: the FP32 sums back into their FP64 variables.
  for (const MixedAcc &m : maccs) {
    const AST::VarExpression &v = *dynamic_cast<const AST::VarExpression *>(&*m.stmt->left);
    std::string fn = m.isPos ? "offset_total(" + mixedAnchor + ", " : "total(";
    *this << nl << v << " = ";
    if (m.comps == 1) {
      *this << v << " + " << m.acc << "." << fn << "0);";
    } else {
      const char *vt = m.comps == 2 ? "float2" : "float3";
      *this << vt << "_add(" << v << ", " << vt << "_create(";
      for (int d = 0; d < m.comps; d++)
        *this << (d ? ", " : "") << m.acc << "." << fn << d << ")";
      *this << "));";
    }
  }
  mixedAccs = savedMixed;
  mixedAnchor = savedAnchor;
  columnOnly = savedColumnOnly;
  nearVar = savedNearVar;
  *this << outdent << nl << "}";
  if (nearNeedsEnd) *this << nl << nearEndLabel << ": ;";
  nearEndLabel = savedLabel;
  nearNeedsEnd = savedNeeds;
}

void CudaPrinter::print(const AST::SimulateStatement &stmt) {
  *this << "abl_simulate(" << *stmt.timestepsExpr << ");";
}

void CudaPrinter::print(const AST::FunctionDeclaration &decl) {
  if (decl.isMain()) {
    fnKind = FnKind::HOST;
    *this << "static int abl_main() {" << indent << *decl.stmts << nl << "return 0;"
          << outdent << nl << "}";
    return;
  }
  if (decl.isParallelStep()) {
    fnKind = FnKind::STEP;
    printStepFunction(decl);
    fnKind = FnKind::HOST;
    return;
  }
  if (decl.isSequentialStep()) {
    fnKind = FnKind::SEQ;
    printSeqStep(decl);
    fnKind = FnKind::HOST;
    return;
  }
  fnKind = FnKind::USER;
  printUserFunction(decl);
  fnKind = FnKind::HOST;
}

// The sequential step runs on the host after every timestep; its builtins
// (count, sum, log_csv, getLastExecTime) call the runtime's reductions.
void CudaPrinter::printSeqStep(const AST::FunctionDeclaration &decl) {
  seqStep = &decl;
  *this << "static int abl_seq_" << decl.name
        << "(abl_ctx *abl_C, const void *abl_gp) {" << indent << nl
        << "const abl_globals &abl_G = *(const abl_globals *) abl_gp;" << nl
        << "abl::rng abl_R_host;" << nl << "abl::rng &abl_R = abl_R_host;" << nl
        << "(void) abl_G; (void) abl_R;" << *decl.stmts << nl << "return ABL_OK;" << outdent
        << nl << "}";
}

// Functions that reach a host-only builtin (the sequential RNG of
// asset/c/libabl.c:8-39, add, save) run on the host only.
bool CudaPrinter::hostOnlyFunction(const AST::FunctionDeclaration *f, int depth) {
  auto it = hostOnlyMemo.find(f);
  if (it != hostOnlyMemo.end()) return it->second;
  if (depth > 64) return true;
  hostOnlyMemo[f] = false;
  Collector c = collect(*const_cast<AST::FunctionDeclaration *>(f));
  bool h = false;
  for (auto *call : c.calls) {
    // random()/randomInt() run on both sides (abl_random); the rest of the
    // simulation builtins exist on the host only.
    if (call->isBuiltin() && isHostOnlyBuiltin(call->name) && call->name != "random"
        && call->name != "randomInt") h = true;
    if (call->kind == AST::CallExpression::Kind::USER && call->calledFunc
        && hostOnlyFunction(call->calledFunc, depth + 1)) h = true;
  }
  hostOnlyMemo[f] = h;
  return h;
}

void CudaPrinter::printUserFunction(const AST::FunctionDeclaration &decl) {
  bool host = hostOnlyFunction(&decl, 0);
  *this << (host ? "static inline " : "__host__ __device__ static inline ")
        << *decl.returnType << " " << decl.sig.name << "(const abl_globals &abl_G, abl::rng &abl_R";
  if (!decl.params->empty()) *this << ", ";
  printParams(decl);
  *this << ") {" << indent << *decl.stmts << outdent << nl << "}";
}

void CudaPrinter::printStepFunction(const AST::FunctionDeclaration &decl) {
  StepInfo info;
  info.decl = &decl;
  const AST::AgentDeclaration &agent = decl.stepAgent();
  info.agentType = agentIndex(&agent);
  Collector c = collect(*const_cast<AST::FunctionDeclaration *>(&decl));
  for (auto *call : c.calls) {
    if (call->isBuiltin() && call->name == "removeCurrent") info.usesRemove = true;
  }
  // Random numbers, drawn directly or through user functions.
  std::set<const AST::FunctionDeclaration *> seen;
  std::function<bool(const Collector &)> draws = [&](const Collector &cc) -> bool {
    for (auto *call : cc.calls) {
      if (call->isBuiltin() && (call->name == "random" || call->name == "randomInt")) return true;
      if (call->kind == AST::CallExpression::Kind::USER && call->calledFunc
          && seen.insert(call->calledFunc).second
          && draws(collect(*const_cast<AST::FunctionDeclaration *>(call->calledFunc)))) {
        return true;
      }
    }
    return false;
  };
  info.usesRng = draws(c);
  if (decl.runtimeAddedAgent) info.addType = agentIndex(decl.runtimeAddedAgent);
  if (!c.nearLoops.empty()) {
    const AST::ForStatement *loop = c.nearLoops[0];
    info.nearLoop = loop;
    const AST::AgentDeclaration *nearAgent = loop->type->resolved.getAgentDecl();
    info.nearType = agentIndex(nearAgent);
    // Mixed precision: the FP32 sums do not depend on the visiting order
    // (they are not the reference's bits in any order), so a body whose only
    // order-dependent statements they were runs without sorting neighbours.
    std::set<const AST::AssignOpStatement *> fp32Sums;
    for (const MixedAcc &m : findMixedAccs(*loop, *nearAgent)) fp32Sums.insert(m.stmt);
    info.ordered = nearBodyIsOrdered(*loop, &fp32Sums);
    for (size_t k = 0; k < nearAgent->members->size(); k++) {
      const AST::AgentMember &m = *(*nearAgent->members)[k];
      if (decl.accessedMembers.count(m.name) || m.isPosition) info.nearMembers |= 1u << k;
    }
    // Mixed precision: members read only by FP32 sums come from float
    // copies and need no FP64 copy (the position's is kept for the radius
    // test).
    std::vector<MixedAcc> maccs = findMixedAccs(*loop, *nearAgent);
    if (!maccs.empty()) {
      std::map<int, int> reads;
      for (auto *ma : collect(*loop->stmt).members) {
        auto *v = dynamic_cast<const AST::VarExpression *>(&*ma->expr);
        if (!v || v->var->id != loop->var->id) continue;
        for (size_t k = 0; k < nearAgent->members->size(); k++)
          if ((*nearAgent->members)[k]->name == ma->member) reads[(int) k]++;
      }
      for (const MixedAcc &m : maccs) {
        reads[m.member]--;
        if (m.isPos) info.nearPosLo = true;
        else info.nearMembersF32 |= 1u << m.member;
      }
      for (auto &kv : reads) {
        if (kv.second <= 0 && !(*nearAgent->members)[kv.first]->isPosition)
          info.nearMembers &= ~(1u << kv.first);
      }
    }
    // The radius must not depend on the agent: it sizes the grid search.  A
    // step-local variable holding a value of globals (`float radius = 125;`
    // in keratinocyte.abl) stands for its initialiser.
    if (auto *rv = dynamic_cast<const AST::VarExpression *>(&loop->getNearRadius())) {
      if (!isGlobal(*rv->var)) {
        for (const AST::StatementPtr &st : *decl.stmts) {
          auto *d = dynamic_cast<const AST::VarDeclarationStatement *>(&*st);
          if (d && d->var->id == rv->var->id && d->initializer) info.radiusLocal = d;
        }
        auto assigned = [&](const AST::Expression &left) {
          const AST::VarExpression *root = targetRoot(left);
          return root && root->var->id == rv->var->id;
        };
        for (auto *a : c.assigns) if (assigned(*a->left)) info.radiusLocal = nullptr;
        for (auto *a : c.assignOps) if (assigned(*a->left)) info.radiusLocal = nullptr;
      }
    }
    Collector rc = collect(info.radiusLocal
                               ? *const_cast<AST::Expression *>(&*info.radiusLocal->initializer)
                               : *const_cast<AST::Expression *>(&loop->getNearRadius()));
    for (auto *v : rc.varExprs) {
      if (!isGlobal(*v->var)) {
        throw BackendError("The cuda backend needs a near() radius that does not depend on "
                           "the agent");
      }
    }
    auto *center = dynamic_cast<const AST::VarExpression *>(&loop->getNearAgent());
    const bool selfCentred = center && center->var->id == decl.stepParam().var->id;
    info.presorted = info.ordered && c.nearLoops.size() == 1 && rc.calls.empty() && selfCentred;
    // One near loop around the step's own agent, with a radius of plain
    // arithmetic on globals (evaluated alike on host and device): its
    // neighbours are a function of the population's positions alone.
    info.nearCacheable = c.nearLoops.size() == 1 && selfCentred && rc.calls.empty();
  }
  // Members of `out` written by the function: any assignment rooted at
  // out.m may write it; a top-level `out.m = e` always does, provided `out`
  // is never read and the function never returns early.
  const AST::Param &param = decl.stepParam();
  VarId outId = param.outVar->id;
  auto memberBit = [&](const std::string &name) -> unsigned {
    for (size_t k = 0; k < agent.members->size(); k++) {
      if ((*agent.members)[k]->name == name) return 1u << k;
    }
    return 0;
  };
  unsigned all = agent.members->size() >= 32 ? ~0u : ((1u << agent.members->size()) - 1);
  int outTargets = 0;
  auto noteTarget = [&](const AST::Expression &left) {
    const AST::VarExpression *root = targetRoot(left);
    if (!root || root->var->id != outId) return;
    outTargets++;
    std::string m = targetMember(left);
    info.outMaybe |= m.empty() ? all : memberBit(m);
  };
  for (auto *a : c.assigns) noteTarget(*a->left);
  for (auto *a : c.assignOps) noteTarget(*a->left);
  // Members the body may set to anything but the agent's own value: every
  // write except `out.m = in.m` (same member) counts.
  VarId inId = param.var->id;
  auto selfCopy = [&](const AST::AssignStatement &a) {
    auto *l = dynamic_cast<const AST::MemberAccessExpression *>(&*a.left);
    auto *r = dynamic_cast<const AST::MemberAccessExpression *>(&*a.right);
    if (!l || !r || l->member != r->member) return false;
    auto *lv = dynamic_cast<const AST::VarExpression *>(&*l->expr);
    auto *rv = dynamic_cast<const AST::VarExpression *>(&*r->expr);
    return lv && rv && lv->var->id == outId && rv->var->id == inId;
  };
  for (auto *a : c.assigns) {
    const AST::VarExpression *root = targetRoot(*a->left);
    if (!root || root->var->id != outId || selfCopy(*a)) continue;
    std::string m = targetMember(*a->left);
    info.outChanged |= m.empty() ? all : memberBit(m);
  }
  for (auto *a : c.assignOps) {
    const AST::VarExpression *root = targetRoot(*a->left);
    if (!root || root->var->id != outId) continue;
    std::string m = targetMember(*a->left);
    info.outChanged |= m.empty() ? all : memberBit(m);
  }
  int outUses = 0;
  for (auto *v : c.varExprs) outUses += v->var->id == outId;
  if (c.returns == 0 && outUses == outTargets) {
    for (const AST::StatementPtr &s : *decl.stmts) {
      auto *a = dynamic_cast<const AST::AssignStatement *>(&*s);
      if (!a) continue;
      const AST::VarExpression *root = targetRoot(*a->left);
      if (!root || root->var->id != outId) continue;
      auto *ma = dynamic_cast<const AST::MemberAccessExpression *>(&*a->left);
      if (dynamic_cast<const AST::VarExpression *>(&*a->left)) {
        info.outAlways |= all;
      } else if (ma && dynamic_cast<const AST::VarExpression *>(&*ma->expr)) {
        info.outAlways |= memberBit(ma->member);
      }
    }
  }
  steps.push_back(info);

  *this << "__device__ static void " << decl.name
        << "(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, ";
  printParams(decl);
  *this << ") {" << indent << nl << "abl::rng &abl_R = abl_K.R;" << nl
        << "(void) abl_R; (void) abl_NB;" << *decl.stmts << outdent << nl << "}" << nl;
  printKernel(steps.back());
}

// Phase one of a presorted step kernel: this thread's agent (abl_i1, valid
// when abl_has) gathers its sorted neighbour list and the block picks the
// agent each thread runs (abl_j).  The radius test is the near loop's own.
void CudaPrinter::printPresortPhase(const StepInfo &info, const std::string &view,
                                    const std::string &pos) {
  const AST::ForStatement &loop = *info.nearLoop;
  AST::AgentDeclaration *nearAgent = loop.type->resolved.getAgentDecl();
  AST::AgentMember *posMember = nearAgent->getPositionMember();
  bool is3 = posMember->type->resolved == Type::VEC3;
  int dim = is3 ? 3 : 2;
  std::string pt = cType(posMember->type->resolved);
  int posIdx = memberIndex(nearAgent, posMember);
  *this << "const " << pt << " abl_p1 = abl_has ? " << pos << " : " << pt << "{};" << nl
        << "const abl::near_query<" << dim << "> abl_q0(" << view
        << ", (double) abl_p1.x, (double) abl_p1.y, " << (is3 ? "(double) abl_p1.z" : "0.0")
        << ", abl_has ? abl_i1 : -1);" << nl
        << "auto abl_x0 = [&](int abl_s) -> bool {" << indent << nl
        << "const " << pt << " abl_p = ((const " << pt << " *) " << view << ".cols[" << posIdx
        << "])[abl_s];" << nl << "return !(" << (is3 ? "dist_float3" : "dist_float2")
        << "(abl_p, abl_p1) > ";
  printNearRadius(info);
  *this << ");" << outdent << nl << "};" << nl
        << "abl_j = abl::presort_block<" << dim << ">(" << view << ", abl_has, abl_q0, abl_x0);";
}

// The near radius outside the step body (phase one of a presorted kernel,
// the host's radius function): a step-local radius variable is replaced by
// its initialiser converted to the variable's type.
void CudaPrinter::printNearRadius(const StepInfo &info) {
  if (info.radiusLocal) {
    *this << "((" << *info.radiusLocal->type << ") (" << *info.radiusLocal->initializer << "))";
  } else {
    *this << info.nearLoop->getNearRadius();
  }
}

void CudaPrinter::printKernel(const StepInfo &info) {
  const AST::FunctionDeclaration &decl = *info.decl;
  const AST::AgentDeclaration &agent = decl.stepAgent();
  const std::string &T = agent.name;
  const std::string &name = decl.name;
  bool copy = copyOut();
  // The per-phase kernels and their launchers are compiled once, without
  // ABL_PERSIST; the persistent ensemble kernel's compilation (ABL_PERSIST)
  // needs only the step bodies.
  *this << nl << "#ifndef ABL_PERSIST";
  *this << nl << "struct abl_kargs_" << name << " {" << indent << nl
        << "abl_globals G;" << nl << "long n;" << nl << "const int *visit;" << nl
        << "abl_cols_" << T << " in, out;" << nl << "abl_near_view NB;" << nl
        << "uint8_t *removed;" << nl << "uint8_t *child_flag;" << nl
        << "void *child_cols[ABL_MAX_MEMBERS];" << nl << "uint64_t seed;" << nl
        << "long timestep;" << nl << "int step_index;" << nl << "uint32_t skip_store;" << nl
        << "unsigned long long *serial_rng;" << outdent << nl << "};"
        << nl << "__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_" << name
        << "(const __grid_constant__ abl_kargs_" << name << " A) {" << indent << nl;
  if (info.presorted) {
    *this << "int abl_j;" << nl << "{" << indent << nl
          << "const abl_globals &abl_G = A.G;" << nl
          << "const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;" << nl
          << "const bool abl_has = abl_t1 < A.n;" << nl
          << "const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;"
          << nl;
    printPresortPhase(info, "A.NB", "A.in." + agent.getPositionMember()->name + "[abl_i1]");
    *this << outdent << nl << "}" << nl
          << "const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;" << nl;
  } else {
    *this << "const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;" << nl;
  }
  *this << "if (abl_t >= A.n) return;" << nl
        << "const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;" << nl
        << "abl::step_ctx abl_K;" << nl
        << "abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);"
        << nl << "abl_K.R.xs = A.serial_rng;"
        << nl << "abl_K.self = abl_i;" << nl << "abl_K.removed = 0;" << nl << "abl_K.added = 0;"
        << nl << "abl_K.child_cols = A.child_cols;" << nl
        << "abl_K.near_col = " << (info.presorted ? "abl_j" : "-1") << ";" << nl
        << T << " abl_in, abl_out;";
  for (size_t k = 0; k < agent.members->size(); k++) {
    const std::string &m = (*agent.members)[k]->name;
    *this << nl << "abl_in." << m << " = A.in." << m << "[abl_i];";
  }
  if (copy) {
    // Models with runtime add/remove: `out` starts as a copy of `in`, as the
    // MASON backend's prepareOutState does (MasonPrinter.cpp:480-486).
    *this << nl << "abl_out = abl_in;";
  } else {
    for (size_t k = 0; k < agent.members->size(); k++) {
      const std::string &m = (*agent.members)[k]->name;
      bool maybe = info.outMaybe & (1u << k), always = info.outAlways & (1u << k);
      // The double buffer keeps whatever it held for members the step does
      // not always write (the reference's agents_X_dbuf, CPrinter.cpp:210-228).
      if (maybe && !always) *this << nl << "abl_out." << m << " = A.out." << m << "[abl_i];";
    }
  }
  *this << nl << name << "(A.G, A.NB, abl_K, &abl_in, &abl_out);";
  for (size_t k = 0; k < agent.members->size(); k++) {
    const std::string &m = (*agent.members)[k]->name;
    if (copy || (info.outMaybe & (1u << k))) {
      // A member the step only copies from `in` (out.m = in.m) is stored
      // unless the runtime knows the double buffer holds the same value.
      const bool selfCopyOnly = !copy && !(info.outChanged & (1u << k));
      *this << nl << (selfCopyOnly ? "if (!(A.skip_store & " + std::to_string(1u << k) + "u)) " : "")
            << "A.out." << m << "[abl_i] = abl_out." << m << ";";
    }
  }
  if (info.usesRemove) *this << nl << "A.removed[abl_i] = (uint8_t) abl_K.removed;";
  if (info.addType >= 0) *this << nl << "A.child_flag[abl_i] = (uint8_t) abl_K.added;";
  *this << outdent << nl << "}" << nl
        << "static int abl_launch_" << name
        << "(const abl_step_launch *L, cudaStream_t abl_stream) {" << indent << nl
        << "abl_kargs_" << name << " A;" << nl
        << "A.G = *(const abl_globals *) L->globals;" << nl
        << "A.n = L->n;" << nl << "A.visit = L->visit_order;";
  for (size_t k = 0; k < agent.members->size(); k++) {
    const AST::AgentMember &m = *(*agent.members)[k];
    std::string ty = cType(m.type->resolved);
    *this << nl << "A.in." << m.name << " = (" << ty << " *) L->in_cols[" << (int) k << "];"
          << nl << "A.out." << m.name << " = (" << ty << " *) L->out_cols[" << (int) k << "];";
  }
  *this << nl << "A.NB = L->near;" << nl << "A.removed = L->removed;" << nl
        << "A.child_flag = L->child_flag;" << nl
        << "for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];" << nl
        << "A.seed = L->seed;" << nl << "A.timestep = L->timestep;" << nl
        << "A.step_index = L->step_index;" << nl << "A.skip_store = L->skip_store;" << nl
        << "A.serial_rng = L->serial_rng;" << nl
        << "const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : "
           "ABL_STEP_BLOCK;" << nl
        << "const long abl_grid = (A.n + abl_block - 1) / abl_block;" << nl
        << "abl_kernel_" << name << "<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);" << nl
        << "return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;" << outdent << nl
        << "}" << nl << "#endif" << nl;
  if (ensembleStep(info)) {
    // Ensemble variant: every agent reads its replica's globals and grid.
    // Random numbers are keyed by the replica's seed and the agent's index
    // within its replica, so each replica draws what it would draw alone.
    // The body runs the agents of virtual block abl_vb at timestep abl_ts:
    // the per-phase kernel passes its block index, the persistent kernel
    // strides over the blocks of every step function of every timestep.
    *this << "__device__ __forceinline__ void abl_ens_body_" << name
          << "(const abl_ens_launch &A, long abl_vb, long abl_ts) {" << indent << nl;
    if (info.presorted) {
      int posIdx = memberIndex(&agent, agent.getPositionMember());
      *this << "int abl_j;" << nl << "{" << indent << nl
            << "const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;" << nl
            << "const bool abl_has = abl_t1 < A.n;" << nl
            << "const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] "
               ": abl_t1) : 0;" << nl
            << "const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;" << nl
            << "const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];" << nl
            << "const abl_near_view &abl_V1 = A.views[abl_r1];" << nl;
      printPresortPhase(info, "abl_V1",
                        "((const " + cType(agent.getPositionMember()->type->resolved)
                            + " *) A.in_cols[" + std::to_string(posIdx) + "])[abl_i1]");
      *this << outdent << nl << "}" << nl
            << "const long abl_t = abl_vb * blockDim.x + abl_j;" << nl;
    } else {
      *this << "const long abl_t = abl_vb * blockDim.x + threadIdx.x;" << nl;
    }
    *this << "if (abl_t >= A.n) return;" << nl
          << "const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;" << nl
          << "const int abl_r = A.replica[abl_i];" << nl
          << "const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];" << nl
          << "abl::step_ctx abl_K;" << nl
          << "abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), "
             "(uint32_t) A.step_index, (uint64_t) abl_ts);"
          << nl << "abl_K.self = abl_i;" << nl << "abl_K.removed = 0;" << nl
          << "abl_K.added = 0;" << nl << "abl_K.child_cols = nullptr;" << nl
          << "abl_K.near_col = " << (info.presorted ? "abl_j" : "-1") << ";" << nl
          << T << " abl_in, abl_out;";
    for (size_t k = 0; k < agent.members->size(); k++) {
      const AST::AgentMember &m = *(*agent.members)[k];
      std::string ty = cType(m.type->resolved);
      *this << nl << "abl_in." << m.name << " = ((const " << ty << " *) A.in_cols[" << (int) k
            << "])[abl_i];";
    }
    for (size_t k = 0; k < agent.members->size(); k++) {
      const AST::AgentMember &m = *(*agent.members)[k];
      std::string ty = cType(m.type->resolved);
      bool maybe = info.outMaybe & (1u << k), always = info.outAlways & (1u << k);
      if (copy) {
        *this << nl << "abl_out." << m.name << " = abl_in." << m.name << ";";
      } else if (maybe && !always) {
        *this << nl << "abl_out." << m.name << " = ((const " << ty << " *) A.out_cols["
              << (int) k << "])[abl_i];";
      }
    }
    *this << nl << name << "(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);";
    for (size_t k = 0; k < agent.members->size(); k++) {
      const AST::AgentMember &m = *(*agent.members)[k];
      std::string ty = cType(m.type->resolved);
      if (copy || (info.outMaybe & (1u << k))) {
        *this << nl << "((" << ty << " *) A.out_cols[" << (int) k << "])[abl_i] = abl_out."
              << m.name << ";";
      }
    }
    *this << outdent << nl << "}" << nl << "#ifndef ABL_PERSIST" << nl
          << "__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_"
          << name << "(const __grid_constant__ abl_ens_launch A) {" << indent << nl
          << "abl_ens_body_" << name << "(A, blockIdx.x, A.timestep);" << outdent << nl << "}"
          << nl << "static int abl_launch_ens_" << name
          << "(const abl_ens_launch *L, cudaStream_t abl_stream) {" << indent << nl
          << "const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : "
             "ABL_STEP_BLOCK;" << nl
          << "const long abl_grid = (L->n + abl_block - 1) / abl_block;" << nl
          << "abl_kernel_ens_" << name << "<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);" << nl
          << "return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;" << outdent << nl
          << "}" << nl << "#endif" << nl;
  }
  if (info.nearLoop) {
    *this << "#ifndef ABL_PERSIST" << nl
          << "static double abl_radius_" << name << "(const void *abl_gp) {" << indent << nl
          << "const abl_globals &abl_G = *(const abl_globals *) abl_gp;" << nl
          << "abl::rng abl_R;" << nl << "(void) abl_G; (void) abl_R;" << nl
          << "return (double) (";
    printNearRadius(info);
    *this << ");" << outdent << nl
          << "}" << nl << "#endif" << nl;
  }
}

// Steps with an ensemble variant: no runtime population changes, and no
// mixed-precision sums (the ensemble builds no float copies).
bool CudaPrinter::ensembleStep(const StepInfo &s) const {
  return s.addType < 0 && !s.usesRemove && !s.nearMembersF32 && !s.nearPosLo;
}

// The model supports ensembles when every step function in simulate order
// has an ensemble variant and there is no sequential step.
bool CudaPrinter::ensembleModel() const {
  if (seqStep || !script.simStmt) return false;
  for (AST::FunctionDeclaration *f : script.simStmt->stepFuncDecls) {
    for (const StepInfo &s : steps) {
      if (s.decl == f && !ensembleStep(s)) return false;
    }
  }
  return !script.simStmt->stepFuncDecls.empty();
}

// The persistent ensemble kernel (compiled with ABL_PERSIST, into its own
// object): every binning and step function of every timestep in one
// cooperative launch (abl_persist.cuh).  step_index is the step's place in
// simulate order, as the runtime numbers the model's steps.
void CudaPrinter::printPersistentKernel() {
  // The binning phases are compiled for the dimension of the positions the
  // near loops bin (0: types of both dimensions, chosen per binning).
  int dim = -1;
  for (const StepInfo &s : steps) {
    if (!s.nearLoop) continue;
    AST::AgentDeclaration *a = s.nearLoop->type->resolved.getAgentDecl();
    int d = a->getPositionMember()->type->resolved == Type::VEC3 ? 3 : 2;
    dim = dim < 0 || dim == d ? d : 0;
  }
  if (dim < 0) dim = 2;
  *this << "__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_PERSIST_MIN_BLOCKS) "
           "abl_kernel_ens_persist(const abl::persist_prog *abl_P, int *abl_err) {"
        << indent << nl
        << "abl::persist_run<abl_float, " << dim << ">(abl_P, abl_err, [&](const abl_ens_launch "
           "&abl_L, long abl_vb, long abl_ts) {" << indent << nl
        << "switch (abl_L.step_index) {" << indent;
  const auto &order = script.simStmt->stepFuncDecls;
  for (size_t k = 0; k < order.size(); k++) {
    *this << nl << "case " << (int) k << ": abl_ens_body_" << order[k]->name
          << "(abl_L, abl_vb, abl_ts); break;";
  }
  *this << nl << "default: break;" << outdent << nl << "}" << outdent << nl << "});"
        << outdent << nl << "}" << nl;
}

void CudaPrinter::printGlobals() {
  *this << "struct abl_globals {" << indent;
  for (AST::ConstDeclaration *decl : script.consts) {
    if (decl->isArray) {
      // A constant array (`int A[] = {...}`) becomes a fixed-size field,
      // initialised like the reference's C array (GenericCPrinter.cpp:77-80).
      auto *init = dynamic_cast<const AST::ArrayInitExpression *>(&*decl->expr);
      if (!init) throw BackendError("Unexpected constant array initializer");
      *this << nl << *decl->type << " " << decl->var->name << "[" << init->exprs->size() << "];";
      continue;
    }
    *this << nl << *decl->type << " " << decl->var->name << ";";
  }
  *this << outdent << nl << "};" << nl
        << "static const abl_globals abl_globals_default = {" << indent;
  for (AST::ConstDeclaration *decl : script.consts) {
    *this << nl;
    if (decl->type->resolved.isVec()) {
      auto *call = dynamic_cast<const AST::CallExpression *>(&*decl->expr);
      if (!call) throw BackendError("Unexpected vector constant initializer");
      *this << "{";
      printCommaSeparated(*call->args, [&](const AST::ExpressionPtr &arg) { *this << *arg; });
      *this << "},";
    } else {
      *this << *decl->expr << ",";
    }
  }
  *this << outdent << nl << "};" << nl
        << "static abl_globals abl_G = abl_globals_default;" << nl;
}

// -C cuda.device_init=true: main()'s loops `for (int i : a..b) add(T{...})`
// run as kernels, one thread per iteration, instead of building the
// population on the host.  Every add() of main() must be such a loop's only
// statement, with member initialisers that read the loop variable and
// globals and call builtins or device-capable user functions; random() draws
// from the counter-based stream keyed by the iteration's index and the
// loop's number (not the reference's sequential xorshift stream: host
// initialisation stays the way to reproduce reference results).
void CudaPrinter::findDeviceInit(const AST::FunctionDeclaration &mainDecl) {
  int adds = 0;
  Collector all = collect(*const_cast<AST::FunctionDeclaration *>(&mainDecl));
  for (auto *call : all.calls) adds += call->isBuiltin() && call->name == "add";
  for (const AST::StatementPtr &st : *mainDecl.stmts) {
    auto *loop = dynamic_cast<const AST::ForStatement *>(&*st);
    if (!loop || !loop->isRange()) continue;
    const AST::Statement *body = &*loop->stmt;
    if (auto *b = dynamic_cast<const AST::BlockStatement *>(body)) {
      if (b->stmts->size() != 1) continue;
      body = &*(*b->stmts)[0];
    }
    auto *es = dynamic_cast<const AST::ExpressionStatement *>(body);
    if (!es) continue;
    auto *call = dynamic_cast<const AST::CallExpression *>(&*es->expr);
    if (!call || !call->isBuiltin() || call->name != "add") continue;
    auto *create = dynamic_cast<const AST::AgentCreationExpression *>(&call->getArg(0));
    if (!create) continue;
    Collector c = collect(*const_cast<AST::AgentCreationExpression *>(create));
    bool ok = true;
    for (auto *v : c.varExprs) {
      const VarId id = v->var->id;
      const bool global = script.scope.has(id) && script.scope.get(id).isGlobal;
      if (!global && id != loop->var->id) ok = false;
    }
    for (auto *cl : c.calls) {
      if (cl->isBuiltin() && isHostOnlyBuiltin(cl->name) && cl->name != "random"
          && cl->name != "randomInt") ok = false;
      if (cl->kind == AST::CallExpression::Kind::USER
          && (!cl->calledFunc || hostOnlyFunction(cl->calledFunc, 0))) ok = false;
    }
    if (!ok) continue;
    DevInit d;
    d.loop = loop;
    d.create = create;
    d.agentType = agentIndex(call->calledSig.paramTypes[0].getAgentDecl());
    devInit.push_back(d);
  }
  if ((int) devInit.size() != adds) {
    devInit.clear();
    throw BackendError("cuda.device_init: every add() of main() must be the only statement of "
                       "a `for (int i : a..b)` loop whose agent reads only the loop variable "
                       "and globals");
  }
}

void CudaPrinter::printDeviceInit() {
  if (devInit.empty()) return;
  *this << "// Device initialisation (-C cuda.device_init=true): main()'s add() loops." << nl
        << "static const uint64_t abl_init_seed = 0x5eedull;" << nl
        << "static long abl_dev_first[" << (int) devInit.size() << "], abl_dev_count["
        << (int) devInit.size() << "];" << nl
        << "static void abl_devinit_record(int k, long first, long last) {" << indent << nl
        << "abl_dev_first[k] = first;" << nl << "abl_dev_count[k] = last > first ? last - first : 0;"
        << outdent << nl << "}" << nl;
  FnKind saved = fnKind;
  fnKind = FnKind::USER;
  for (size_t k = 0; k < devInit.size(); k++) {
    const DevInit &d = devInit[k];
    const AST::AgentDeclaration &a = *script.agents[d.agentType];
    *this << "__global__ void abl_init_" << (int) k << "(const abl_globals abl_G, long abl_first, "
          << "long abl_count, long abl_base, abl_cols_" << a.name << " abl_c) {" << indent << nl
          << "const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;" << nl
          << "if (abl_t >= abl_count) return;" << nl
          << "const int " << *d.loop->var << " = (int) (abl_first + abl_t);" << nl
          << "abl::rng abl_R;" << nl
          << "abl_R.init(abl_init_seed, (uint32_t) abl_t, 0xffffff00u + " << (int) k << "u, 0);"
          << nl << "const " << a.name << " abl_v = " << *d.create << ";";
    for (const AST::AgentMemberPtr &m : *a.members) {
      *this << nl << "abl_c." << m->name << "[abl_base + abl_t] = abl_v." << m->name << ";";
    }
    *this << outdent << nl << "}" << nl;
  }
  fnKind = saved;
}

void CudaPrinter::printHostSimulate() {
  // Hands the host-built population to the device runtime for the simulate
  // loop and reads it back for the statements after it.
  *this << "static void abl_check(int r, const char *what) {" << indent << nl
        << "if (r != ABL_OK) {" << indent << nl
        << "std::fprintf(stderr, \"%s failed: %s\\n\", what, abl_strerror(r));" << nl
        << "std::exit(1);" << outdent << nl << "}" << outdent << nl << "}" << nl
        << "static void abl_simulate(int abl_timesteps) {" << indent << nl
        << "abl_ctx *ctx = nullptr;" << nl
        << "abl_check(abl_create(&abl_desc, 0, &ctx), \"abl_create\");" << nl;
  if (seed) {
    *this << "abl_check(abl_set_seed(ctx, " << std::to_string((unsigned long) seed)
          << "ull), \"abl_set_seed\");" << nl;
  }
  if (nearMode >= 0)
    *this << "abl_check(abl_set_near_mode(ctx, " << nearMode << "), \"abl_set_near_mode\");" << nl;
  if (nearCache >= 0)
    *this << "abl_check(abl_set_near_cache(ctx, " << nearCache << "), \"abl_set_near_cache\");"
          << nl;
  if (balance >= 0)
    *this << "abl_check(abl_set_balance(ctx, " << balance << "), \"abl_set_balance\");" << nl;
  *this << "abl_check(abl_set_globals(ctx, &abl_G, sizeof abl_G), \"abl_set_globals\");";
  for (size_t ti = 0; ti < script.agents.size() && !devInit.empty(); ti++) {
    const AST::AgentDeclaration &a = *script.agents[ti];
    const std::string &T = a.name;
    *this << nl << "{" << indent << nl << "long n = 0;";
    for (size_t k = 0; k < devInit.size(); k++) {
      if (devInit[k].agentType == (int) ti) *this << nl << "n += abl_dev_count[" << (int) k << "];";
    }
    *this << nl << "void *cols[" << (int) a.members->size() << "];" << nl
          << "abl_check(abl_reserve(ctx, " << (int) ti << ", (size_t) n, cols), \"abl_reserve\");"
          << nl << "abl_cols_" << T << " c;";
    for (size_t k = 0; k < a.members->size(); k++) {
      const AST::AgentMember &m = *(*a.members)[k];
      *this << nl << "c." << m.name << " = (" << cType(m.type->resolved) << " *) cols[" << (int) k
            << "];";
    }
    *this << nl << "long base = 0;";
    for (size_t k = 0; k < devInit.size(); k++) {
      if (devInit[k].agentType != (int) ti) continue;
      std::string K = std::to_string(k);
      *this << nl << "if (abl_dev_count[" << K << "] > 0) {" << indent << nl << "abl_init_" << K
            << "<<<(abl_dev_count[" << K << "] + 255) / 256, 256>>>(abl_G, abl_dev_first[" << K
            << "], abl_dev_count[" << K << "], base, c);" << nl << "base += abl_dev_count[" << K
            << "];" << outdent << nl << "}";
    }
    *this << nl << "abl_check(cudaDeviceSynchronize() == cudaSuccess ? ABL_OK : ABL_E_CUDA, "
          << "\"device initialisation\");" << nl
          << "abl_check(abl_commit(ctx, " << (int) ti << "), \"abl_commit\");" << outdent << nl
          << "}";
  }
  for (size_t ti = 0; ti < script.agents.size() && devInit.empty(); ti++) {
    const AST::AgentDeclaration &a = *script.agents[ti];
    const std::string &T = a.name;
    *this << nl << "{" << indent << nl
          << "size_t n = agents.agents_" << T << ".len;" << nl
          << "const " << T << " *aos = (const " << T << " *) agents.agents_" << T << ".values;";
    for (size_t k = 0; k < a.members->size(); k++) {
      const AST::AgentMember &m = *(*a.members)[k];
      std::string ty = cType(m.type->resolved);
      *this << nl << ty << " *c" << k << " = (" << ty << " *) std::malloc(sizeof(" << ty
            << ") * (n ? n : 1));" << nl << "for (size_t i = 0; i < n; i++) c" << k
            << "[i] = aos[i]." << m.name << ";";
    }
    *this << nl << "const void *cols[] = {";
    for (size_t k = 0; k < a.members->size(); k++) *this << (k ? ", " : "") << "c" << k;
    *this << "};" << nl << "abl_check(abl_upload(ctx, " << (int) ti
          << ", cols, n), \"abl_upload\");";
    for (size_t k = 0; k < a.members->size(); k++) *this << nl << "std::free(c" << k << ");";
    *this << outdent << nl << "}";
  }
  // -DABL_SERIAL_RANDOM: random() in steps continues the host's xorshift
  // stream in agent order, as the reference program does on one thread.
  *this << nl << "#ifdef ABL_SERIAL_RANDOM" << nl << "uint64_t abl_xs[2];" << nl
        << "abl_host_rng_get(abl_xs);" << nl
        << "abl_check(abl_set_serial_random(ctx, abl_xs), \"abl_set_serial_random\");" << nl
        << "#endif";
  *this << nl << "abl_check(abl_run(ctx, abl_timesteps), \"abl_run\");";
  *this << nl << "#ifdef ABL_SERIAL_RANDOM" << nl
        << "abl_check(abl_get_serial_random(ctx, abl_xs), \"abl_get_serial_random\");" << nl
        << "abl_host_rng_set(abl_xs);" << nl << "#endif";
  for (size_t ti = 0; ti < script.agents.size(); ti++) {
    const AST::AgentDeclaration &a = *script.agents[ti];
    const std::string &T = a.name;
    *this << nl << "{" << indent << nl << "size_t n = 0;" << nl
          << "abl_check(abl_count(ctx, " << (int) ti << ", &n), \"abl_count\");";
    for (size_t k = 0; k < a.members->size(); k++) {
      const AST::AgentMember &m = *(*a.members)[k];
      std::string ty = cType(m.type->resolved);
      *this << nl << ty << " *c" << k << " = (" << ty << " *) std::malloc(sizeof(" << ty
            << ") * (n ? n : 1));";
    }
    *this << nl << "void *cols[] = {";
    for (size_t k = 0; k < a.members->size(); k++) *this << (k ? ", " : "") << "c" << k;
    *this << "};" << nl << "size_t cap = n;" << nl
          << "abl_check(abl_download(ctx, " << (int) ti << ", cols, &cap), \"abl_download\");"
          << nl << "dyn_array_clean(&agents.agents_" << T << ");" << nl
          << "agents.agents_" << T << " = dyn_array_create_fixed(sizeof(" << T << "), n);" << nl
          << T << " *aos = (" << T << " *) agents.agents_" << T << ".values;" << nl
          << "for (size_t i = 0; i < n; i++) {" << indent;
    for (size_t k = 0; k < a.members->size(); k++) {
      *this << nl << "aos[i]." << (*a.members)[k]->name << " = c" << k << "[i];";
    }
    *this << outdent << nl << "}";
    for (size_t k = 0; k < a.members->size(); k++) *this << nl << "std::free(c" << k << ");";
    *this << outdent << nl << "}";
  }
  *this << nl << "size_t abl_log_len = 0;" << nl << "abl_log_text(ctx, nullptr, 0, &abl_log_len);"
        << nl << "if (abl_log_len > 0) {" << indent << nl
        << "char *abl_log = (char *) std::malloc(abl_log_len + 1);" << nl
        << "abl_log_text(ctx, abl_log, abl_log_len + 1, nullptr);" << nl
        << "FILE *abl_f = std::fopen(\"log.csv\", \"w\");" << nl
        << "if (abl_f) { std::fputs(abl_log, abl_f); std::fclose(abl_f); }" << nl
        << "std::free(abl_log);" << outdent << nl << "}" << nl
        << "abl_destroy(ctx);" << outdent << nl << "}" << nl;
}

void CudaPrinter::printDescriptor() {
  for (const AST::AgentDeclaration *a : script.agents) {
    *this << "static const abl_member_desc abl_members_" << a->name << "[] = {" << indent;
    for (const AST::AgentMemberPtr &m : *a->members) {
      Type t = m->type->resolved;
      int comps = t.isVec() ? (int) t.getVecLen() : 1;
      std::string scalar = t.isBool() ? "1" : t.isInt() ? "4" : (useFloat ? "4" : "8");
      *this << nl << "{\"" << m->name << "\", " << ablTypeId(t) << ", " << comps << ", " << scalar
            << ", " << (m->isPosition ? 1 : 0) << "},";
    }
    *this << outdent << nl << "};" << nl;
  }
  *this << "static const abl_agent_desc abl_agents[] = {" << indent;
  for (const AST::AgentDeclaration *a : script.agents) {
    int posIdx = -1, dim = 0;
    for (size_t k = 0; k < a->members->size(); k++) {
      if ((*a->members)[k]->isPosition) {
        posIdx = (int) k;
        dim = (int) (*a->members)[k]->type->resolved.getVecLen();
      }
    }
    *this << nl << "{\"" << a->name << "\", " << (int) a->members->size() << ", abl_members_"
          << a->name << ", " << posIdx << ", " << dim << "},";
  }
  *this << outdent << nl << "};" << nl;
  *this << "static const abl_global_desc abl_global_table[] = {" << indent;
  int scalarConsts = 0;
  for (AST::ConstDeclaration *decl : script.consts) {
    if (decl->isArray) continue;  // constant arrays are not set by name
    *this << nl << "{\"" << decl->var->name << "\", " << ablTypeId(decl->type->resolved)
          << ", offsetof(abl_globals, " << decl->var->name << ")},";
    scalarConsts++;
  }
  *this << nl << "{nullptr, 0, 0}" << outdent << nl << "};" << nl;

  // Environment bounds and granularity (src/AnalysisVisitor.cpp:474-538).
  AST::EnvironmentDeclaration *env = script.envDecl;
  int envDim = env && env->hasEnvDimension() ? (int) env->getEnvDimension() : 0;
  const AST::Expression *minE = nullptr, *maxE = nullptr, *granE = nullptr;
  if (env) {
    for (const AST::MemberInitEntryPtr &m : *env->members) {
      if (m->name == "min") minE = &*m->expr;
      if (m->name == "max") maxE = &*m->expr;
      if (m->name == "granularity") granE = &*m->expr;
    }
  }
  *this << "static void abl_env_bounds(const void *abl_gp, double *abl_min, double *abl_max) {"
        << indent << nl << "const abl_globals &abl_G = *(const abl_globals *) abl_gp;" << nl
        << "abl::rng abl_R;" << nl << "(void) abl_G; (void) abl_R;";
  if (envDim > 0) {
    std::string vt = envDim == 2 ? "float2" : "float3";
    *this << nl << vt << " abl_lo = ";
    if (minE) *this << *minE;
    else *this << vt << "_fill(0)";
    *this << ";" << nl << vt << " abl_hi = ";
    if (maxE) *this << *maxE;
    else *this << vt << "_fill(0)";
    *this << ";" << nl << "abl_min[0] = abl_lo.x; abl_min[1] = abl_lo.y; abl_min[2] = "
          << (envDim == 3 ? "abl_lo.z" : "0") << ";" << nl
          << "abl_max[0] = abl_hi.x; abl_max[1] = abl_hi.y; abl_max[2] = "
          << (envDim == 3 ? "abl_hi.z" : "0") << ";";
  } else {
    *this << nl << "for (int d = 0; d < 3; d++) abl_min[d] = abl_max[d] = 0;";
  }
  *this << outdent << nl << "}" << nl;
  if (granE) {
    *this << "static double abl_granularity(const void *abl_gp) {" << indent << nl
          << "const abl_globals &abl_G = *(const abl_globals *) abl_gp;" << nl
          << "abl::rng abl_R;" << nl << "(void) abl_G; (void) abl_R;"
          << nl << "return (double) (" << *granE << ");" << outdent << nl << "}" << nl;
  }

  *this << "static const abl_step_desc abl_steps[] = {" << indent;
  for (const StepInfo &s : steps) {
    const std::string &n = s.decl->name;
    *this << nl << "{\"" << n << "\", " << s.agentType << ", " << s.nearType << ", "
          << (s.ordered ? 1 : 0) << ", " << (s.nearLoop ? "abl_radius_" + n : "nullptr") << ", "
          << s.nearMembers << "u, " << s.outAlways << "u, abl_launch_" << n << ", "
          << (s.usesRemove ? 1 : 0) << ", " << s.addType << ", " << (copyOut() ? 1 : 0) << ", "
          << (ensembleStep(s) ? "abl_launch_ens_" + n : std::string("nullptr"))
          << ", " << (s.usesRng ? 1 : 0) << ", " << (s.presorted ? 1 : 0) << ", " << s.outChanged
          << "u, " << (s.nearCacheable ? 1 : 0);
    if (s.nearMembersF32 || s.nearPosLo)
      *this << ", " << s.nearMembersF32 << "u, " << (s.nearPosLo ? 1 : 0);
    *this << "},";
  }
  if (steps.empty()) *this << nl << "{nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0, 0},";
  *this << outdent << nl << "};" << nl;
  // The runtime runs the steps in simulate order (SimulateStatement::stepFuncDecls,
  // CPrinter.cpp:196); abl_steps above is in declaration order.
  *this << "static const abl_step_desc abl_steps_ordered[] = {" << indent;
  if (script.simStmt) {
    for (AST::FunctionDeclaration *f : script.simStmt->stepFuncDecls) {
      for (size_t k = 0; k < steps.size(); k++) {
        if (steps[k].decl == f) *this << nl << "abl_steps[" << (int) k << "],";
      }
    }
  }
  *this << nl << "{nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0}" << outdent
        << nl << "};" << nl;
  int numSteps = 0;
  if (script.simStmt) numSteps = (int) script.simStmt->stepFuncDecls.size();
  *this << "extern const abl_model_desc abl_desc = {" << indent << nl
        << "\"" << modelName << "\", " << (int) script.agents.size() << ", abl_agents, "
        << numSteps << ", abl_steps_ordered, sizeof(abl_globals), &abl_globals_default, "
        << scalarConsts << ", abl_global_table, " << envDim
        << ", abl_env_bounds, " << (granE ? "abl_granularity" : "nullptr") << ", "
        << (useFloat ? 1 : 0) << ", "
        << (seqStep ? "abl_seq_" + seqStep->name : std::string("nullptr")) << ", "
        << (ensembleModel() ? "abl_persist_launch_" + modelName : std::string("nullptr"))
        << outdent << nl << "};" << nl;
}

void CudaPrinter::print(const AST::Script &) {
  *this << "// Generated by OpenABL -b cuda (model \"" << modelName << "\")." << nl
        << "#include \"abl_gen.cuh\"" << nl << nl
        << "namespace abl_model_" << modelName << " {" << nl << nl
        << "typedef " << (useFloat ? "float" : "double") << " abl_float;" << nl
        << "#include \"abl_math.cuh\"" << nl << nl;
  for (AST::AgentDeclaration *decl : script.agents) *this << *decl << nl;
  *this << "struct agent_struct {" << indent;
  for (AST::AgentDeclaration *decl : script.agents) {
    *this << nl << "dyn_array agents_" << decl->name << ";" << nl << "dyn_array agents_"
          << decl->name << "_dbuf;";
  }
  *this << outdent << nl << "};" << nl << "static struct agent_struct agents;" << nl
        << "static const agent_info agents_info[] = {" << indent << nl;
  for (AST::AgentDeclaration *decl : script.agents) {
    *this << "{ " << decl->name << "_info, offsetof(struct agent_struct, agents_" << decl->name
          << "), \"" << decl->name << "\" }," << nl;
  }
  *this << "{ NULL, 0, NULL }" << outdent << nl << "};" << nl << nl;
  printGlobals();
  *this << "static abl::rng abl_R;  // unused on the host: main() draws from the host stream" << nl;
  for (AST::AgentDeclaration *a : script.agents) {
    *this << "struct abl_cols_" << a->name << " {" << indent;
    for (const AST::AgentMemberPtr &m : *a->members) {
      *this << nl << cType(m->type->resolved) << " *" << m->name << ";";
    }
    *this << outdent << nl << "};" << nl;
  }
  // add() inside a step: the child is staged at its parent's index and
  // appended to the population after the step (abl_runtime.cu).
  if (script.usesRuntimeAddition) {
    for (AST::AgentDeclaration *a : script.agents) {
      *this << "__device__ static void abl_add_" << a->name << "(abl::step_ctx &K, const "
            << a->name << " &c) {" << indent << nl << "K.added = 1;";
      for (size_t k = 0; k < a->members->size(); k++) {
        const AST::AgentMember &m = *(*a->members)[k];
        *this << nl << "((" << cType(m.type->resolved) << " *) K.child_cols[" << (int) k
              << "])[K.self] = c." << m.name << ";";
      }
      *this << outdent << nl << "}" << nl;
    }
  }
  *this << nl;
  const AST::FunctionDeclaration *mainDecl = nullptr;
  for (AST::FunctionDeclaration *decl : script.funcs) {
    if (decl->isMain()) {
      mainDecl = decl;
      continue;
    }
    *this << *decl << nl;
  }
  *this << nl;
  if (deviceInit && mainDecl) findDeviceInit(*mainDecl);
  const bool persist = ensembleModel();
  *this << "#ifndef ABL_PERSIST" << nl;
  printDeviceInit();
  if (persist) {
    *this << "extern \"C\" int abl_persist_launch_" << modelName
          << "(const void *, int *, int, size_t, int *, cudaStream_t);" << nl;
  }
  printDescriptor();
  if (mainDecl) {
    printHostSimulate();
    *this << *mainDecl << nl;
  }
  *this << "#else" << nl;
  if (persist) printPersistentKernel();
  *this << "#endif" << nl;
  *this << nl << "}  // namespace abl_model_" << modelName << nl << nl;
  if (persist) {
    *this << "#ifdef ABL_PERSIST" << nl << "extern \"C\" int abl_persist_launch_" << modelName
          << "(const void *abl_prog, int *abl_err, int abl_block, size_t abl_smem, int *abl_grid, "
             "cudaStream_t abl_stream) {" << indent << nl
          << "return abl::persist_launch((const void *) abl_model_" << modelName
          << "::abl_kernel_ens_persist, abl_prog, abl_err, abl_block, abl_smem, abl_grid, "
             "abl_stream);" << outdent << nl << "}" << nl << "#endif" << nl;
  }
  *this << "#ifndef ABL_PERSIST" << nl
        << "extern \"C\" const abl_model_desc *abl_model_desc_" << modelName << "(void) {"
        << indent << nl << "return &abl_model_" << modelName << "::abl_desc;" << outdent << nl
        << "}" << nl << "#endif" << nl;
  if (mainDecl) {
    *this << nl << "#if defined(ABL_STANDALONE_MAIN) && !defined(ABL_PERSIST)" << nl
          << "extern \"C\" const abl_model_desc *const abl_builtin_models[] = {" << nl
          << "    &abl_model_" << modelName << "::abl_desc, nullptr};" << nl
          << "int main() { return abl_model_" << modelName << "::abl_main(); }" << nl
          << "#endif" << nl;
  }
}

}  // namespace OpenABL
