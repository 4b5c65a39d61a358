// Parser interface expected by the reference compiler's src/ParserContext.cpp:18-22
// (`Parser parser(ctx); parser.parse() == 0`).  In the reference this header is
// generated by bison from src/Parser.y; here it fronts a hand-written lexer and
// recursive-descent parser (AblParser.cpp) that builds the same AST::* nodes
// with the same source locations.
#pragma once

#include <cstdio>
#include <string>
#include "AST.hpp"

namespace OpenABL {

struct ParserContext;

class Parser {
public:
  explicit Parser(ParserContext &ctx) : ctx(ctx) {}

  // Parses ctx.file into ctx.script.  Returns 0 on success, 1 on a syntax
  // error (after printing "Parse error: ... on line N" to stderr, as
  // src/Parser.y:366-369 does).
  int parse();

private:
  ParserContext &ctx;
};

}  // namespace OpenABL
