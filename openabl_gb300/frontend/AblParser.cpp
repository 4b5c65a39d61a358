// Hand-written lexer and recursive-descent parser for the ABL language.
//
// The reference compiler generates its scanner and parser with flex and bison
// from src/Lexer.l and src/Parser.y.  Neither tool is part of this build
// environment, so this file implements the same token set and the same
// grammar directly, producing the identical OpenABL::AST node tree through the
// node constructors declared in src/AST.hpp.  Everything after parsing
// (analysis, the backends, the driver) is the reference code, unchanged.
//
// Behaviour kept deliberately identical to the generated code:
//   * tokens, keywords and the longest-match rules of src/Lexer.l:57-160,
//     including "0..n" lexing as INT DOTDOT (Lexer.l:79-83);
//   * operator precedence and associativity of src/Parser.y:108-127 (C-like,
//     ternary right-associative, ".." non-associative, unary ops binding
//     tighter than binary ops but looser than "." and "[]");
//   * source locations: the scanner's running location is stepped at the
//     start of every token, after blanks and after a block comment, but NOT
//     after newlines or line comments (Lexer.l:57-60, 150-160), so a token at
//     column 1 of a line inherits the begin line of the preceding blank
//     region.  A rule's location spans its first to its last symbol and an
//     empty rule sits at the end of the previous token, as bison's default
//     location action does.  Diagnostics print `loc.begin.line`, so the
//     reference's lint goldens (test/*.exp) depend on these rules.
#include <cctype>
#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ParserContext.hpp"

namespace OpenABL {

using namespace AST;

namespace {

enum class Tok {
  END, AGENT, BREAK, CONTINUE, ELSE, ENVIRONMENT, IF, FOR, NEW, PARAM, POSITION,
  RETURN, SEQUENTIAL, SIMULATE, STEP, WHILE,
  ADD, SUB, MUL, DIV, MOD, BITWISE_AND, BITWISE_XOR, BITWISE_OR, SHIFT_LEFT,
  SHIFT_RIGHT, NOT, BITWISE_NOT, QM, DOT, DOTDOT, COMMA, COLON, SEMI, LPAREN,
  RPAREN, LBRACKET, RBRACKET, LBRACE, RBRACE, ASSIGN, ARROW, EQUALS, NOT_EQUALS,
  SMALLER, GREATER, SMALLER_EQUALS, GREATER_EQUALS, LOGICAL_AND, LOGICAL_OR,
  ADD_ASSIGN, SUB_ASSIGN, MUL_ASSIGN, DIV_ASSIGN, MOD_ASSIGN, BITWISE_AND_ASSIGN,
  BITWISE_XOR_ASSIGN, BITWISE_OR_ASSIGN, SHIFT_LEFT_ASSIGN, SHIFT_RIGHT_ASSIGN,
  BOOL, INT, FLOAT, STRING, IDENTIFIER,
};

const char *tokName(Tok t) {
  switch (t) {
    case Tok::END: return "\"end of file\"";
    case Tok::AGENT: return "AGENT";
    case Tok::BREAK: return "BREAK";
    case Tok::CONTINUE: return "CONTINUE";
    case Tok::ELSE: return "ELSE";
    case Tok::ENVIRONMENT: return "ENVIRONMENT";
    case Tok::IF: return "IF";
    case Tok::FOR: return "FOR";
    case Tok::NEW: return "NEW";
    case Tok::PARAM: return "PARAM";
    case Tok::POSITION: return "POSITION";
    case Tok::RETURN: return "RETURN";
    case Tok::SEQUENTIAL: return "SEQUENTIAL";
    case Tok::SIMULATE: return "SIMULATE";
    case Tok::STEP: return "STEP";
    case Tok::WHILE: return "WHILE";
    case Tok::ADD: return "ADD";
    case Tok::SUB: return "SUB";
    case Tok::MUL: return "MUL";
    case Tok::DIV: return "DIV";
    case Tok::MOD: return "MOD";
    case Tok::BITWISE_AND: return "BITWISE_AND";
    case Tok::BITWISE_XOR: return "BITWISE_XOR";
    case Tok::BITWISE_OR: return "BITWISE_OR";
    case Tok::SHIFT_LEFT: return "SHIFT_LEFT";
    case Tok::SHIFT_RIGHT: return "SHIFT_RIGHT";
    case Tok::NOT: return "NOT";
    case Tok::BITWISE_NOT: return "BITWISE_NOT";
    case Tok::QM: return "QM";
    case Tok::DOT: return "DOT";
    case Tok::DOTDOT: return "DOTDOT";
    case Tok::COMMA: return "COMMA";
    case Tok::COLON: return "COLON";
    case Tok::SEMI: return "SEMI";
    case Tok::LPAREN: return "LPAREN";
    case Tok::RPAREN: return "RPAREN";
    case Tok::LBRACKET: return "LBRACKET";
    case Tok::RBRACKET: return "RBRACKET";
    case Tok::LBRACE: return "LBRACE";
    case Tok::RBRACE: return "RBRACE";
    case Tok::ASSIGN: return "ASSIGN";
    case Tok::ARROW: return "ARROW";
    case Tok::EQUALS: return "EQUALS";
    case Tok::NOT_EQUALS: return "NOT_EQUALS";
    case Tok::SMALLER: return "SMALLER";
    case Tok::GREATER: return "GREATER";
    case Tok::SMALLER_EQUALS: return "SMALLER_EQUALS";
    case Tok::GREATER_EQUALS: return "GREATER_EQUALS";
    case Tok::LOGICAL_AND: return "LOGICAL_AND";
    case Tok::LOGICAL_OR: return "LOGICAL_OR";
    case Tok::ADD_ASSIGN: return "ADD_ASSIGN";
    case Tok::SUB_ASSIGN: return "SUB_ASSIGN";
    case Tok::MUL_ASSIGN: return "MUL_ASSIGN";
    case Tok::DIV_ASSIGN: return "DIV_ASSIGN";
    case Tok::MOD_ASSIGN: return "MOD_ASSIGN";
    case Tok::BITWISE_AND_ASSIGN: return "BITWISE_AND_ASSIGN";
    case Tok::BITWISE_XOR_ASSIGN: return "BITWISE_XOR_ASSIGN";
    case Tok::BITWISE_OR_ASSIGN: return "BITWISE_OR_ASSIGN";
    case Tok::SHIFT_LEFT_ASSIGN: return "SHIFT_LEFT_ASSIGN";
    case Tok::SHIFT_RIGHT_ASSIGN: return "SHIFT_RIGHT_ASSIGN";
    case Tok::BOOL: return "BOOL";
    case Tok::INT: return "INT";
    case Tok::FLOAT: return "FLOAT";
    case Tok::STRING: return "STRING";
    case Tok::IDENTIFIER: return "IDENTIFIER";
  }
  return "?";
}

struct Token {
  Tok kind;
  location loc;
  std::string text;  // IDENTIFIER name or decoded STRING contents
  long ival = 0;
  double fval = 0;
  bool bval = false;
};

// ---------------------------------------------------------------- scanner

class Scanner {
public:
  explicit Scanner(std::string src) : s(std::move(src)) {}

  std::vector<Token> run() {
    std::vector<Token> out;
    for (;;) {
      Token t = next();
      out.push_back(t);
      if (t.kind == Tok::END) break;
    }
    return out;
  }

private:
  std::string s;
  size_t p = 0;
  location loc;        // the scanner's running location (Lexer.l:24)
  bool inComment = false;

  char at(size_t i) const { return i < s.size() ? s[i] : '\0'; }
  static bool isIdStart(char c) { return std::isalpha((unsigned char) c) || c == '_'; }
  static bool isIdChar(char c) { return std::isalnum((unsigned char) c) || c == '_'; }
  static bool isDigit(char c) { return c >= '0' && c <= '9'; }
  static bool isHex(char c) { return std::isxdigit((unsigned char) c) != 0; }

  Token make(Tok k) {
    Token t;
    t.kind = k;
    t.loc = loc;
    return t;
  }

  // Consumes `len` characters as one match; the per-match column update of
  // YY_USER_ACTION (Lexer.l:26) is applied by the caller.
  void eat(size_t len) { p += len; }

  size_t digitsAt(size_t i) const {
    size_t n = 0;
    while (isDigit(at(i + n))) ++n;
    return n;
  }

  // Length of the FLOAT pattern starting at p (0 if it does not match).
  size_t floatLen() const {
    size_t i = p;
    size_t d = digitsAt(i);
    if (d > 0) {
      if (at(i + d) != '.') return 0;
      i += d + 1;
      i += digitsAt(i);
    } else {
      if (at(i) != '.') return 0;
      size_t d2 = digitsAt(i + 1);
      if (d2 == 0) return 0;
      i += 1 + d2;
    }
    if (at(i) == 'e' || at(i) == 'E') {
      size_t j = i + 1;
      if (at(j) == '+' || at(j) == '-') ++j;
      size_t d3 = digitsAt(j);
      if (d3 > 0) i = j + d3;
    }
    return i - p;
  }

  Token next() {
    loc.step();
    for (;;) {
      if (p >= s.size()) return make(Tok::END);
      if (inComment) {
        scanComment();
        continue;
      }
      char c = s[p];
      if (c == ' ' || c == '\t' || c == '\r') {
        size_t n = 0;
        while (at(p + n) == ' ' || at(p + n) == '\t' || at(p + n) == '\r') ++n;
        loc.columns((int) n);
        eat(n);
        loc.step();
        continue;
      }
      if (c == '\n') {
        size_t n = 0;
        while (at(p + n) == '\n') ++n;
        loc.columns((int) n);
        loc.lines((int) n);
        eat(n);
        continue;
      }
      if (c == '/' && at(p + 1) == '/') {
        size_t n = 0;
        while (p + n < s.size() && s[p + n] != '\n') ++n;
        loc.columns((int) n);
        eat(n);
        continue;
      }
      if (c == '/' && at(p + 1) == '*') {
        loc.columns(2);
        eat(2);
        inComment = true;
        continue;
      }
      if (isIdStart(c)) return scanWord();
      if (isDigit(c) || (c == '.' && isDigit(at(p + 1)))) return scanNumber();
      if (c == '"') {
        Token t;
        if (scanString(t)) return t;
      }
      Token op;
      if (scanOperator(op)) return op;
      // No rule matches: flex's default rule echoes the character.
      std::fputc(c, stdout);
      loc.columns(1);
      eat(1);
    }
  }

  // <ST_COMMENT> rules of Lexer.l:150-154, with flex's longest-match choice.
  void scanComment() {
    char c = s[p];
    if (c == '\n') {
      size_t n = 0;
      while (at(p + n) == '\n') ++n;
      loc.columns((int) n);
      loc.lines((int) n);
      eat(n);
    } else if (c == '*') {
      if (at(p + 1) == '/') {
        loc.columns(2);
        eat(2);
        loc.step();
        inComment = false;
      } else {
        size_t n = 0;
        while (at(p + n) == '*') ++n;
        while (p + n < s.size() && s[p + n] != '*' && s[p + n] != '/' && s[p + n] != '\n') ++n;
        loc.columns((int) n);
        eat(n);
      }
    } else {
      size_t n = 0;
      while (p + n < s.size() && s[p + n] != '*' && s[p + n] != '\n') ++n;
      loc.columns((int) n);
      eat(n);
    }
  }

  Token scanWord() {
    size_t n = 0;
    while (isIdChar(at(p + n))) ++n;
    std::string w = s.substr(p, n);
    loc.columns((int) n);
    eat(n);
    static const struct { const char *kw; Tok tok; } kws[] = {
      {"agent", Tok::AGENT}, {"break", Tok::BREAK}, {"continue", Tok::CONTINUE},
      {"else", Tok::ELSE}, {"environment", Tok::ENVIRONMENT}, {"if", Tok::IF},
      {"for", Tok::FOR}, {"new", Tok::NEW}, {"param", Tok::PARAM},
      {"position", Tok::POSITION}, {"return", Tok::RETURN},
      {"sequential", Tok::SEQUENTIAL}, {"simulate", Tok::SIMULATE},
      {"step", Tok::STEP}, {"while", Tok::WHILE},
    };
    for (const auto &k : kws) {
      if (w == k.kw) return make(k.tok);
    }
    if (w == "true" || w == "false") {
      Token t = make(Tok::BOOL);
      t.bval = (w == "true");
      return t;
    }
    Token t = make(Tok::IDENTIFIER);
    t.text = w;
    return t;
  }

  Token scanNumber() {
    // Candidate matches: DNUM, HNUM, FLOAT, DNUM".." (in rule order).
    size_t dnum = digitsAt(p);
    size_t hnum = 0;
    if (at(p) == '0' && (at(p + 1) == 'x' || at(p + 1) == 'X') && isHex(at(p + 2))) {
      hnum = 2;
      while (isHex(at(p + hnum))) ++hnum;
    }
    size_t flt = floatLen();
    size_t range = (dnum > 0 && at(p + dnum) == '.' && at(p + dnum + 1) == '.') ? dnum + 2 : 0;

    size_t best = dnum;
    int rule = 0;
    if (hnum > best) { best = hnum; rule = 1; }
    if (flt > best) { best = flt; rule = 2; }
    if (range > best) { best = range; rule = 3; }

    std::string text = s.substr(p, best);
    loc.columns((int) best);
    if (rule == 3) {
      // yyless(yyleng - 2): hand the ".." back to the scanner.
      text = s.substr(p, dnum);
      eat(dnum);
    } else {
      eat(best);
    }
    if (rule == 2) {
      Token t = make(Tok::FLOAT);
      t.fval = std::stod(text, nullptr);
      return t;
    }
    Token t = make(Tok::INT);
    t.ival = std::stol(text, nullptr, rule == 1 ? 16 : 10);
    return t;
  }

  bool scanString(Token &out) {
    size_t i = p + 1;
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\' && i + 1 < s.size()) i += 2;
      else ++i;
    }
    if (i >= s.size()) return false;
    size_t len = i + 1 - p;
    std::string result;
    for (size_t k = p + 1; k < i; k++) {
      char c = s[k];
      if (c == '\\') result.push_back(s[++k]);
      else result.push_back(c);
    }
    loc.columns((int) len);
    eat(len);
    out = make(Tok::STRING);
    out.text = result;
    return true;
  }

  bool scanOperator(Token &out) {
    static const struct { const char *op; Tok tok; } ops[] = {
      {"<<=", Tok::SHIFT_LEFT_ASSIGN}, {">>=", Tok::SHIFT_RIGHT_ASSIGN},
      {"..", Tok::DOTDOT}, {"->", Tok::ARROW}, {"==", Tok::EQUALS},
      {"!=", Tok::NOT_EQUALS}, {"<=", Tok::SMALLER_EQUALS},
      {">=", Tok::GREATER_EQUALS}, {"<<", Tok::SHIFT_LEFT}, {">>", Tok::SHIFT_RIGHT},
      {"&&", Tok::LOGICAL_AND}, {"||", Tok::LOGICAL_OR}, {"+=", Tok::ADD_ASSIGN},
      {"-=", Tok::SUB_ASSIGN}, {"*=", Tok::MUL_ASSIGN}, {"/=", Tok::DIV_ASSIGN},
      {"%=", Tok::MOD_ASSIGN}, {"&=", Tok::BITWISE_AND_ASSIGN},
      {"^=", Tok::BITWISE_XOR_ASSIGN}, {"|=", Tok::BITWISE_OR_ASSIGN},
      {"+", Tok::ADD}, {"-", Tok::SUB}, {"*", Tok::MUL}, {"/", Tok::DIV},
      {"%", Tok::MOD}, {"&", Tok::BITWISE_AND}, {"^", Tok::BITWISE_XOR},
      {"|", Tok::BITWISE_OR}, {"=", Tok::ASSIGN}, {"!", Tok::NOT},
      {"~", Tok::BITWISE_NOT}, {"?", Tok::QM}, {".", Tok::DOT}, {",", Tok::COMMA},
      {":", Tok::COLON}, {";", Tok::SEMI}, {"<", Tok::SMALLER}, {">", Tok::GREATER},
      {"(", Tok::LPAREN}, {")", Tok::RPAREN}, {"[", Tok::LBRACKET},
      {"]", Tok::RBRACKET}, {"{", Tok::LBRACE}, {"}", Tok::RBRACE},
    };
    for (const auto &o : ops) {
      size_t n = std::char_traits<char>::length(o.op);
      if (s.compare(p, n, o.op) == 0) {
        loc.columns((int) n);
        eat(n);
        out = make(o.tok);
        return true;
      }
    }
    return false;
  }
};

// ----------------------------------------------------------------- parser

struct SyntaxError : std::runtime_error {
  SyntaxError(const std::string &m, location l) : std::runtime_error(m), loc(l) {}
  location loc;
};

// An expression together with the source span of the grammar symbol that
// produced it.  For "( e )" the node keeps e's own location while the span
// covers the parentheses, as Parser.y:308 passes $2 through unchanged.
struct Spanned {
  Expression *expr;
  location span;
};

class RDParser {
public:
  explicit RDParser(std::vector<Token> toks) : t(std::move(toks)) {}

  Script *parseScript() {
    position start = prevEnd;
    auto *decls = new DeclarationList();
    location first, last;
    bool any = false;
    while (peek().kind != Tok::END) {
      Declaration *d = parseDeclaration();
      if (!any) first = d->loc;
      last = d->loc;
      any = true;
      decls->emplace_back(d);
    }
    location l = any ? location(first.begin, last.end) : location(start, start);
    return new Script(decls, l);
  }

private:
  std::vector<Token> t;
  size_t i = 0;
  position prevEnd;  // end of the last consumed token (initially 1.1)

  const Token &peek(size_t k = 0) const {
    size_t j = i + k;
    return j < t.size() ? t[j] : t.back();
  }
  Token take() {
    Token tok = t[i];
    if (i + 1 < t.size()) ++i;
    prevEnd = tok.loc.end;
    return tok;
  }
  bool accept(Tok k) {
    if (peek().kind == k) {
      take();
      return true;
    }
    return false;
  }
  [[noreturn]] void fail() {
    const Token &tok = peek();
    throw SyntaxError(std::string("syntax error, unexpected ") + tokName(tok.kind), tok.loc);
  }
  Token expect(Tok k) {
    if (peek().kind != k) fail();
    return take();
  }
  static location span(const location &a, const location &b) {
    return location(a.begin, b.end);
  }

  // ---- declarations (Parser.y:170-247)

  Declaration *parseDeclaration() {
    const Token &tok = peek();
    switch (tok.kind) {
      case Tok::AGENT: return parseAgent();
      case Tok::ENVIRONMENT: return parseEnvironment();
      case Tok::PARAM: {
        Token kw = take();
        return parseConst(kw.loc, true);
      }
      case Tok::STEP: {
        Token kw = take();
        return parseFunction(nullptr, kw.loc, FunctionDeclaration::STEP);
      }
      case Tok::SEQUENTIAL: {
        Token kw = take();
        Token st = expect(Tok::STEP);
        return parseFunction(nullptr, span(kw.loc, st.loc), FunctionDeclaration::SEQ_STEP);
      }
      case Tok::IDENTIFIER:
        if (peek(1).kind == Tok::IDENTIFIER && peek(2).kind == Tok::LPAREN) {
          AST::Type *type = parseType();
          return parseFunction(type, type->loc, FunctionDeclaration::NORMAL);
        }
        return parseConst(tok.loc, false);
      default:
        fail();
    }
  }

  AgentDeclaration *parseAgent() {
    Token kw = take();
    Token name = expect(Tok::IDENTIFIER);
    expect(Tok::LBRACE);
    auto *members = new AgentMemberList();
    while (peek().kind != Tok::RBRACE) {
      // agent_member: opt_position type IDENTIFIER SEMI; an empty
      // opt_position is located at the end of the previous token.
      position begin = prevEnd;
      bool isPos = false;
      if (peek().kind == Tok::POSITION) {
        begin = peek().loc.begin;
        take();
        isPos = true;
      }
      AST::Type *type = parseType();
      Token mname = expect(Tok::IDENTIFIER);
      Token semi = expect(Tok::SEMI);
      members->emplace_back(new AgentMember(isPos, type, mname.text,
                                            location(begin, semi.loc.end)));
    }
    Token rb = take();
    return new AgentDeclaration(name.text, members, span(kw.loc, rb.loc));
  }

  EnvironmentDeclaration *parseEnvironment() {
    Token kw = take();
    expect(Tok::LBRACE);
    MemberInitList *members = parseMemberInitList();
    Token rb = expect(Tok::RBRACE);
    return new EnvironmentDeclaration(members, span(kw.loc, rb.loc));
  }

  ConstDeclaration *parseConst(location begin, bool isParam) {
    AST::Type *type = parseType();
    Var *var = parseVar();
    bool isArray = false;
    if (peek().kind == Tok::LBRACKET) {
      take();
      expect(Tok::RBRACKET);
      isArray = true;
    }
    expect(Tok::ASSIGN);
    Expression *init;
    if (peek().kind == Tok::LBRACE) {
      init = parseArrayInitializer();
    } else {
      init = parseExpression().expr;
    }
    Token semi = expect(Tok::SEMI);
    return new ConstDeclaration(type, var, init, isArray, isParam, span(begin, semi.loc));
  }

  Expression *parseArrayInitializer() {
    Token lb = take();
    auto *exprs = new ExpressionList();
    exprs->emplace_back(parseExpression().expr);
    while (peek().kind == Tok::COMMA) {
      take();
      if (peek().kind == Tok::RBRACE) break;  // opt_comma
      exprs->emplace_back(parseExpression().expr);
    }
    Token rb = expect(Tok::RBRACE);
    return new ArrayInitExpression(exprs, span(lb.loc, rb.loc));
  }

  FunctionDeclaration *parseFunction(AST::Type *returnType, location begin,
                                     FunctionDeclaration::Kind kind) {
    Token name = expect(Tok::IDENTIFIER);
    expect(Tok::LPAREN);
    auto *params = new ParamList();
    if (peek().kind != Tok::RPAREN) {
      params->emplace_back(parseParam());
      while (accept(Tok::COMMA)) params->emplace_back(parseParam());
    }
    expect(Tok::RPAREN);
    expect(Tok::LBRACE);
    StatementList *stmts = parseStatementList();
    Token rb = expect(Tok::RBRACE);
    if (!returnType) returnType = new SimpleType("void", Location{});
    return new FunctionDeclaration(returnType, name.text, params, stmts, kind,
                                   span(begin, rb.loc));
  }

  Param *parseParam() {
    AST::Type *type = parseType();
    Var *var = parseVar();
    Var *out = nullptr;
    location end = var->loc;
    if (peek().kind == Tok::ARROW) {
      take();
      out = parseVar();
      end = out->loc;
    }
    return new Param(type, var, out, span(type->loc, end));
  }

  AST::Type *parseType() {
    Token id = expect(Tok::IDENTIFIER);
    return new SimpleType(id.text, id.loc);
  }

  Var *parseVar() {
    Token id = expect(Tok::IDENTIFIER);
    return new Var(id.text, id.loc);
  }

  MemberInitList *parseMemberInitList() {
    auto *list = new MemberInitList();
    if (peek().kind == Tok::RBRACE) return list;
    list->emplace_back(parseMemberInitEntry());
    while (peek().kind == Tok::COMMA) {
      take();
      if (peek().kind == Tok::RBRACE) break;  // optional_comma
      list->emplace_back(parseMemberInitEntry());
    }
    return list;
  }

  MemberInitEntry *parseMemberInitEntry() {
    Token name = expect(Tok::IDENTIFIER);
    expect(Tok::COLON);
    Spanned e = parseExpression();
    return new MemberInitEntry(name.text, e.expr, span(name.loc, e.span));
  }

  // ---- statements (Parser.y:257-303)

  StatementList *parseStatementList() {
    auto *list = new StatementList();
    while (peek().kind != Tok::RBRACE && peek().kind != Tok::END) {
      list->emplace_back(parseStatement());
    }
    return list;
  }

  Statement *parseStatement() {
    const Token &tok = peek();
    switch (tok.kind) {
      case Tok::LBRACE: {
        Token lb = take();
        StatementList *stmts = parseStatementList();
        Token rb = expect(Tok::RBRACE);
        return new BlockStatement(stmts, span(lb.loc, rb.loc));
      }
      case Tok::IF: {
        Token kw = take();
        expect(Tok::LPAREN);
        Expression *cond = parseExpression().expr;
        expect(Tok::RPAREN);
        Statement *ifStmt = parseStatement();
        Statement *elseStmt = nullptr;
        location end = ifStmt->loc;
        // The dangling else binds to the nearest if (Parser.y:123-125).
        if (peek().kind == Tok::ELSE) {
          take();
          elseStmt = parseStatement();
          end = elseStmt->loc;
        }
        return new IfStatement(cond, ifStmt, elseStmt, location(kw.loc.begin, lastEnd(end)));
      }
      case Tok::FOR: {
        Token kw = take();
        expect(Tok::LPAREN);
        AST::Type *type = parseType();
        Var *var = parseVar();
        expect(Tok::COLON);
        Expression *expr = parseExpression().expr;
        expect(Tok::RPAREN);
        Statement *body = parseStatement();
        return new ForStatement(type, var, expr, body, location(kw.loc.begin, prevEnd));
      }
      case Tok::WHILE: {
        Token kw = take();
        expect(Tok::LPAREN);
        Expression *cond = parseExpression().expr;
        expect(Tok::RPAREN);
        Statement *body = parseStatement();
        return new WhileStatement(cond, body, location(kw.loc.begin, prevEnd));
      }
      case Tok::RETURN: {
        Token kw = take();
        Expression *e = nullptr;
        if (peek().kind != Tok::SEMI) e = parseExpression().expr;
        Token semi = expect(Tok::SEMI);
        return new ReturnStatement(e, span(kw.loc, semi.loc));
      }
      case Tok::BREAK: {
        Token kw = take();
        Token semi = expect(Tok::SEMI);
        return new BreakStatement(span(kw.loc, semi.loc));
      }
      case Tok::CONTINUE: {
        Token kw = take();
        Token semi = expect(Tok::SEMI);
        return new ContinueStatement(span(kw.loc, semi.loc));
      }
      case Tok::SIMULATE: {
        Token kw = take();
        expect(Tok::LPAREN);
        Expression *steps = parseExpression().expr;
        expect(Tok::RPAREN);
        expect(Tok::LBRACE);
        auto *idents = new IdentList();
        idents->push_back(expect(Tok::IDENTIFIER).text);
        while (peek().kind == Tok::COMMA) {
          take();
          if (peek().kind == Tok::RBRACE) break;  // optional_comma
          idents->push_back(expect(Tok::IDENTIFIER).text);
        }
        Token rb = expect(Tok::RBRACE);
        return new SimulateStatement(steps, idents, span(kw.loc, rb.loc));
      }
      case Tok::IDENTIFIER:
        if (peek(1).kind == Tok::IDENTIFIER) {
          AST::Type *type = parseType();
          Var *var = parseVar();
          Expression *init = nullptr;
          if (peek().kind == Tok::ASSIGN) {
            take();
            init = parseExpression().expr;
          }
          Token semi = expect(Tok::SEMI);
          return new VarDeclarationStatement(type, var, init, span(type->loc, semi.loc));
        }
        break;
      default:
        break;
    }

    Spanned left = parseExpression();
    Tok k = peek().kind;
    if (k == Tok::SEMI) {
      Token semi = take();
      return new ExpressionStatement(left.expr, span(left.span, semi.loc));
    }
    if (k == Tok::ASSIGN) {
      take();
      Expression *right = parseExpression().expr;
      Token semi = expect(Tok::SEMI);
      return new AssignStatement(left.expr, right, span(left.span, semi.loc));
    }
    BinaryOp op;
    switch (k) {
      case Tok::ADD_ASSIGN: op = BinaryOp::ADD; break;
      case Tok::SUB_ASSIGN: op = BinaryOp::SUB; break;
      case Tok::MUL_ASSIGN: op = BinaryOp::MUL; break;
      case Tok::DIV_ASSIGN: op = BinaryOp::DIV; break;
      case Tok::MOD_ASSIGN: op = BinaryOp::MOD; break;
      case Tok::BITWISE_AND_ASSIGN: op = BinaryOp::BITWISE_AND; break;
      case Tok::BITWISE_XOR_ASSIGN: op = BinaryOp::BITWISE_XOR; break;
      case Tok::BITWISE_OR_ASSIGN: op = BinaryOp::BITWISE_OR; break;
      case Tok::SHIFT_LEFT_ASSIGN: op = BinaryOp::SHIFT_LEFT; break;
      case Tok::SHIFT_RIGHT_ASSIGN: op = BinaryOp::SHIFT_RIGHT; break;
      default: fail();
    }
    take();
    Expression *right = parseExpression().expr;
    Token semi = expect(Tok::SEMI);
    return new AssignOpStatement(op, left.expr, right, span(left.span, semi.loc));
  }

  // The location of a nested statement ends where its last token ends.
  position lastEnd(const location &) const { return prevEnd; }

  // ---- expressions (Parser.y:305-367)

  Spanned parseExpression() { return parseTernary(); }

  // expression QM expression COLON expression, right-associative at the
  // lowest expression precedence (Parser.y:109).
  Spanned parseTernary() {
    Spanned cond = parseBinary(1);
    if (peek().kind != Tok::QM) return cond;
    take();
    Spanned ifE = parseExpression();
    expect(Tok::COLON);
    Spanned elseE = parseTernary();
    location l = span(cond.span, elseE.span);
    return { new TernaryExpression(cond.expr, ifE.expr, elseE.expr, l), l };
  }

  // Binary precedence levels, lowest first (Parser.y:110-121).
  static int binaryLevel(Tok k, BinaryOp &op) {
    switch (k) {
      case Tok::LOGICAL_OR: op = BinaryOp::LOGICAL_OR; return 1;
      case Tok::LOGICAL_AND: op = BinaryOp::LOGICAL_AND; return 2;
      case Tok::BITWISE_OR: op = BinaryOp::BITWISE_OR; return 3;
      case Tok::BITWISE_XOR: op = BinaryOp::BITWISE_XOR; return 4;
      case Tok::BITWISE_AND: op = BinaryOp::BITWISE_AND; return 5;
      case Tok::EQUALS: op = BinaryOp::EQUALS; return 6;
      case Tok::NOT_EQUALS: op = BinaryOp::NOT_EQUALS; return 6;
      case Tok::SMALLER: op = BinaryOp::SMALLER; return 7;
      case Tok::SMALLER_EQUALS: op = BinaryOp::SMALLER_EQUALS; return 7;
      case Tok::GREATER: op = BinaryOp::GREATER; return 7;
      case Tok::GREATER_EQUALS: op = BinaryOp::GREATER_EQUALS; return 7;
      case Tok::DOTDOT: op = BinaryOp::RANGE; return 8;
      case Tok::SHIFT_LEFT: op = BinaryOp::SHIFT_LEFT; return 9;
      case Tok::SHIFT_RIGHT: op = BinaryOp::SHIFT_RIGHT; return 9;
      case Tok::ADD: op = BinaryOp::ADD; return 10;
      case Tok::SUB: op = BinaryOp::SUB; return 10;
      case Tok::MUL: op = BinaryOp::MUL; return 11;
      case Tok::DIV: op = BinaryOp::DIV; return 11;
      case Tok::MOD: op = BinaryOp::MOD; return 11;
      default: return 0;
    }
  }

  Spanned parseBinary(int minLevel) {
    Spanned left = parseUnary();
    for (;;) {
      BinaryOp op;
      int level = binaryLevel(peek().kind, op);
      if (level == 0 || level < minLevel) return left;
      take();
      Spanned right = parseBinary(level + 1);
      location l = span(left.span, right.span);
      left = { new BinaryOpExpression(op, left.expr, right.expr, l), l };
      // ".." is non-associative (Parser.y:118).
      if (op == BinaryOp::RANGE && peek().kind == Tok::DOTDOT) fail();
    }
  }

  Spanned parseUnary() {
    UnaryOp op;
    switch (peek().kind) {
      case Tok::NOT: op = UnaryOp::LOGICAL_NOT; break;
      case Tok::BITWISE_NOT: op = UnaryOp::BITWISE_NOT; break;
      case Tok::ADD: op = UnaryOp::PLUS; break;
      case Tok::SUB: op = UnaryOp::MINUS; break;
      default: return parsePostfix();
    }
    Token tok = take();
    Spanned operand = parseUnary();
    location l = span(tok.loc, operand.span);
    return { new UnaryOpExpression(op, operand.expr, l), l };
  }

  Spanned parsePostfix() {
    Spanned e = parsePrimary();
    for (;;) {
      if (peek().kind == Tok::DOT) {
        take();
        Token name = expect(Tok::IDENTIFIER);
        location l = span(e.span, name.loc);
        e = { new MemberAccessExpression(e.expr, name.text, l), l };
      } else if (peek().kind == Tok::LBRACKET) {
        take();
        Expression *off = parseExpression().expr;
        Token rb = expect(Tok::RBRACKET);
        location l = span(e.span, rb.loc);
        e = { new ArrayAccessExpression(e.expr, off, l), l };
      } else {
        return e;
      }
    }
  }

  Spanned parsePrimary() {
    Token tok = peek();
    switch (tok.kind) {
      case Tok::IDENTIFIER: {
        take();
        if (peek().kind == Tok::LPAREN) {
          take();
          auto *args = new ExpressionList();
          if (peek().kind != Tok::RPAREN) {
            args->emplace_back(parseExpression().expr);
            while (peek().kind == Tok::COMMA) {
              take();
              if (peek().kind == Tok::RPAREN) break;  // optional_comma
              args->emplace_back(parseExpression().expr);
            }
          }
          Token rp = expect(Tok::RPAREN);
          location l = span(tok.loc, rp.loc);
          return { new CallExpression(tok.text, args, l), l };
        }
        if (peek().kind == Tok::LBRACE) {
          take();
          MemberInitList *members = parseMemberInitList();
          Token rb = expect(Tok::RBRACE);
          location l = span(tok.loc, rb.loc);
          return { new AgentCreationExpression(tok.text, members, l), l };
        }
        return { new VarExpression(new Var(tok.text, tok.loc), tok.loc), tok.loc };
      }
      case Tok::ENVIRONMENT: {
        take();
        expect(Tok::DOT);
        Token name = expect(Tok::IDENTIFIER);
        location l = span(tok.loc, name.loc);
        return { new EnvironmentAccessExpression(name.text, l), l };
      }
      case Tok::BOOL:
        take();
        return { new BoolLiteral(tok.bval, tok.loc), tok.loc };
      case Tok::INT:
        take();
        return { new IntLiteral(tok.ival, tok.loc), tok.loc };
      case Tok::FLOAT:
        take();
        return { new FloatLiteral(tok.fval, tok.loc), tok.loc };
      case Tok::STRING:
        take();
        return { new StringLiteral(tok.text, tok.loc), tok.loc };
      case Tok::LPAREN: {
        take();
        Spanned inner = parseExpression();
        Token rp = expect(Tok::RPAREN);
        return { inner.expr, span(tok.loc, rp.loc) };
      }
      case Tok::NEW: {
        take();
        AST::Type *type = parseType();
        expect(Tok::LBRACKET);
        Expression *size = parseExpression().expr;
        Token rb = expect(Tok::RBRACKET);
        location l = span(tok.loc, rb.loc);
        return { new NewArrayExpression(type, size, l), l };
      }
      default:
        fail();
    }
  }
};

std::string readAll(FILE *f) {
  std::string out;
  char buf[65536];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
  return out;
}

}  // namespace

int Parser::parse() {
  std::vector<Token> toks = Scanner(readAll(ctx.file)).run();
  try {
    RDParser p(std::move(toks));
    ctx.script = p.parseScript();
    return 0;
  } catch (const SyntaxError &e) {
    std::cerr << "Parse error: " << e.what() << " on line " << e.loc.begin.line << std::endl;
    return 1;
  }
}

// The generated scanner attaches to the input file here (Lexer.l:166-170);
// this scanner reads ctx.file in Parser::parse() instead.
void ParserContext::initLexer() {}

}  // namespace OpenABL
