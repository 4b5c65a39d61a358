// Source positions for the OpenABL front end.
//
// The reference compiler takes `OpenABL::position` / `OpenABL::location` from
// the header that bison writes next to its generated parser (included by
// src/AST.hpp:21 and src/ErrorHandling.hpp:19).  Bison is not available in
// this build environment, so this header provides the same two classes with
// the same observable behaviour: lines and columns count from 1, `step()`
// moves the start of a location to its end, `columns(n)` advances the end
// column and `lines(n)` advances the end line and resets the column to 1.
// Diagnostics only ever read `loc.begin.line` (src/main.cpp:219).
#pragma once

#include <ostream>
#include <string>

namespace OpenABL {

class position {
public:
  typedef unsigned int counter_type;

  explicit position(std::string *f = nullptr, counter_type l = 1, counter_type c = 1)
    : filename(f), line(l), column(c) {}

  void initialize(std::string *f = nullptr, counter_type l = 1, counter_type c = 1) {
    filename = f;
    line = l;
    column = c;
  }

  void lines(int count = 1) {
    if (count) {
      column = 1;
      line = clamp_add(line, count);
    }
  }

  void columns(int count = 1) {
    column = clamp_add(column, count);
  }

  std::string *filename;
  counter_type line;
  counter_type column;

private:
  // Counters never drop below 1.
  static counter_type clamp_add(counter_type lhs, int rhs) {
    long v = static_cast<long>(lhs) + rhs;
    return v < 1 ? 1u : static_cast<counter_type>(v);
  }
};

inline bool operator==(const position &a, const position &b) {
  return a.line == b.line && a.column == b.column;
}
inline bool operator!=(const position &a, const position &b) { return !(a == b); }

inline std::ostream &operator<<(std::ostream &os, const position &pos) {
  if (pos.filename) os << *pos.filename << ':';
  return os << pos.line << '.' << pos.column;
}

class location {
public:
  location(const position &b, const position &e) : begin(b), end(e) {}
  explicit location(const position &p = position()) : begin(p), end(p) {}

  void initialize(std::string *f = nullptr, unsigned l = 1, unsigned c = 1) {
    begin.initialize(f, l, c);
    end = begin;
  }

  void step() { begin = end; }
  void columns(int count = 1) { end.columns(count); }
  void lines(int count = 1) { end.lines(count); }

  position begin;
  position end;
};

inline std::ostream &operator<<(std::ostream &os, const location &loc) {
  os << loc.begin;
  if (loc.end.line != loc.begin.line) {
    os << '-' << loc.end.line << '.' << (loc.end.column ? loc.end.column - 1 : 0);
  } else if (loc.end.column > loc.begin.column + 1) {
    os << '-' << (loc.end.column - 1);
  }
  return os;
}

}  // namespace OpenABL
