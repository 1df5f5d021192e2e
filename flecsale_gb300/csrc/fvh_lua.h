// A small interpreter for the subset of Lua that FleCSALE's input files use
// (apps/hydro/2d/shock_box_2d.lua, apps/hydro/3d/shock_box_3d.lua, read by
// apps/hydro/inputs.h:100-135 through an embedded Lua state): global
// assignments of numbers, strings, nested tables and function literals; inside
// functions local variables, if/elseif/else, numeric for, while, return of
// several values and table constructors; arithmetic, comparison and logical
// operators with Lua's precedence; the math library functions an initial
// condition needs.  Host code only; it runs at setup, never in the time loop.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace fvh {
namespace lua {

struct Table;
struct Function;
struct Value;
using TablePtr = std::shared_ptr<Table>;
using FunctionPtr = std::shared_ptr<Function>;

struct Value {
  enum Kind { NIL, BOOL, NUMBER, STRING, TABLE, FUNCTION } kind = NIL;
  bool b = false;
  double n = 0;
  std::string s;
  TablePtr t;
  FunctionPtr f;

  static Value number(double v) {
    Value r;
    r.kind = NUMBER;
    r.n = v;
    return r;
  }
  static Value boolean(bool v) {
    Value r;
    r.kind = BOOL;
    r.b = v;
    return r;
  }
  static Value string(std::string v) {
    Value r;
    r.kind = STRING;
    r.s = std::move(v);
    return r;
  }
  bool truthy() const { return !(kind == NIL || (kind == BOOL && !b)); }
};

struct Table {
  std::vector<Value> array;            // t[1..n]
  std::map<std::string, Value> hash;   // string keys (and non-sequence numeric keys as text)
  ~Table();  // frees nested tables and closures without recursing per level
  Value get(const Value &key) const;
  void set(const Value &key, const Value &v);
};

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

class State {
 public:
  State();
  ~State();
  // Parse and run a chunk; throws Error with "name:line: message".
  void run(const std::string &source, const std::string &chunk_name);
  Value global(const std::string &name) const;
  // Call a function value with numeric arguments; returns all results.
  std::vector<Value> call(const Value &fn, const std::vector<Value> &args);

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
};

// "a.b.c" or "a.b[2]" lookup starting from a value; NIL when absent.
Value lookup(const Value &root, const std::string &path);

}  // namespace lua
}  // namespace fvh
