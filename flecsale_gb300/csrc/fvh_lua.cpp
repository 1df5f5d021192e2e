// Lua-subset interpreter for FleCSALE input files (see fvh_lua.h).
#include "fvh_lua.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <functional>
#include <sstream>

namespace fvh {
namespace lua {

// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
static std::string key_text(const Value &k) {
  if (k.kind == Value::STRING) return k.s;
  if (k.kind == Value::NUMBER) {
    std::ostringstream o;
    o.precision(17);
    o << "#" << k.n;
    return o.str();
  }
  if (k.kind == Value::BOOL) return k.b ? "#true" : "#false";
  throw Error("unsupported table key type");
}

Value Table::get(const Value &key) const {
  if (key.kind == Value::NUMBER && key.n >= 1 && key.n == std::floor(key.n) &&
      key.n <= (double)array.size())
    return array[(size_t)key.n - 1];
  if (key.kind == Value::NIL) return Value();
  auto it = hash.find(key_text(key));
  return it == hash.end() ? Value() : it->second;
}

// Tables, scopes and closures reference one another through shared_ptr, and a
// script can chain them arbitrarily deep (t = {t} in a loop, or a closure that
// captures the previous one).  Freed member by member, such a chain recurses
// once per link in the destructors and overflows the stack; instead each
// destructor moves its children to a list that the outermost destructor of the
// thread empties in a loop.
namespace {
thread_local std::vector<std::shared_ptr<void>> *t_release = nullptr;

void take(Value &v, std::vector<std::shared_ptr<void>> &out) {
  if (v.t) out.push_back(std::move(v.t));
  if (v.f) out.push_back(std::move(v.f));
}
}  // namespace

template <class Collect>
static void release_children(Collect &&collect) {
  std::vector<std::shared_ptr<void>> list;
  const bool outermost = t_release == nullptr;
  if (outermost) t_release = &list;
  collect(*t_release);
  if (!outermost) return;
  while (!list.empty()) {
    std::shared_ptr<void> p = std::move(list.back());
    list.pop_back();
    p.reset();  // may append this object's own children to the list
  }
  t_release = nullptr;
}

Table::~Table() {
  release_children([this](std::vector<std::shared_ptr<void>> &out) {
    for (auto &v : array) take(v, out);
    for (auto &kv : hash) take(kv.second, out);
  });
}

void Table::set(const Value &key, const Value &v) {
  if (key.kind == Value::NUMBER && key.n >= 1 && key.n == std::floor(key.n) &&
      key.n <= (double)array.size() + 1) {
    if (key.n == (double)array.size() + 1)
      array.push_back(v);
    else
      array[(size_t)key.n - 1] = v;
    return;
  }
  if (key.kind == Value::NIL) throw Error("table index is nil");
  hash[key_text(key)] = v;
}

// ---------------------------------------------------------------------------
// lexer
// ---------------------------------------------------------------------------
namespace {

enum Tok { T_EOF, T_NAME, T_NUMBER, T_STRING, T_SYM, T_KEYWORD };

struct Token {
  Tok type = T_EOF;
  std::string text;  // name / keyword / symbol / string contents
  double num = 0;
  int line = 0;
};

const char *const kKeywords[] = {"and",   "break", "do",     "else", "elseif", "end",
                                 "false", "for",   "function", "if", "in",     "local",
                                 "nil",   "not",   "or",     "repeat", "return", "then",
                                 "true",  "until", "while"};

bool is_keyword(const std::string &s) {
  for (const char *k : kKeywords)
    if (s == k) return true;
  return false;
}

class Lexer {
 public:
  Lexer(const std::string &src, const std::string &name) : s_(src), name_(name) {}

  std::vector<Token> all() {
    std::vector<Token> out;
    for (;;) {
      Token t = next();
      out.push_back(t);
      if (t.type == T_EOF) break;
    }
    return out;
  }

 private:
  const std::string &s_;
  std::string name_;
  size_t i_ = 0;
  int line_ = 1;

  [[noreturn]] void fail(const std::string &m) {
    throw Error(name_ + ":" + std::to_string(line_) + ": " + m);
  }
  char peek(size_t k = 0) const { return i_ + k < s_.size() ? s_[i_ + k] : '\0'; }

  // [[ ... ]] or [==[ ... ]==] starting at i_ (which points at '['); returns
  // false if this is not a long bracket
  bool long_bracket(std::string *out) {
    size_t j = i_ + 1;
    int level = 0;
    while (j < s_.size() && s_[j] == '=') ++level, ++j;
    if (j >= s_.size() || s_[j] != '[') return false;
    j++;
    const std::string close = "]" + std::string(level, '=') + "]";
    const size_t e = s_.find(close, j);
    if (e == std::string::npos) fail("unfinished long string/comment");
    for (size_t k = i_; k < e; ++k)
      if (s_[k] == '\n') ++line_;
    if (out) {
      size_t b = j;
      if (b < s_.size() && s_[b] == '\n') ++b;  // a first newline is skipped
      *out = s_.substr(b, e - b);
    }
    i_ = e + close.size();
    return true;
  }

  void skip_space_and_comments() {
    for (;;) {
      while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) {
        if (s_[i_] == '\n') ++line_;
        ++i_;
      }
      if (peek() == '-' && peek(1) == '-') {
        i_ += 2;
        if (peek() == '[' && long_bracket(nullptr)) continue;
        while (i_ < s_.size() && s_[i_] != '\n') ++i_;
        continue;
      }
      break;
    }
  }

  Token next() {
    skip_space_and_comments();
    Token t;
    t.line = line_;
    if (i_ >= s_.size()) return t;
    const char c = s_[i_];
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t j = i_;
      while (j < s_.size() && (std::isalnum((unsigned char)s_[j]) || s_[j] == '_')) ++j;
      t.text = s_.substr(i_, j - i_);
      t.type = is_keyword(t.text) ? T_KEYWORD : T_NAME;
      i_ = j;
      return t;
    }
    if (std::isdigit((unsigned char)c) || (c == '.' && std::isdigit((unsigned char)peek(1)))) {
      const char *b = s_.c_str() + i_;
      char *e = nullptr;
      if (c == '0' && (peek(1) == 'x' || peek(1) == 'X'))
        t.num = (double)std::strtoull(b, &e, 16);
      else
        t.num = std::strtod(b, &e);
      if (e == b) fail("malformed number");
      i_ += (size_t)(e - b);
      t.type = T_NUMBER;
      return t;
    }
    if (c == '"' || c == '\'') {
      ++i_;
      std::string v;
      while (i_ < s_.size() && s_[i_] != c) {
        char ch = s_[i_++];
        if (ch == '\n') fail("unfinished string");
        if (ch == '\\') {
          const char x = i_ < s_.size() ? s_[i_++] : '\0';
          switch (x) {
            case 'n': ch = '\n'; break;
            case 't': ch = '\t'; break;
            case 'r': ch = '\r'; break;
            case '0': ch = '\0'; break;
            default: ch = x; break;
          }
        }
        v.push_back(ch);
      }
      if (i_ >= s_.size()) fail("unfinished string");
      ++i_;
      t.type = T_STRING;
      t.text = v;
      return t;
    }
    if (c == '[' && (peek(1) == '[' || peek(1) == '=')) {
      std::string v;
      if (long_bracket(&v)) {
        t.type = T_STRING;
        t.text = v;
        return t;
      }
    }
    static const char *const three[] = {"..."};
    static const char *const two[] = {"==", "~=", "<=", ">=", ".."};
    for (const char *op : three)
      if (s_.compare(i_, 3, op) == 0) {
        t.type = T_SYM;
        t.text = op;
        i_ += 3;
        return t;
      }
    for (const char *op : two)
      if (s_.compare(i_, 2, op) == 0) {
        t.type = T_SYM;
        t.text = op;
        i_ += 2;
        return t;
      }
    if (std::string("+-*/%^#<>=(){}[];:,.").find(c) != std::string::npos) {
      t.type = T_SYM;
      t.text = std::string(1, c);
      ++i_;
      return t;
    }
    fail(std::string("unexpected character '") + c + "'");
  }
};

// ---------------------------------------------------------------------------
// syntax tree
// ---------------------------------------------------------------------------
enum NodeKind {
  // expressions
  E_NIL, E_TRUE, E_FALSE, E_NUMBER, E_STRING, E_NAME, E_INDEX, E_CALL, E_FUNCTION,
  E_TABLE, E_BINARY, E_UNARY, E_AND, E_OR, E_PAREN,
  // statements
  S_LOCAL, S_ASSIGN, S_CALL, S_IF, S_WHILE, S_NUMFOR, S_RETURN, S_BREAK, S_DO, S_BLOCK
};

struct Node {
  NodeKind kind;
  int line = 0;
  double num = 0;
  std::string text;                        // name, string, operator
  std::vector<std::unique_ptr<Node>> kids; // operands / statements / list items
  std::vector<std::string> names;          // locals, parameters
  std::vector<std::string> keys;           // table constructor: "" = positional, else field name
  std::vector<int> key_is_expr;            // table constructor: [expr] = value
  explicit Node(NodeKind k, int l) : kind(k), line(l) {}
};
using NodeP = std::unique_ptr<Node>;

class Parser {
 public:
  Parser(std::vector<Token> toks, std::string name) : t_(std::move(toks)), name_(std::move(name)) {}

  NodeP chunk() {
    NodeP b = block();
    if (cur().type != T_EOF) fail("'<eof>' expected near '" + cur().text + "'");
    return b;
  }

 private:
  std::vector<Token> t_;
  std::string name_;
  size_t p_ = 0;

  // Depth of the tree along the current path: one level per block() or expr()
  // in progress and one per operator or suffix folded into a left-deep chain
  // (a + b + c ..., a.b.c ...).  The bound keeps the parser's own recursion,
  // and the recursion of the evaluator and of the tree's destruction, within a
  // small part of the thread's stack.
  static constexpr int kMaxDepth = 1000;
  int depth_ = 0;
  struct Deeper {
    Parser &p;
    int levels = 0;
    explicit Deeper(Parser &parser) : p(parser) { add(); }
    void add() {
      ++levels;
      if (++p.depth_ > kMaxDepth) p.fail("chunk has too many syntax levels");
    }
    ~Deeper() { p.depth_ -= levels; }
  };

  const Token &cur() const { return t_[p_]; }
  [[noreturn]] void fail(const std::string &m) const {
    throw Error(name_ + ":" + std::to_string(cur().line) + ": " + m);
  }
  bool is(Tok ty, const char *text) const { return cur().type == ty && cur().text == text; }
  bool sym(const char *s) const { return is(T_SYM, s); }
  bool kw(const char *s) const { return is(T_KEYWORD, s); }
  void expect_sym(const char *s) {
    if (!sym(s)) fail(std::string("'") + s + "' expected near '" + cur().text + "'");
    ++p_;
  }
  void expect_kw(const char *s) {
    if (!kw(s)) fail(std::string("'") + s + "' expected near '" + cur().text + "'");
    ++p_;
  }
  std::string name() {
    if (cur().type != T_NAME) fail("name expected near '" + cur().text + "'");
    return t_[p_++].text;
  }

  bool block_end() const {
    return cur().type == T_EOF || kw("end") || kw("else") || kw("elseif") || kw("until");
  }

  NodeP block() {
    Deeper guard(*this);
    auto b = std::make_unique<Node>(S_BLOCK, cur().line);
    while (!block_end()) {
      if (kw("return")) {
        auto r = std::make_unique<Node>(S_RETURN, cur().line);
        ++p_;
        if (!block_end() && !sym(";")) r->kids = explist();
        if (sym(";")) ++p_;
        b->kids.push_back(std::move(r));
        if (!block_end()) fail("'end' expected after return");
        break;
      }
      b->kids.push_back(statement());
      if (sym(";")) ++p_;
    }
    return b;
  }

  NodeP statement() {
    const int line = cur().line;
    if (kw("local")) {
      ++p_;
      if (kw("function")) {
        ++p_;
        auto n = std::make_unique<Node>(S_LOCAL, line);
        n->names.push_back(name());
        n->kids.push_back(funcbody(line));
        return n;
      }
      auto n = std::make_unique<Node>(S_LOCAL, line);
      n->names.push_back(name());
      while (sym(",")) {
        ++p_;
        n->names.push_back(name());
      }
      if (sym("=")) {
        ++p_;
        n->kids = explist();
      }
      return n;
    }
    if (kw("function")) {
      ++p_;
      auto target = std::make_unique<Node>(E_NAME, line);
      target->text = name();
      NodeP t = std::move(target);
      while (sym(".")) {
        ++p_;
        auto idx = std::make_unique<Node>(E_INDEX, line);
        auto key = std::make_unique<Node>(E_STRING, line);
        key->text = name();
        idx->kids.push_back(std::move(t));
        idx->kids.push_back(std::move(key));
        t = std::move(idx);
      }
      auto a = std::make_unique<Node>(S_ASSIGN, line);
      a->kids.push_back(std::move(t));
      a->names.push_back("1");  // one target
      a->kids.push_back(funcbody(line));
      return a;
    }
    if (kw("if")) {
      ++p_;
      auto n = std::make_unique<Node>(S_IF, line);
      n->kids.push_back(expr());
      expect_kw("then");
      n->kids.push_back(block());
      while (kw("elseif")) {
        ++p_;
        n->kids.push_back(expr());
        expect_kw("then");
        n->kids.push_back(block());
      }
      if (kw("else")) {
        ++p_;
        n->kids.push_back(block());
      }
      expect_kw("end");
      return n;
    }
    if (kw("while")) {
      ++p_;
      auto n = std::make_unique<Node>(S_WHILE, line);
      n->kids.push_back(expr());
      expect_kw("do");
      n->kids.push_back(block());
      expect_kw("end");
      return n;
    }
    if (kw("for")) {
      ++p_;
      auto n = std::make_unique<Node>(S_NUMFOR, line);
      n->names.push_back(name());
      expect_sym("=");
      n->kids.push_back(expr());
      expect_sym(",");
      n->kids.push_back(expr());
      if (sym(",")) {
        ++p_;
        n->kids.push_back(expr());
      } else {
        auto one = std::make_unique<Node>(E_NUMBER, line);
        one->num = 1;
        n->kids.push_back(std::move(one));
      }
      expect_kw("do");
      n->kids.push_back(block());
      expect_kw("end");
      return n;
    }
    if (kw("do")) {
      ++p_;
      auto n = std::make_unique<Node>(S_DO, line);
      n->kids.push_back(block());
      expect_kw("end");
      return n;
    }
    if (kw("break")) {
      ++p_;
      return std::make_unique<Node>(S_BREAK, line);
    }
    // assignment or call
    NodeP first = suffixed();
    if (sym("=") || sym(",")) {
      auto a = std::make_unique<Node>(S_ASSIGN, line);
      std::vector<NodeP> targets;
      targets.push_back(std::move(first));
      while (sym(",")) {
        ++p_;
        targets.push_back(suffixed());
      }
      for (auto &t : targets)
        if (t->kind != E_NAME && t->kind != E_INDEX) fail("cannot assign to this expression");
      expect_sym("=");
      std::vector<NodeP> values = explist();
      a->names.push_back(std::to_string(targets.size()));
      for (auto &t : targets) a->kids.push_back(std::move(t));
      for (auto &v : values) a->kids.push_back(std::move(v));
      return a;
    }
    if (first->kind != E_CALL) fail("syntax error near '" + cur().text + "'");
    auto s = std::make_unique<Node>(S_CALL, line);
    s->kids.push_back(std::move(first));
    return s;
  }

  std::vector<NodeP> explist() {
    std::vector<NodeP> v;
    v.push_back(expr());
    while (sym(",")) {
      ++p_;
      v.push_back(expr());
    }
    return v;
  }

  NodeP funcbody(int line) {
    auto f = std::make_unique<Node>(E_FUNCTION, line);
    expect_sym("(");
    if (!sym(")")) {
      f->names.push_back(name());
      while (sym(",")) {
        ++p_;
        f->names.push_back(name());
      }
    }
    expect_sym(")");
    f->kids.push_back(block());
    expect_kw("end");
    return f;
  }

  NodeP primary() {
    const int line = cur().line;
    if (cur().type == T_NAME) {
      auto n = std::make_unique<Node>(E_NAME, line);
      n->text = name();
      return n;
    }
    if (sym("(")) {
      ++p_;
      auto n = std::make_unique<Node>(E_PAREN, line);
      n->kids.push_back(expr());
      expect_sym(")");
      return n;
    }
    fail("unexpected symbol near '" + cur().text + "'");
  }

  NodeP suffixed() {
    Deeper guard(*this);
    NodeP e = primary();
    for (;;) {
      const int line = cur().line;
      if (sym(".") || sym("[") || sym("(") || sym("{") || cur().type == T_STRING) guard.add();
      if (sym(".")) {
        ++p_;
        auto idx = std::make_unique<Node>(E_INDEX, line);
        auto key = std::make_unique<Node>(E_STRING, line);
        key->text = name();
        idx->kids.push_back(std::move(e));
        idx->kids.push_back(std::move(key));
        e = std::move(idx);
      } else if (sym("[")) {
        ++p_;
        auto idx = std::make_unique<Node>(E_INDEX, line);
        idx->kids.push_back(std::move(e));
        idx->kids.push_back(expr());
        expect_sym("]");
        e = std::move(idx);
      } else if (sym("(") || sym("{") || cur().type == T_STRING) {
        auto call = std::make_unique<Node>(E_CALL, line);
        call->kids.push_back(std::move(e));
        if (sym("(")) {
          ++p_;
          if (!sym(")"))
            for (auto &a : explist()) call->kids.push_back(std::move(a));
          expect_sym(")");
        } else if (sym("{")) {
          call->kids.push_back(table());
        } else {
          auto s = std::make_unique<Node>(E_STRING, line);
          s->text = t_[p_++].text;
          call->kids.push_back(std::move(s));
        }
        e = std::move(call);
      } else {
        return e;
      }
    }
  }

  NodeP table() {
    auto t = std::make_unique<Node>(E_TABLE, cur().line);
    expect_sym("{");
    while (!sym("}")) {
      if (sym("[")) {
        ++p_;
        t->kids.push_back(expr());
        expect_sym("]");
        expect_sym("=");
        t->kids.push_back(expr());
        t->keys.push_back("");
        t->key_is_expr.push_back(1);
      } else if (cur().type == T_NAME && p_ + 1 < t_.size() && t_[p_ + 1].type == T_SYM &&
                 t_[p_ + 1].text == "=") {
        t->keys.push_back(name());
        ++p_;  // '='
        t->kids.push_back(expr());
        t->key_is_expr.push_back(0);
      } else {
        t->keys.push_back("");
        t->kids.push_back(expr());
        t->key_is_expr.push_back(0);
      }
      if (sym(",") || sym(";"))
        ++p_;
      else
        break;
    }
    expect_sym("}");
    return t;
  }

  NodeP simple() {
    const int line = cur().line;
    if (cur().type == T_NUMBER) {
      auto n = std::make_unique<Node>(E_NUMBER, line);
      n->num = t_[p_++].num;
      return n;
    }
    if (cur().type == T_STRING) {
      auto n = std::make_unique<Node>(E_STRING, line);
      n->text = t_[p_++].text;
      return n;
    }
    if (kw("nil")) return ++p_, std::make_unique<Node>(E_NIL, line);
    if (kw("true")) return ++p_, std::make_unique<Node>(E_TRUE, line);
    if (kw("false")) return ++p_, std::make_unique<Node>(E_FALSE, line);
    if (kw("function")) {
      ++p_;
      return funcbody(line);
    }
    if (sym("{")) return table();
    return suffixed();
  }

  // precedence climbing with Lua 5.3 priorities
  static int left_prio(const std::string &op) {
    if (op == "or") return 1;
    if (op == "and") return 2;
    if (op == "<" || op == ">" || op == "<=" || op == ">=" || op == "~=" || op == "==") return 3;
    if (op == "..") return 9;
    if (op == "+" || op == "-") return 10;
    if (op == "*" || op == "/" || op == "%") return 11;
    if (op == "^") return 14;
    return -1;
  }
  static int right_prio(const std::string &op) {
    if (op == "..") return 8;  // right associative
    if (op == "^") return 13;  // right associative
    return left_prio(op);
  }
  static constexpr int kUnaryPrio = 12;

  std::string binop() const {
    if (cur().type == T_SYM || cur().type == T_KEYWORD) {
      const std::string &s = cur().text;
      if (left_prio(s) > 0) return s;
    }
    return "";
  }

  NodeP expr(int limit = 0) {
    Deeper guard(*this);
    NodeP left;
    const int line = cur().line;
    if (kw("not") || sym("-") || sym("#")) {
      auto u = std::make_unique<Node>(E_UNARY, line);
      u->text = cur().text;
      ++p_;
      u->kids.push_back(expr(kUnaryPrio));
      left = std::move(u);
    } else {
      left = simple();
    }
    for (std::string op = binop(); !op.empty() && left_prio(op) > limit; op = binop()) {
      ++p_;
      guard.add();
      NodeP right = expr(right_prio(op));
      auto b = std::make_unique<Node>(op == "and" ? E_AND : op == "or" ? E_OR : E_BINARY, line);
      b->text = op;
      b->kids.push_back(std::move(left));
      b->kids.push_back(std::move(right));
      left = std::move(b);
    }
    return left;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// evaluation
// ---------------------------------------------------------------------------
struct Scope {
  std::map<std::string, Value> vars;
  std::shared_ptr<Scope> parent;
  ~Scope() {
    release_children([this](std::vector<std::shared_ptr<void>> &out) {
      for (auto &kv : vars) take(kv.second, out);
      if (parent) out.push_back(std::move(parent));
    });
  }
};
using ScopeP = std::shared_ptr<Scope>;

struct Function {
  const Node *def = nullptr;  // E_FUNCTION node (owned by the State)
  ScopeP closure;
  std::function<std::vector<Value>(const std::vector<Value> &)> builtin;
  ~Function() {
    release_children([this](std::vector<std::shared_ptr<void>> &out) {
      if (closure) out.push_back(std::move(closure));
    });
  }
};

struct State::Impl {
  std::vector<NodeP> chunks;
  TablePtr globals = std::make_shared<Table>();
  std::string chunk_name;
  // Nested Lua calls (Lua's own limit is 200 C levels) and nested eval()/exec()
  // frames (each a few hundred bytes of native stack), both restored when an
  // error unwinds them.
  static constexpr int kMaxCalls = 200;
  static constexpr int kMaxFrames = 3000;
  int depth = 0, frames = 0;
  struct Enter {
    int &count;
    Enter(const Impl &s, int &c, int limit, const Node *n) : count(c) {
      if (count >= limit) s.fail(n, "stack overflow");
      ++count;
    }
    ~Enter() { --count; }
  };

  enum Flow { NORMAL, RETURN, BREAK };

  [[noreturn]] void fail(const Node *n, const std::string &m) const {
    throw Error(chunk_name + ":" + std::to_string(n ? n->line : 0) + ": " + m);
  }

  Value *find(const ScopeP &sc, const std::string &name) {
    for (Scope *s = sc.get(); s; s = s->parent.get()) {
      auto it = s->vars.find(name);
      if (it != s->vars.end()) return &it->second;
    }
    return nullptr;
  }

  double num(const Node *n, const Value &v, const char *what) {
    if (v.kind == Value::NUMBER) return v.n;
    if (v.kind == Value::STRING) {  // Lua coerces numeric strings in arithmetic
      char *e = nullptr;
      const double d = std::strtod(v.s.c_str(), &e);
      if (e != v.s.c_str() && *e == '\0') return d;
    }
    fail(n, std::string("attempt to perform arithmetic on a non-number (") + what + ")");
  }

  std::vector<Value> call(const Node *n, const Value &fn, const std::vector<Value> &args) {
    if (fn.kind != Value::FUNCTION) fail(n, "attempt to call a non-function value");
    if (fn.f->builtin) return fn.f->builtin(args);
    Enter call_level(*this, depth, kMaxCalls, n);
    auto sc = std::make_shared<Scope>();
    sc->parent = fn.f->closure;
    const Node *def = fn.f->def;
    for (size_t i = 0; i < def->names.size(); ++i)
      sc->vars[def->names[i]] = i < args.size() ? args[i] : Value();
    std::vector<Value> ret;
    exec_block(def->kids[0].get(), sc, ret);
    return ret;
  }

  // evaluate a list of expressions; the last one contributes all its values
  std::vector<Value> eval_list(const std::vector<NodeP> &list, size_t from, const ScopeP &sc) {
    std::vector<Value> out;
    for (size_t i = from; i < list.size(); ++i) {
      if (i + 1 == list.size() && list[i]->kind == E_CALL) {
        for (auto &v : eval_multi(list[i].get(), sc)) out.push_back(v);
      } else {
        out.push_back(eval(list[i].get(), sc));
      }
    }
    return out;
  }

  std::vector<Value> eval_multi(const Node *n, const ScopeP &sc) {
    if (n->kind == E_CALL) {
      const Value fn = eval(n->kids[0].get(), sc);
      return call(n, fn, eval_list(n->kids, 1, sc));
    }
    return {eval(n, sc)};
  }

  Value index(const Node *n, const Value &obj, const Value &key) {
    if (obj.kind != Value::TABLE) fail(n, "attempt to index a non-table value");
    return obj.t->get(key);
  }

  static bool equal(const Value &a, const Value &b) {
    if (a.kind != b.kind) return false;
    switch (a.kind) {
      case Value::NIL: return true;
      case Value::BOOL: return a.b == b.b;
      case Value::NUMBER: return a.n == b.n;
      case Value::STRING: return a.s == b.s;
      case Value::TABLE: return a.t == b.t;
      case Value::FUNCTION: return a.f == b.f;
    }
    return false;
  }

  bool less(const Node *n, const Value &a, const Value &b, bool or_equal) {
    if (a.kind == Value::NUMBER && b.kind == Value::NUMBER) return or_equal ? a.n <= b.n : a.n < b.n;
    if (a.kind == Value::STRING && b.kind == Value::STRING) return or_equal ? a.s <= b.s : a.s < b.s;
    fail(n, "attempt to compare incompatible values");
  }

  Value eval(const Node *n, const ScopeP &sc) {
    Enter frame(*this, frames, kMaxFrames, n);
    switch (n->kind) {
      case E_NIL: return Value();
      case E_TRUE: return Value::boolean(true);
      case E_FALSE: return Value::boolean(false);
      case E_NUMBER: return Value::number(n->num);
      case E_STRING: return Value::string(n->text);
      case E_PAREN: return eval(n->kids[0].get(), sc);
      case E_NAME: {
        if (Value *v = find(sc, n->text)) return *v;
        return globals->get(Value::string(n->text));
      }
      case E_INDEX:
        return index(n, eval(n->kids[0].get(), sc), eval(n->kids[1].get(), sc));
      case E_CALL: {
        auto r = eval_multi(n, sc);
        return r.empty() ? Value() : r[0];
      }
      case E_FUNCTION: {
        Value v;
        v.kind = Value::FUNCTION;
        v.f = std::make_shared<Function>();
        v.f->def = n;
        v.f->closure = sc;
        return v;
      }
      case E_TABLE: {
        Value v;
        v.kind = Value::TABLE;
        v.t = std::make_shared<Table>();
        size_t k = 0;
        double next = 1;
        for (size_t i = 0; i < n->keys.size(); ++i) {
          if (n->key_is_expr[i]) {
            const Value key = eval(n->kids[k].get(), sc);
            v.t->set(key, eval(n->kids[k + 1].get(), sc));
            k += 2;
          } else if (!n->keys[i].empty()) {
            v.t->set(Value::string(n->keys[i]), eval(n->kids[k++].get(), sc));
          } else if (i + 1 == n->keys.size() && n->kids[k]->kind == E_CALL) {
            for (auto &x : eval_multi(n->kids[k++].get(), sc)) v.t->set(Value::number(next++), x);
          } else {
            v.t->set(Value::number(next++), eval(n->kids[k++].get(), sc));
          }
        }
        return v;
      }
      case E_AND: {
        const Value a = eval(n->kids[0].get(), sc);
        return a.truthy() ? eval(n->kids[1].get(), sc) : a;
      }
      case E_OR: {
        const Value a = eval(n->kids[0].get(), sc);
        return a.truthy() ? a : eval(n->kids[1].get(), sc);
      }
      case E_UNARY: {
        const Value a = eval(n->kids[0].get(), sc);
        if (n->text == "not") return Value::boolean(!a.truthy());
        if (n->text == "-") return Value::number(-num(n, a, "unary minus"));
        if (a.kind == Value::STRING) return Value::number((double)a.s.size());
        if (a.kind == Value::TABLE) return Value::number((double)a.t->array.size());
        fail(n, "attempt to get length of a non-table value");
      }
      case E_BINARY: {
        const Value a = eval(n->kids[0].get(), sc), b = eval(n->kids[1].get(), sc);
        const std::string &op = n->text;
        if (op == "==") return Value::boolean(equal(a, b));
        if (op == "~=") return Value::boolean(!equal(a, b));
        if (op == "<") return Value::boolean(less(n, a, b, false));
        if (op == "<=") return Value::boolean(less(n, a, b, true));
        if (op == ">") return Value::boolean(less(n, b, a, false));
        if (op == ">=") return Value::boolean(less(n, b, a, true));
        if (op == "..") {
          auto text = [&](const Value &v) {
            if (v.kind == Value::STRING) return v.s;
            if (v.kind == Value::NUMBER) {
              std::ostringstream o;
              o.precision(14);
              o << v.n;
              return o.str();
            }
            fail(n, "attempt to concatenate a non-string value");
          };
          return Value::string(text(a) + text(b));
        }
        const double x = num(n, a, op.c_str()), y = num(n, b, op.c_str());
        if (op == "+") return Value::number(x + y);
        if (op == "-") return Value::number(x - y);
        if (op == "*") return Value::number(x * y);
        if (op == "/") return Value::number(x / y);
        if (op == "%") return Value::number(x - std::floor(x / y) * y);
        if (op == "^") return Value::number(std::pow(x, y));
        fail(n, "unknown operator " + op);
      }
      default:
        fail(n, "statement used as an expression");
    }
  }

  void assign(const Node *target, const Value &v, const ScopeP &sc) {
    if (target->kind == E_NAME) {
      if (Value *slot = find(sc, target->text))
        *slot = v;
      else
        globals->set(Value::string(target->text), v);
      return;
    }
    const Value obj = eval(target->kids[0].get(), sc);
    if (obj.kind != Value::TABLE) fail(target, "attempt to index a non-table value");
    obj.t->set(eval(target->kids[1].get(), sc), v);
  }

  Flow exec_block(const Node *b, const ScopeP &parent, std::vector<Value> &ret) {
    auto sc = std::make_shared<Scope>();
    sc->parent = parent;
    for (const auto &s : b->kids) {
      const Flow f = exec(s.get(), sc, ret);
      if (f != NORMAL) return f;
    }
    return NORMAL;
  }

  Flow exec(const Node *s, ScopeP &sc, std::vector<Value> &ret) {
    Enter frame(*this, frames, kMaxFrames, s);
    switch (s->kind) {
      case S_LOCAL: {
        if (!s->kids.empty() && s->kids[0]->kind == E_FUNCTION && s->names.size() == 1 &&
            s->kids.size() == 1) {  // local function f: visible inside its own body
          sc->vars[s->names[0]] = Value();
          sc->vars[s->names[0]] = eval(s->kids[0].get(), sc);
          return NORMAL;
        }
        const std::vector<Value> vals = eval_list(s->kids, 0, sc);
        auto fresh = std::make_shared<Scope>();  // new locals shadow from here on
        fresh->parent = sc;
        for (size_t i = 0; i < s->names.size(); ++i)
          fresh->vars[s->names[i]] = i < vals.size() ? vals[i] : Value();
        sc = fresh;
        return NORMAL;
      }
      case S_ASSIGN: {
        const size_t nt = (size_t)std::stoul(s->names[0]);
        const std::vector<Value> vals = eval_list(s->kids, nt, sc);
        for (size_t i = 0; i < nt; ++i)
          assign(s->kids[i].get(), i < vals.size() ? vals[i] : Value(), sc);
        return NORMAL;
      }
      case S_CALL:
        eval_multi(s->kids[0].get(), sc);
        return NORMAL;
      case S_IF: {
        size_t i = 0;
        for (; i + 1 < s->kids.size(); i += 2)
          if (eval(s->kids[i].get(), sc).truthy()) return exec_block(s->kids[i + 1].get(), sc, ret);
        if (i < s->kids.size()) return exec_block(s->kids[i].get(), sc, ret);
        return NORMAL;
      }
      case S_WHILE: {
        long guard = 0;
        while (eval(s->kids[0].get(), sc).truthy()) {
          if (++guard > 100000000L) fail(s, "loop limit exceeded");
          const Flow f = exec_block(s->kids[1].get(), sc, ret);
          if (f == BREAK) break;
          if (f == RETURN) return f;
        }
        return NORMAL;
      }
      case S_NUMFOR: {
        const double a = num(s, eval(s->kids[0].get(), sc), "for start");
        const double b = num(s, eval(s->kids[1].get(), sc), "for limit");
        const double st = num(s, eval(s->kids[2].get(), sc), "for step");
        if (st == 0) fail(s, "'for' step is zero");
        long guard = 0;
        for (double x = a; st > 0 ? x <= b : x >= b; x += st) {
          if (++guard > 100000000L) fail(s, "loop limit exceeded");
          auto body = std::make_shared<Scope>();
          body->parent = sc;
          body->vars[s->names[0]] = Value::number(x);
          const Flow f = exec_block(s->kids[3].get(), body, ret);
          if (f == BREAK) break;
          if (f == RETURN) return f;
        }
        return NORMAL;
      }
      case S_DO:
        return exec_block(s->kids[0].get(), sc, ret);
      case S_BREAK:
        return BREAK;
      case S_RETURN:
        ret = eval_list(s->kids, 0, sc);
        return RETURN;
      default:
        fail(s, "expression used as a statement");
    }
  }

  void install_math() {
    Value math;
    math.kind = Value::TABLE;
    math.t = std::make_shared<Table>();
    auto fn1 = [&](const char *name, double (*f)(double)) {
      Value v;
      v.kind = Value::FUNCTION;
      v.f = std::make_shared<Function>();
      v.f->builtin = [f, name](const std::vector<Value> &a) -> std::vector<Value> {
        if (a.empty() || a[0].kind != Value::NUMBER)
          throw Error(std::string("bad argument #1 to 'math.") + name + "' (number expected)");
        return {Value::number(f(a[0].n))};
      };
      math.t->set(Value::string(name), v);
    };
    fn1("sqrt", [](double x) { return std::sqrt(x); });
    fn1("abs", [](double x) { return std::fabs(x); });
    fn1("sin", [](double x) { return std::sin(x); });
    fn1("cos", [](double x) { return std::cos(x); });
    fn1("tan", [](double x) { return std::tan(x); });
    fn1("exp", [](double x) { return std::exp(x); });
    fn1("log", [](double x) { return std::log(x); });
    fn1("floor", [](double x) { return std::floor(x); });
    fn1("ceil", [](double x) { return std::ceil(x); });
    fn1("atan", [](double x) { return std::atan(x); });
    auto fnn = [&](const char *name, bool is_max) {
      Value v;
      v.kind = Value::FUNCTION;
      v.f = std::make_shared<Function>();
      v.f->builtin = [is_max, name](const std::vector<Value> &a) -> std::vector<Value> {
        if (a.empty()) throw Error(std::string("bad argument #1 to 'math.") + name + "'");
        double r = 0;
        for (size_t i = 0; i < a.size(); ++i) {
          if (a[i].kind != Value::NUMBER)
            throw Error(std::string("bad argument to 'math.") + name + "' (number expected)");
          r = i == 0 ? a[i].n : (is_max ? std::max(r, a[i].n) : std::min(r, a[i].n));
        }
        return {Value::number(r)};
      };
      math.t->set(Value::string(name), v);
    };
    fnn("min", false);
    fnn("max", true);
    math.t->set(Value::string("pi"), Value::number(3.14159265358979323846));
    math.t->set(Value::string("huge"), Value::number(HUGE_VAL));
    globals->set(Value::string("math"), math);
  }
};

State::State() : impl_(new Impl) { impl_->install_math(); }
State::~State() = default;

void State::run(const std::string &source, const std::string &chunk_name) {
  impl_->chunk_name = chunk_name;
  Lexer lx(source, chunk_name);
  Parser ps(lx.all(), chunk_name);
  impl_->chunks.push_back(ps.chunk());
  std::vector<Value> ret;
  auto sc = std::make_shared<Scope>();
  impl_->exec_block(impl_->chunks.back().get(), sc, ret);
}

Value State::global(const std::string &name) const {
  return impl_->globals->get(Value::string(name));
}

std::vector<Value> State::call(const Value &fn, const std::vector<Value> &args) {
  return impl_->call(nullptr, fn, args);
}

Value lookup(const Value &root, const std::string &path) {
  Value cur = root;
  size_t i = 0;
  while (i < path.size()) {
    if (cur.kind != Value::TABLE) return Value();
    if (path[i] == '.') {
      ++i;
      continue;
    }
    if (path[i] == '[') {
      const size_t e = path.find(']', i);
      if (e == std::string::npos) return Value();
      cur = cur.t->get(Value::number(std::atof(path.substr(i + 1, e - i - 1).c_str())));
      i = e + 1;
      continue;
    }
    size_t e = i;
    while (e < path.size() && path[e] != '.' && path[e] != '[') ++e;
    cur = cur.t->get(Value::string(path.substr(i, e - i)));
    i = e;
  }
  return cur;
}

}  // namespace lua
}  // namespace fvh
