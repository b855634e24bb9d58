// HamiltonianGen: the reference's operator-expression evaluator (src/QMspins/driver/
// ham_gen.cc) restated.  The expression is parsed by recursive descent into a postfix list
// (ham_gen.cc:446-697), then the list runs on a stack of numbers and matrices
// (ham_gen.cc:738-1150, 1163-1212).  The scalar functions are BlochLib's complex formulas
// (src/container/complex.h:990-1110), so values, branch choices and quirks match.
#include "bl_hamgen.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace bl {

namespace {

const char *kSymbols = "+-*/%^=()<>&|!";  // ham_gen.cc:57 (its terminator counts too)
const char *kMathSymbols = "+-*/%^=<>&|!";

bool is_symbol(char c) { return std::strchr(kSymbols, c) != nullptr; }
bool is_math_symbol(char c) { return std::strchr(kMathSymbols, c) != nullptr; }
bool digit(char c) { return std::isdigit(static_cast<unsigned char>(c)) != 0; }
char at(const std::string &s, size_t i) { return i < s.size() ? s[i] : '\0'; }

bool is_function(const std::string &f) {
  static const char *names[] = {"abs",  "acos", "asin", "atan", "cos",  "real", "imag",   "exp",  "floor",
                                "frac", "int",  "ln",   "log",  "pow",  "round", "ceil",  "sin",  "sqrt",
                                "tan",  "trunc", "sinh", "cosh", "tanh", "CHSSGN", "FAC"};
  for (const char *n : names)
    if (f == n) return true;
  return false;
}

std::string no_blanks(const std::string &s) {
  std::string o;
  for (char c : s)
    if (!std::isspace(static_cast<unsigned char>(c))) o += c;
  return o;
}

struct SpinSpec {  // ham_gen.cc:270-314
  char type = 'N', cart = 'N';
  int l = 0, m = 0, s1 = -1, s2 = -1;
  bool ok() const { return type == 'T' || type == 'I'; }
};

SpinSpec chop_spin(const std::string &in) {
  const std::string t = no_blanks(in);
  SpinSpec o;
  if (t.size() < 2) return o;
  if (t[0] == 'T') {
    o.type = 'T';
    if (t.size() < 5) return SpinSpec();
    if (digit(at(t, 1))) o.l = at(t, 1) - '0';
    int gm = 0;
    if (at(t, 2) == 'm' && digit(at(t, 3))) gm = 1, o.m = -(at(t, 3) - '0');
    else if (digit(at(t, 2))) o.m = at(t, 2) - '0';
    else return SpinSpec();
    if (at(t, 3 + gm) != '_') return SpinSpec();
    if (digit(at(t, 4 + gm))) o.s1 = at(t, 4 + gm) - '0';
    if (int(t.size()) < 7 + gm) {
      o.s2 = o.s1;
      return o;
    }
    if (at(t, 5 + gm) != ',') return o;
    if (digit(at(t, 6 + gm))) o.s2 = at(t, 6 + gm) - '0';
    return o;
  }
  if (t[0] == 'I') {
    o.type = 'I';
    if (std::strchr("xyzmpe", t[1]) == nullptr || t[1] == '\0') return SpinSpec();
    o.cart = t[1];
    if (t.size() >= 4) {
      if (t[2] != '_') return SpinSpec();
      if (digit(t[3])) o.s1 = t[3] - '0';
    }
    return o;
  }
  return SpinSpec();
}

struct SpaceSpec {  // ham_gen.cc:375-404
  int l = -10, m = -10;
  bool ok() const { return l != -10 && m != -10; }
};

SpaceSpec chop_space(const std::string &in) {
  const std::string t = no_blanks(in);
  SpaceSpec o;
  if (t.size() < 3 || t[0] != 'A') return o;
  if (!digit(t[1])) return SpaceSpec();
  o.l = t[1] - '0';
  if (t.size() > 3) {
    if (t[2] == 'm' && digit(t[3])) o.m = -(t[3] - '0');
  } else if (digit(t[2])) {
    o.m = t[2] - '0';
  } else {
    return SpaceSpec();
  }
  return o;
}

// ---------------------------------------------------------------- BlochLib complex formulas
double phase(cplx z) { return (z.real() == 0.0 && z.imag() == 0.0) ? 0.0 : std::atan2(z.imag(), z.real()); }
cplx c_exp(cplx z) {
  const double e = std::exp(z.real());
  return cplx(e * std::cos(z.imag()), e * std::sin(z.imag()));
}
cplx c_log(cplx z) { return cplx(std::log(std::abs(z)), phase(z)); }
cplx c_log10(cplx z) { return cplx(std::log10(std::abs(z)), phase(z)); }  // imag: the phase itself
cplx c_pow(cplx z, cplx w) { return c_exp(w * c_log(z)); }
cplx c_sqrt(cplx z) {
  double r = std::abs(z);
  if (r == 0.0) return cplx(0, 0);
  const double p = phase(z) / 2;
  r = std::sqrt(r);
  return cplx(r * std::cos(p), r * std::sin(p));
}
cplx c_sin(cplx z) {
  const double a = std::exp(z.imag()), b = 1 / a;
  return cplx(std::sin(z.real()) * (a + b) / 2, std::cos(z.real()) * (a - b) / 2);
}
cplx c_cos(cplx z) {
  const double a = std::exp(z.imag()), b = 1 / a;
  return cplx(std::cos(z.real()) * (a + b) / 2, -std::sin(z.real()) * (a - b) / 2);
}
cplx c_tan(cplx z) {
  const double a = std::exp(2 * z.imag()), b = 1 / a, d = std::cos(2 * z.real()) + (a + b) / 2;
  return cplx(std::sin(2 * z.real()) / d, (a - b) / (2 * d));
}
cplx c_sinh(cplx z) { return cplx(std::sinh(z.real()) * std::cos(z.imag()), std::cosh(z.real()) * std::sin(z.imag())); }
cplx c_cosh(cplx z) { return cplx(std::cosh(z.real()) * std::cos(z.imag()), std::sinh(z.real()) * std::sin(z.imag())); }
cplx c_tanh(cplx z) {  // as the reference computes it (the tan formula)
  const double t = std::cos(2 * z.real()) + std::cosh(2 * z.imag());
  return cplx(std::sin(2 * z.real()) / t, std::sinh(2 * z.imag()) / t);
}
const cplx kI(0, 1);
cplx c_asin(cplx z) { return -kI * c_log(kI * z + c_sqrt(1.0 - z * z)); }
cplx c_acos(cplx z) { return cplx(0, -1) * c_log(z + c_sqrt(z * z - 1.0)); }
cplx c_atan(cplx z) { return cplx(0, -0.5) * c_log((1.0 + kI * z) / (1.0 - kI * z)); }

// ---------------------------------------------------------------- matrices
CMatrix mat_mul(const CMatrix &x, const CMatrix &y) {
  CMatrix z(x.n);
  for (int i = 0; i < x.n; ++i)
    for (int k = 0; k < x.n; ++k) {
      const cplx v = x(i, k);
      if (v == cplx(0, 0)) continue;
      for (int j = 0; j < x.n; ++j) z(i, j) += v * y(k, j);
    }
  return z;
}

CMatrix mat_inverse(const CMatrix &a) {  // Gauss-Jordan, partial pivoting
  const int n = a.n;
  CMatrix m = a, inv(n);
  for (int i = 0; i < n; ++i) inv(i, i) = 1.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::abs(m(r, c)) > std::abs(m(p, c))) p = r;
    if (std::abs(m(p, c)) == 0.0) throw Error(1, "HamiltonianGen: division by a singular matrix");
    if (p != c)
      for (int j = 0; j < n; ++j) std::swap(m(p, j), m(c, j)), std::swap(inv(p, j), inv(c, j));
    const cplx d = 1.0 / m(c, c);
    for (int j = 0; j < n; ++j) m(c, j) *= d, inv(c, j) *= d;
    for (int r = 0; r < n; ++r) {
      if (r == c || m(r, c) == cplx(0, 0)) continue;
      const cplx f = m(r, c);
      for (int j = 0; j < n; ++j) m(r, j) -= f * m(c, j), inv(r, j) -= f * inv(c, j);
    }
  }
  return inv;
}

template <class F>
CMatrix elementwise(const CMatrix &x, F f) {
  CMatrix z(x.n);
  for (size_t i = 0; i < x.a.size(); ++i) z.a[i] = f(x.a[i]);
  return z;
}

CMatrix total(const SpinSystem &S, char w) {
  CMatrix t(S.dim());
  if (w == 'e') {
    for (int i = 0; i < S.dim(); ++i) t(i, i) = 1.0;
    return t;
  }
  for (int s = 0; s < S.spins(); ++s) {
    const CMatrix x = S.single(w, s);
    for (size_t i = 0; i < t.a.size(); ++i) t.a[i] += x.a[i];
  }
  return t;
}

CMatrix spin_tensor(const SpinSystem &S, const SpinSpec &sp) {  // ham_gen.cc:323-371
  auto check = [&](int s) {
    if (s < 0 || s >= S.spins()) throw Error(1, "HamiltonianGen: spin " + std::to_string(s) + " does not exist");
  };
  if (sp.type == 'I') {
    if (sp.s1 == -1) return total(S, sp.cart);
    check(sp.s1);
    return S.single(sp.cart, sp.s1);
  }
  // spin tensors (spin_ten.cc:41-120)
  check(sp.s1);
  if (sp.l == 0) return S.single('e', sp.s1);
  if (sp.l == 1) {
    if (sp.m == 1) return elementwise(S.single('m', sp.s1), [](cplx v) { return -v; });
    if (sp.m == 0) return S.single('z', sp.s1);
    if (sp.m == -1) return S.single('p', sp.s1);
    throw Error(1, "HamiltonianGen: rank-1 spin tensors have m in {-1, 0, 1}");
  }
  if (sp.l == 2) {
    check(sp.s2);
    const int a = sp.s1, b = sp.s2;
    auto mm = [&](char x, char y) { return mat_mul(S.single(x, a), S.single(y, b)); };
    auto lin = [](double ca, const CMatrix &x, double cb, const CMatrix &y) {
      CMatrix z(x.n);
      for (size_t i = 0; i < z.a.size(); ++i) z.a[i] = ca * x.a[i] + cb * y.a[i];
      return z;
    };
    switch (sp.m) {
      case -2: return elementwise(mm('m', 'm'), [](cplx v) { return 0.5 * v; });
      case -1: return lin(0.5, mm('m', 'z'), 0.5, mm('z', 'm'));
      case 0: {
        const CMatrix zz = mm('z', 'z'), xy = lin(1.0, mm('x', 'x'), 1.0, mm('y', 'y'));
        const double c = 1. / std::pow(6., 0.5);
        CMatrix z(zz.n);
        for (size_t i = 0; i < z.a.size(); ++i) z.a[i] = c * (2.0 * zz.a[i] - xy.a[i]);
        return z;
      }
      case 1: return lin(-0.5, mm('p', 'z'), -0.5, mm('z', 'p'));
      case 2: return elementwise(mm('p', 'p'), [](cplx v) { return 0.5 * v; });
    }
    throw Error(1, "HamiltonianGen: rank-2 spin tensors have m in {-2 .. 2}");
  }
  throw Error(1, "HamiltonianGen: spin tensor rank " + std::to_string(sp.l) + " is not available");
}

cplx space_tensor(const SpaceSpec &sp, double th, double ph) {  // space_ten.cc:36-71
  const double r38 = std::pow(3. / 8., 0.5);
  auto e = [&](double k) { return c_exp(cplx(0, k * ph)); };
  if (sp.l == 0) return 1.0;
  if (sp.l == 1) {
    if (sp.m == 1) return -r38 * std::sin(th) * e(1);
    if (sp.m == 0) return std::pow(3. / 4., 0.5) * std::cos(th);
    if (sp.m == -1) return r38 * std::sin(th) * e(-1);
    throw Error(1, "HamiltonianGen: rank-1 space tensors have m in {-1, 0, 1}");
  }
  if (sp.l == 2) {
    switch (sp.m) {
      case -2: return r38 * std::sin(th) * std::sin(th) * e(2);
      case -1: return r38 * std::sin(2. * th) * e(1);
      case 0: return 1. / 2. * (3. * std::cos(th) * std::cos(th) - 1.);
      case 1: return -r38 * std::sin(2. * th) * e(-1);
      case 2: return r38 * std::sin(th) * std::sin(th) * e(-2);
    }
    throw Error(1, "HamiltonianGen: rank-2 space tensors have m in {-2 .. 2}");
  }
  throw Error(1, "HamiltonianGen: space tensor rank " + std::to_string(sp.l) + " is not available");
}

// ---------------------------------------------------------------- parser
enum Kind { kNone, kSymbol, kNumber, kVariable, kFunction, kSpinOp, kSpaceOp };

struct Item {
  enum { Num, Var, Spin, Space, Fun } t;
  cplx v;
  std::string name;
  SpinSpec sp;
  SpaceSpec sa;
};

class Parser {
 public:
  Parser(const std::string &e, const std::map<std::string, cplx> &vars) : e_(e), vars_(vars) {}

  std::vector<Item> parse() {  // First (ham_gen.cc:507-514): trailing tokens are not read
    next();
    if (tok_.empty()) fail("empty expression");
    third();
    return out_;
  }

 private:
  const std::string &e_;
  const std::map<std::string, cplx> &vars_;
  size_t n_ = 0;
  std::string tok_;
  Kind kind_ = kNone;
  std::vector<Item> out_;

  [[noreturn]] void fail(const std::string &why) { throw Error(2, "HamiltonianGen: " + why + " in '" + e_ + "'"); }
  char c0() const { return tok_.empty() ? '\0' : tok_[0]; }
  bool known_var(const std::string &v) const {
    static const char *builtin[] = {"e", "pi", "Pi", "PI", "deg2rad", "rad2deg", "complexi"};
    if (vars_.count(v)) return true;
    for (const char *b : builtin)
      if (v == b) return true;
    return false;
  }
  void push_fun(const std::string &f) { out_.push_back(Item{Item::Fun, 0.0, f, {}, {}}); }

  void next() {  // GetNext (ham_gen.cc:446-505)
    tok_.clear();
    if (n_ >= e_.size()) return;
    while (n_ < e_.size() && std::isspace(static_cast<unsigned char>(e_[n_]))) ++n_;
    if (n_ >= e_.size()) {  // only blanks were left: the end (the reference reads the terminator)
      kind_ = kSymbol;
      return;
    }
    const char ch = e_[n_];
    if (is_symbol(ch)) {
      kind_ = kSymbol;
      tok_ += ch;
      ++n_;
      if (n_ < e_.size() && is_math_symbol(e_[n_ - 1]) && is_math_symbol(e_[n_])) tok_ += e_[n_++];
    } else if (std::isalpha(static_cast<unsigned char>(ch))) {
      while (n_ < e_.size() && !is_symbol(e_[n_]) && (n_ == 0 || e_[n_ - 1] != ']')) {
        if (!std::isspace(static_cast<unsigned char>(e_[n_]))) tok_ += e_[n_];
        ++n_;
      }
      if (is_function(tok_)) kind_ = kFunction;
      else if (known_var(tok_)) kind_ = kVariable;
      else if (chop_spin(tok_).ok()) kind_ = kSpinOp;
      else if (chop_space(tok_).ok()) kind_ = kSpaceOp;
      else fail("'" + tok_ + "' not found");
    } else if (digit(ch) || ch == '.') {
      while (n_ < e_.size()) {
        const char c = e_[n_];
        if (digit(c) || c == '.') {
          tok_ += c, kind_ = kNumber, ++n_;
        } else if (c == 'e' && n_ + 1 < e_.size() && (e_[n_ + 1] == '-' || e_[n_ + 1] == '+' || digit(e_[n_ + 1]))) {
          tok_ += c, tok_ += e_[n_ + 1], kind_ = kNumber, n_ += 2;
        } else {
          break;  // (the reference stops at a trailing 'e' and loops on 'e' before any other character)
        }
      }
    } else {
      fail(std::string("unexpected character '") + ch + "'");
    }
  }

  void third() {  // + - and comparisons (ham_gen.cc:516-552)
    fourth();
    const char sec = tok_.size() > 1 ? tok_[1] : '\0';  // read once, as the reference does
    char sign = c0();
    while (sign && std::strchr("+-<>%&|!=", sign)) {
      next();
      fourth();
      std::string f;
      if (sign == '+') f = "PLUS";
      else if (sign == '-') f = "MINUS";
      else if (sign == '>' && sec == '\0') f = "GREATER";
      else if (sign == '<' && sec == '\0') f = "LESS";
      else if (sign == '=' && sec == '=') f = "EQEQ";
      else if (sign == '!' && sec == '=') f = "NEEQ";
      else if (sign == '>' && sec == '=') f = "GREATEREQ";
      else if (sign == '<' && sec == '=') f = "LESSEQ";
      else if (sign == '&' && sec == '&') f = "ANDAND";
      else if (sign == '|' && sec == '|') f = "OROR";
      else if (sign == '%') f = "MOD";
      push_fun(f);  // an unmatched pair ("=", "&") leaves both operands: a no-op
      sign = c0();
    }
  }

  void fourth() {  // * /
    fifth();
    char sign = c0();
    while (sign == '*' || sign == '/') {
      next();
      fifth();
      push_fun(sign == '*' ? "MULT" : "DIV");
      sign = c0();
    }
  }

  void fifth() {  // ^, right to left
    sixth();
    if (c0() == '^') {
      next();
      fifth();
      push_fun("pow");
    }
  }

  void sixth() {  // unary + - !
    char sign = ' ';
    if ((kind_ == kSymbol && c0() == '+') || c0() == '-' || c0() == '!') {
      sign = c0();
      next();
    }
    seventh();
    if (sign == '-') push_fun("CHSSGN");
    if (sign == '!') push_fun("NOT");
  }

  void seventh() {  // ( )
    if (c0() == '(' && kind_ == kSymbol) {
      next();
      third();
      if (c0() != ')') fail("missing ')'");
      next();
    } else {
      eighth();
    }
  }

  void eighth() {
    if (kind_ == kNumber) {
      out_.push_back(Item{Item::Num, cplx(std::atof(tok_.c_str()), 0.0), "", {}, {}});
      next();
    } else if (kind_ == kVariable) {
      out_.push_back(Item{Item::Var, 0.0, tok_, {}, {}});
      next();
    } else if (kind_ == kSpinOp) {
      out_.push_back(Item{Item::Spin, 0.0, tok_, chop_spin(tok_), {}});
      next();
    } else if (kind_ == kSpaceOp) {
      out_.push_back(Item{Item::Space, 0.0, tok_, {}, chop_space(tok_)});
      next();
    } else {
      ninth();
    }
  }

  void ninth() {  // function ( expr )
    if (kind_ != kFunction) fail("syntax error");
    const std::string f = tok_;
    next();
    if (c0() == '(') {  // (a function name without '(' adds nothing, as in the reference)
      next();
      third();
      if (c0() != ')') fail("missing ')'");
      push_fun(f);
      next();
    }
  }
};

struct Val {
  bool mat = false;
  cplx c;
  CMatrix m;
};

}  // namespace

HamiltonianGen::HamiltonianGen() {}

void HamiltonianGen::add_var(const std::string &name, cplx value) { vars_[name] = value; }

CMatrix HamiltonianGen::evaluate(const SpinSystem &S, const std::string &expr, double theta, double phi,
                                 double gamma) const {
  (void)gamma;  // the spatial tensors depend on theta and phi only (ham_gen.cc:413-425)
  const std::vector<Item> prog = Parser(expr, vars_).parse();
  const double kPi = 3.141592653589793238;
  const std::map<std::string, cplx> builtin = {{"e", 2.718281828459045235}, {"pi", kPi},
                                               {"Pi", kPi},                 {"PI", kPi},
                                               {"deg2rad", kPi / 180.0},    {"rad2deg", 180.0 / kPi},
                                               {"complexi", cplx(0.0, 1.0)}};
  std::vector<Val> st;
  auto pop = [&]() {
    if (st.empty()) throw Error(2, "HamiltonianGen: missing operand in '" + expr + "'");
    Val v = st.back();
    st.pop_back();
    return v;
  };
  auto num = [](cplx c) {
    Val v;
    v.c = c;
    return v;
  };
  auto matv = [](CMatrix m) {
    Val v;
    v.mat = true;
    v.m = std::move(m);
    return v;
  };
  auto no_mat = [&](const Val &a, const char *what) {
    if (a.mat) throw Error(1, std::string("HamiltonianGen: '") + what + "' is not allowed on matrices");
  };
  for (const Item &it : prog) {
    switch (it.t) {
      case Item::Num: st.push_back(num(it.v)); break;
      case Item::Var: {
        auto v = vars_.find(it.name);
        st.push_back(num(v != vars_.end() ? v->second : builtin.at(it.name)));
        break;
      }
      case Item::Space: st.push_back(num(space_tensor(it.sa, theta, phi))); break;
      case Item::Spin: st.push_back(matv(spin_tensor(S, it.sp))); break;
      case Item::Fun: {
        const std::string &f = it.name;
        if (f == "PLUS" || f == "MINUS") {
          const Val t1 = pop(), t2 = pop();  // t2 op t1
          const double sg = f == "PLUS" ? 1.0 : -1.0;
          if (!t1.mat && !t2.mat) st.push_back(num(t2.c + sg * t1.c));
          else if (t1.mat && !t2.mat)
            st.push_back(matv(elementwise(t1.m, [&](cplx v) { return t2.c + sg * v; })));
          else if (!t1.mat && t2.mat)
            st.push_back(matv(elementwise(t2.m, [&](cplx v) { return v + sg * t1.c; })));
          else {
            if (t1.m.n != t2.m.n) throw Error(1, "HamiltonianGen: matrix sizes differ");
            CMatrix z = t2.m;
            for (size_t i = 0; i < z.a.size(); ++i) z.a[i] += sg * t1.m.a[i];
            st.push_back(matv(std::move(z)));
          }
        } else if (f == "MULT") {
          const Val t1 = pop(), t2 = pop();
          if (!t1.mat && !t2.mat) st.push_back(num(t2.c * t1.c));
          else if (t1.mat && !t2.mat) st.push_back(matv(elementwise(t1.m, [&](cplx v) { return v * t2.c; })));
          else if (!t1.mat && t2.mat) st.push_back(matv(elementwise(t2.m, [&](cplx v) { return t1.c * v; })));
          else st.push_back(matv(mat_mul(t2.m, t1.m)));
        } else if (f == "DIV") {
          const Val t1 = pop(), t2 = pop();
          if (!t1.mat && !t2.mat) st.push_back(num(t2.c / t1.c));
          else if (t1.mat && !t2.mat)
            st.push_back(matv(elementwise(mat_inverse(t1.m), [&](cplx v) { return t2.c * v; })));
          else if (!t1.mat && t2.mat) st.push_back(matv(elementwise(t2.m, [&](cplx v) { return v / t1.c; })));
          else st.push_back(matv(mat_mul(t2.m, mat_inverse(t1.m))));
        } else if (f == "pow") {
          const Val t1 = pop(), t2 = pop();
          no_mat(t1, "pow");
          if (!t2.mat) {
            st.push_back(num(c_pow(t2.c, t1.c)));
          } else {
            CMatrix m = t2.m;
            if (t1.c.real() > 0)
              for (int i = 0; i < int(t1.c.real()); ++i) m = mat_mul(m, t2.m);
            st.push_back(matv(std::move(m)));
          }
        } else if (f == "GREATER" || f == "LESS" || f == "GREATEREQ" || f == "LESSEQ" || f == "EQEQ" ||
                   f == "NEEQ" || f == "ANDAND" || f == "OROR" || f == "MOD") {
          const Val t1 = pop(), t2 = pop();
          no_mat(t1, f.c_str());
          no_mat(t2, f.c_str());
          const double a = std::abs(t2.c), b = std::abs(t1.c);  // Complex ordering compares moduli
          double r = 0;
          if (f == "GREATER") r = a > b;
          else if (f == "LESS") r = a < b;
          else if (f == "GREATEREQ") r = a >= b;
          else if (f == "LESSEQ") r = a <= b;
          else if (f == "EQEQ") r = t2.c == t1.c;
          else if (f == "NEEQ") r = t2.c != t1.c;
          else if (f == "ANDAND") r = t2.c.real() && t1.c.real();
          else if (f == "OROR") r = t2.c.real() || t1.c.real();
          else {
            const int d = int(t1.c.real());
            if (d == 0) throw Error(1, "HamiltonianGen: modulo by zero");
            r = double(int(t2.c.real()) % d);
          }
          st.push_back(num(r));
        } else if (f == "NOT") {
          const Val t1 = pop();
          no_mat(t1, "!");
          st.push_back(num(cplx(!int(t1.c.real()), !int(t1.c.imag()))));
        } else if (f == "int") {
          const Val t1 = pop();
          no_mat(t1, "int");
          st.push_back(num(double(int(t1.c.real()))));
        } else if (f.empty() || f == "frac" || f == "round" || f == "trunc" || f == "FAC") {
          // no computation in the reference: the operands stay where they are
        } else {
          cplx (*fn)(cplx) = nullptr;
          if (f == "abs") fn = [](cplx v) { return cplx(std::abs(v), 0.0); };
          else if (f == "acos") fn = c_acos;
          else if (f == "asin") fn = c_asin;
          else if (f == "atan") fn = c_atan;
          else if (f == "cos") fn = c_cos;
          else if (f == "sin") fn = c_sin;
          else if (f == "tan") fn = c_tan;
          else if (f == "exp") fn = c_exp;
          else if (f == "sqrt") fn = c_sqrt;
          else if (f == "ln") fn = c_log;
          else if (f == "log") fn = c_log10;
          else if (f == "sinh") fn = c_sinh;
          else if (f == "cosh") fn = c_cosh;
          else if (f == "tanh") fn = c_tanh;
          else if (f == "real") fn = [](cplx v) { return cplx(v.real(), 0.0); };
          else if (f == "imag") fn = [](cplx v) { return cplx(v.imag(), 0.0); };
          else if (f == "ceil") fn = [](cplx v) { return cplx(std::ceil(v.real()), 0.0); };
          else if (f == "floor") fn = [](cplx v) { return cplx(std::floor(v.real()), 0.0); };
          else if (f == "CHSSGN") fn = [](cplx v) { return -v; };
          else throw Error(2, "HamiltonianGen: unknown function '" + f + "'");
          const Val t1 = pop();
          // on matrices the reference's sinh and cosh evaluate sin and cos element by element
          // (its scalar forms are the hyperbolic ones)
          cplx (*fm)(cplx) = f == "sinh" ? c_sin : f == "cosh" ? c_cos : fn;
          st.push_back(t1.mat ? matv(elementwise(t1.m, fm)) : num(fn(t1.c)));
        }
        break;
      }
    }
  }
  // the result is the bottom of the stack (ham_gen.cc:1210)
  if (st.empty() || !st.front().mat)
    throw Error(1, "HamiltonianGen: '" + expr + "' evaluates to a number, not an operator");
  return st.front().m;
}

}  // namespace bl
