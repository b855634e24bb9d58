// Operator expressions evaluated to spin-space matrices: the reference's HamiltonianGen
// (src/QMspins/driver/ham_gen.h, ham_gen.cc), which solid-2.0 and the qmsims examples use
// for initial density matrices and detection operators ("Ix_0 + complexi*Iy_1",
// "T2m1_0,1*A21", ...).
//
// Grammar (ham_gen.cc:428-697; lowest to highest precedence):
//   expr   := term  { (+ - < > <= >= == != && || %) term }     left to right
//   term   := power { (* /) power }                            left to right
//   power  := unary [ ^ power ]                                right to left
//   unary  := [+ - !] primary
//   primary:= ( expr ) | number | variable | spin op | space op | function ( expr )
// Tokens: symbols + - * / % ^ = ( ) < > & | ! (two adjacent operator symbols form one
// token whose first character decides the operation, so "2*-3" is 2*3); names run to the
// next symbol with blanks removed; numbers are digits, '.', and 'e' followed by a sign or a
// digit.  Names: functions abs acos asin atan cos sin tan exp sqrt ln log sinh cosh tanh
// real imag floor ceil int (frac round trunc FAC pass their argument through), variables
// pi Pi PI e deg2rad rad2deg complexi and any added with add_var, spin operators
// I{x,y,z,p,m,e} (total) and I{x,y,z,p,m,e}_k, spin tensors T{l}{m}_k[,j] with m written
// 'm1' for -1 (T0 = Ie, T1 = {-I-, Iz, I+}, T2 = spin_ten.cc:93-120), and spatial
// tensors A{l}{m} of the powder angles (space_ten.cc:36-71).
// Evaluation (ham_gen.cc:738-1150): numbers are complex; a number and a matrix combine
// element by element for + and -, scale for *, and n / M = n M^-1, M / n element by
// element, M1 / M2 = M1 M2^-1; M ^ n multiplies M by itself int(n) more times (so M^2 is
// M^3, M^0 and negative powers are M); functions act element by element on matrices (where
// the reference's sinh and cosh compute sin and cos, and its tanh the tan formula);
// comparisons take moduli and refuse matrices.  The result must be a matrix.
#pragma once

#include <map>
#include <string>

#include "bl_host.h"

namespace bl {

class HamiltonianGen {
 public:
  HamiltonianGen();
  void add_var(const std::string &name, cplx value);  // HamiltonianGen::addVar
  // HamiltonianGen::Hamiltonian(SpinSys&, string, theta, phi, gamma) (ham_gen.h:295-299)
  CMatrix evaluate(const SpinSystem &sys, const std::string &expr, double theta = 0, double phi = 0,
                   double gamma = 0) const;

 private:
  std::map<std::string, cplx> vars_;
};

}  // namespace bl
