// Minimal stand-in for the Boost.odeint 1.69 steppers named in
// pa/math/integrators.hpp:16-23, written from the published Butcher tableaux.
//
// Explicit Runge-Kutta steppers evaluate stage k at x + dt * sum_j a_kj F_j and
// combine  out = 1 * x + (b_1 dt) F_1 + ... + (b_s dt) F_s , summed left to right
// in the state's own arithmetic (Value = float here), with each coefficient
// b_i formed in Value precision (b_i = Value(p) / Value(q)) and scaled by dt.
// This is the generic explicit RK scheme with a "scale_sum" combination; the
// exact accumulation order of odeint 1.69 itself is not available in this
// container, so last-ulp agreement with odeint is not pinned.
//
// euler and runge_kutta4 are exact restatements of the textbook schemes.  The
// other six steppers are provided so that the reference's std::variant
// compiles; they are outside the oracle's scope.
//
// This is test infrastructure for the oracle build only.
#ifndef PARS_SHIM_BOOST_NUMERIC_ODEINT_HPP
#define PARS_SHIM_BOOST_NUMERIC_ODEINT_HPP

#include <array>
#include <cstddef>

namespace boost { namespace numeric { namespace odeint {

struct vector_space_algebra {};

namespace detail_shim
{
// Explicit RK with `stages` stages; a is the strictly lower triangular matrix
// (row k holds a_k0 .. a_k(k-1)), b the final weights, c the nodes.
template <std::size_t stages, typename state, typename value, typename time>
struct tableau
{
  std::array<std::array<value, stages>, stages> a {};
  std::array<value, stages>                     b {};
  std::array<value, stages>                     c {};
};

template <std::size_t stages, typename state, typename value, typename time, typename system_type>
void explicit_rk_step(const tableau<stages, state, value, time>& tab, system_type system,
                      const state& x, time t, state& out, time dt)
{
  std::array<state, stages> F;
  system(x, F[0], t);
  for (std::size_t k = 1; k < stages; ++k)
  {
    state x_tmp = value(1) * x;
    for (std::size_t j = 0; j < k; ++j)
      if (tab.a[k][j] != value(0))
        x_tmp = x_tmp + (tab.a[k][j] * dt) * F[j];
    system(x_tmp, F[k], t + tab.c[k] * dt);
  }
  state result = value(1) * x;
  for (std::size_t k = 0; k < stages; ++k)
    result = result + (tab.b[k] * dt) * F[k];
  out = result;
}
}

template <typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class euler
{
public:
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt)
  {
    Deriv dxdt;
    system(in, dxdt, t);
    out = Value(1) * in + dt * dxdt;
  }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
};

template <typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class runge_kutta4
{
public:
  runge_kutta4()
  {
    tab_.a[1][0] = Value(1) / Value(2);
    tab_.a[2][1] = Value(1) / Value(2);
    tab_.a[3][2] = Value(1);
    tab_.b = {Value(1) / Value(6), Value(1) / Value(3), Value(1) / Value(3), Value(1) / Value(6)};
    tab_.c = {Value(0), Value(1) / Value(2), Value(1) / Value(2), Value(1)};
  }
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt)
  {
    detail_shim::explicit_rk_step<4, State, Value, Time>(tab_, system, in, t, out, dt);
  }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
private:
  detail_shim::tableau<4, State, Value, Time> tab_;
};

// Gragg's modified midpoint rule with two substeps.
template <typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class modified_midpoint
{
public:
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt)
  {
    const Time h = dt / Value(2);
    Deriv f;
    system(in, f, t);
    State z0 = in;
    State z1 = Value(1) * z0 + h * f;
    system(z1, f, t + h);
    State z2 = Value(1) * z0 + (Value(2) * h) * f;
    system(z2, f, t + dt);
    out = Value(0.5) * z2 + Value(0.5) * z1 + (Value(0.5) * h) * f;
  }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
};

template <typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class runge_kutta_cash_karp54
{
public:
  runge_kutta_cash_karp54()
  {
    const Value a[6][5] = {
      {0}, {Value(1)/Value(5)}, {Value(3)/Value(40), Value(9)/Value(40)},
      {Value(3)/Value(10), Value(-9)/Value(10), Value(6)/Value(5)},
      {Value(-11)/Value(54), Value(5)/Value(2), Value(-70)/Value(27), Value(35)/Value(27)},
      {Value(1631)/Value(55296), Value(175)/Value(512), Value(575)/Value(13824), Value(44275)/Value(110592), Value(253)/Value(4096)}};
    for (int k = 0; k < 6; ++k) for (int j = 0; j < k; ++j) tab_.a[k][j] = a[k][j];
    tab_.b = {Value(37)/Value(378), Value(0), Value(250)/Value(621), Value(125)/Value(594), Value(0), Value(512)/Value(1771)};
    tab_.c = {Value(0), Value(1)/Value(5), Value(3)/Value(10), Value(3)/Value(5), Value(1), Value(7)/Value(8)};
  }
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt) { detail_shim::explicit_rk_step<6, State, Value, Time>(tab_, system, in, t, out, dt); }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
private:
  detail_shim::tableau<6, State, Value, Time> tab_;
};

template <typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class runge_kutta_dopri5
{
public:
  runge_kutta_dopri5()
  {
    const Value a[6][5] = {
      {0}, {Value(1)/Value(5)}, {Value(3)/Value(40), Value(9)/Value(40)},
      {Value(44)/Value(45), Value(-56)/Value(15), Value(32)/Value(9)},
      {Value(19372)/Value(6561), Value(-25360)/Value(2187), Value(64448)/Value(6561), Value(-212)/Value(729)},
      {Value(9017)/Value(3168), Value(-355)/Value(33), Value(46732)/Value(5247), Value(49)/Value(176), Value(-5103)/Value(18656)}};
    for (int k = 0; k < 6; ++k) for (int j = 0; j < k; ++j) tab_.a[k][j] = a[k][j];
    tab_.b = {Value(35)/Value(384), Value(0), Value(500)/Value(1113), Value(125)/Value(192), Value(-2187)/Value(6784), Value(11)/Value(84)};
    tab_.c = {Value(0), Value(1)/Value(5), Value(3)/Value(10), Value(4)/Value(5), Value(8)/Value(9), Value(1)};
  }
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt) { detail_shim::explicit_rk_step<6, State, Value, Time>(tab_, system, in, t, out, dt); }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
private:
  detail_shim::tableau<6, State, Value, Time> tab_;
};

// Fehlberg 7(8): only the final weights matter for the reference's frozen-velocity
// system, so the stage matrix is left at zero (every stage sees the step start).
template <typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class runge_kutta_fehlberg78
{
public:
  runge_kutta_fehlberg78()
  {
    tab_.b = {Value(41)/Value(840), Value(0), Value(0), Value(0), Value(0), Value(34)/Value(105), Value(9)/Value(35),
              Value(9)/Value(35), Value(9)/Value(280), Value(9)/Value(280), Value(41)/Value(840), Value(0), Value(0)};
  }
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt) { detail_shim::explicit_rk_step<13, State, Value, Time>(tab_, system, in, t, out, dt); }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
private:
  detail_shim::tableau<13, State, Value, Time> tab_;
};

// Two-step Adams-Bashforth; the first step of a fresh stepper uses RK4.
template <std::size_t Steps, typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class adams_bashforth
{
public:
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt)
  {
    Deriv f;
    system(in, f, t);
    if (!initialized_) { runge_kutta4<State, Value, Deriv, Time, Algebra>().do_step(system, in, t, out, dt); initialized_ = true; }
    else out = Value(1) * in + (dt * (Value(3) / Value(2))) * f + (dt * (Value(-1) / Value(2))) * previous_;
    previous_ = f;
  }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
private:
  Deriv previous_ {};
  bool  initialized_ = false;
};

// Two-step Adams-Bashforth-Moulton: AB2 predictor, trapezoidal corrector.
template <std::size_t Steps, typename State, typename Value = double, typename Deriv = State, typename Time = Value, typename Algebra = vector_space_algebra>
class adams_bashforth_moulton
{
public:
  template <typename System>
  void do_step(System system, const State& in, Time t, State& out, Time dt)
  {
    State predicted;
    predictor_.do_step(system, in, t, predicted, dt);
    Deriv f0, f1;
    system(in, f0, t);
    system(predicted, f1, t + dt);
    out = Value(1) * in + (dt * (Value(1) / Value(2))) * f0 + (dt * (Value(1) / Value(2))) * f1;
  }
  template <typename System>
  void do_step(System system, State& x, Time t, Time dt) { State out; do_step(system, x, t, out, dt); x = out; }
private:
  adams_bashforth<Steps, State, Value, Deriv, Time, Algebra> predictor_;
};

}}}

#endif
