// Check of the CudaMap plugin built against the reference's own libcasadi: the cart-pole RK4
// step mapped over 8 instances with CudaMap::create and with Function::map(8, "serial"), its
// class, I/O and sparsity as CasADi reports them, then one numeric call of each. Without a GPU
// the CudaMap call must fail cleanly with the library's message. Prints key=value lines.
#include <cmath>
#include <iostream>

#include <casadi/casadi.hpp>

#include "../../casadi_gb300/plugin/cuda_map.hpp"

using namespace casadi;

static Function cartpole_step() {
  SX x = SX::sym("x", 4), u = SX::sym("u");
  const double mc = 1.0, mp = 0.1, l = 0.5, g = 9.81, dt = 0.02;
  auto ode = [&](const SX& s) {
    SX th = s(2), om = s(3), sn = sin(th), cs = cos(th);
    SX den = mc + mp * sn * sn;
    SX acc = (u + mp * sn * (l * om * om + g * cs)) / den;
    SX alpha = (-u * cs - mp * l * om * om * cs * sn - (mc + mp) * g * sn) / (l * den);
    return vertcat(std::vector<SX>{s(1), acc, om, alpha});
  };
  SX k1 = ode(x), k2 = ode(x + dt / 2 * k1), k3 = ode(x + dt / 2 * k2), k4 = ode(x + dt * k3);
  return Function("f", {x, u}, {x + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)});
}

int main() {
  Function f = cartpole_step();
  const casadi_int n = 8;
  Function cm = CudaMap::create(f, n);
  Function sm = f.map(n, "serial");
  std::cout << "class=" << cm.class_name() << "\n";
  std::cout << "is_map=" << cm.is_a("Map") << "\n";
  std::cout << "is_cuda_map=" << cm.is_a("CudaMap") << "\n";
  std::cout << "n_in=" << cm.n_in() << "\n" << "n_out=" << cm.n_out() << "\n";
  std::cout << "size_in0=" << cm.size1_in(0) << "x" << cm.size2_in(0) << "\n";
  std::cout << "size_out0=" << cm.size1_out(0) << "x" << cm.size2_out(0) << "\n";
  std::cout << "same_sparsity=" << (cm.sparsity_in(0) == sm.sparsity_in(0) &&
                                    cm.sparsity_out(0) == sm.sparsity_out(0)) << "\n";
  DM x = DM::rand(4, n), u = DM::rand(1, n);
  DM want = sm(std::vector<DM>{x, u}).at(0);
  try {
    DM got = cm(std::vector<DM>{x, u}).at(0);
    std::cout << "eval_ok=1\n";
    std::cout << "max_abs_diff=" << static_cast<double>(norm_inf(got - want)) << "\n";
  } catch (std::exception& e) {
    std::string msg = e.what();
    for (char& c : msg) if (c == '\n') c = ' ';
    std::cout << "eval_ok=0\n" << "eval_error=" << msg << "\n";
  }
  return 0;
}
