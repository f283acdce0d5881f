// Check of the CudaMap plugin built against the reference's own libcasadi: the cart-pole RK4
// step mapped over 8 instances with CudaMap::create and with Function::map(8, "serial"), its
// class, I/O and sparsity as CasADi reports them, then one numeric call of each. Without a GPU
// the CudaMap call must fail cleanly with the library's message. Then a Function::serialize()
// round trip, with the "Map" entry of CasADi's deserializer table dispatching "CudaMap" as
// the one-line patch of Map::deserialize would. Prints key=value lines.
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

// Map::deserialize with the "CudaMap" branch (the classes CasADi itself knows are not needed
// here: this check serializes a CudaMap only)
static ProtoFunction* map_deserialize_with_cuda(DeserializingStream& s) {
  std::string class_name;
  s.unpack("Map::class_name", class_name);
  casadi_assert(class_name == "CudaMap", "this check reads CudaMap only, got " + class_name);
  return CudaMap::deserialize(s);
}

static void call(const char* key, const Function& fn, const std::vector<DM>& in, const DM& want) {
  try {
    DM got = fn(in).at(0);
    std::cout << key << "_ok=1\n";
    std::cout << key << "_max_abs_diff=" << static_cast<double>(norm_inf(got - want)) << "\n";
  } catch (std::exception& e) {
    std::string msg = e.what();
    for (char& c : msg) if (c == '\n') c = ' ';
    std::cout << key << "_ok=0\n" << key << "_error=" << msg << "\n";
  }
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
  call("eval", cm, {x, u}, want);
  // serialize, then read back through CasADi's own Function::deserialize
  const std::string text = cm.serialize();
  FunctionInternal::deserialize_map["Map"] = &map_deserialize_with_cuda;
  Function back = Function::deserialize(text);
  std::cout << "back_class=" << back.class_name() << "\n";
  std::cout << "back_same_sparsity=" << (back.sparsity_in(0) == cm.sparsity_in(0) &&
                                         back.sparsity_out(0) == cm.sparsity_out(0)) << "\n";
  call("back_eval", back, {x, u}, want);
  return 0;
}
