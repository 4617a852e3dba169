// QASM front end: reads QASM lines on standard input and drives one GPU register through the
// drop-in iqs::QubitRegister<ComplexDP> (include/iqs_gb300/qureg.hpp). It accepts the command
// set of the reference's interface program (interface/src/intelqs_interface_main.cpp:17-55,
// interface/src/interface_api_qasm.cpp:21-140, interface_api_memory.cpp,
// interface_api_qubitid.cpp) and prints the same lines:
//
//   .malloc N        allocate N qubits (1..43) in |0...0>        "Allocated [N] qubits."
//   .free            release them                                 "Qubits successfully free."
//   .iversion        interface version                            "RC-1.1.0"
//   .version         library version
//   H q / X q / T q / S q / Tdag q / CNOT c,t    gates            "<op> [<args>]"
//   MeasZ q          prints "<op> [<args>]" and then P(q = 1) as a complex number
//   PrepZ q          printed, no operation
//   qubit q / cbit c scaffold declarations, printed
//
// Operand names become register positions in the order they first appear (the table is kept
// across .free). A line's first word is the operation, the rest its argument string; an empty
// line or the end of input stops the program. A failed operation prints
// "Qasm Op failed - [<op>]" on standard error and the program goes on.
#include <complex>
#include <functional>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include "iqs_gb300/qureg.hpp"

namespace {

using Register = iqs::QubitRegister<ComplexDP>;

constexpr double kTdagAngle = -0.785398163397448;  // -pi/4 as the reference's interface writes it
constexpr int kMaxQubits = 43;

std::unique_ptr<Register> reg;

class OperandNames {
 public:
  unsigned position(const std::string& name) {
    auto it = ids_.find(name);
    if (it == ids_.end()) it = ids_.emplace(name, (unsigned)ids_.size()).first;
    return it->second;
  }

 private:
  std::unordered_map<std::string, unsigned> ids_;
};
OperandNames names;

Register& live() {
  if (!reg) throw std::runtime_error("no register: .malloc first");
  return *reg;
}

void echo(const std::string& op, const std::string& args) { std::cout << op << " [" << args << "]" << std::endl; }

int one_qubit(const std::string& op, const std::string& args, void (Register::*gate)(unsigned)) {
  echo(op, args);
  (live().*gate)(names.position(args));
  return 0;
}

int op_malloc(const std::string& args) {
  if (reg) {
    std::cerr << ".malloc called before .free - memory leak detected." << std::endl;
    return 1;
  }
  int n = 0;
  try {
    n = std::stoi(args, nullptr, 10);
  } catch (const std::invalid_argument&) {
    std::cerr << ".malloc (size) - size parameter was not an integer." << std::endl;
  } catch (const std::out_of_range&) {
    std::cerr << ".malloc (size) - size parameter was too large to fit in an integer." << std::endl;
  }
  if (n < 1 || n > kMaxQubits) {
    std::cerr << ".malloc (size) - allocations in the range from 1..43 only." << std::endl;
    return 1;
  }
  reg.reset(new Register((std::size_t)n));
  (*reg)[0] = ComplexDP(1.0, 0.0);
  std::cout << "Allocated [" << n << "] qubits." << std::endl;
  return 0;
}

int op_free(const std::string&) {
  if (!reg) {
    std::cerr << "Harmless attempt to .free before .malloc. Nothing done." << std::endl;
    return 1;
  }
  reg.reset();
  std::cout << "Qubits successfully free." << std::endl;
  return 0;
}

const std::unordered_map<std::string, std::function<int(const std::string&)>>& table() {
  static const std::unordered_map<std::string, std::function<int(const std::string&)>> t = {
      {".malloc", op_malloc},
      {".free", op_free},
      {".iversion", [](const std::string&) { std::cout << "RC-1.1.0" << std::endl; return 0; }},
      {".version", [](const std::string&) { std::cout << "iqs_gb300 " << iqsg_version() << std::endl; return 0; }},
      {"H", [](const std::string& a) { return one_qubit("H", a, &Register::ApplyHadamard); }},
      {"X", [](const std::string& a) { return one_qubit("X", a, &Register::ApplyPauliX); }},
      {"T", [](const std::string& a) { return one_qubit("T", a, &Register::ApplyT); }},
      {"S", [](const std::string& a) { return one_qubit("S", a, &Register::ApplyPauliSqrtZ); }},
      {"Tdag",
       [](const std::string& a) {
         echo("Tdag", a);
         live().ApplyRotationZ(names.position(a), kTdagAngle);
         return 0;
       }},
      {"CNOT",
       [](const std::string& a) {
         const std::size_t comma = a.find(',');
         const unsigned c = names.position(a.substr(0, comma));
         const unsigned t = names.position(comma == std::string::npos ? std::string() : a.substr(comma + 1));
         echo("CNOT", a);
         live().ApplyCPauliX(c, t);
         return 0;
       }},
      {"MeasZ",
       [](const std::string& a) {
         echo("MeasZ", a);
         const ComplexDP p(live().GetProbability(names.position(a)), 0.0);
         std::cout << p << std::endl;
         return 0;
       }},
      {"PrepZ", [](const std::string& a) { echo("PrepZ", a); return 0; }},
      {"qubit", [](const std::string& a) { std::cout << "Qubit (scaffold syntax): " << a << std::endl; return 0; }},
      {"cbit", [](const std::string& a) { std::cout << "Cbit (scaffold syntax): " << a << std::endl; return 0; }},
  };
  return t;
}

int execute(const std::string& op, const std::string& args) {
  const auto& t = table();
  const auto it = t.find(op);
  if (it == t.end()) return 1;
  try {
    return it->second(args);
  } catch (const std::exception& e) {
    std::cerr << op << ": " << e.what() << std::endl;
    return 1;
  }
}

}  // namespace

int main() {
  std::string line;
  while (std::getline(std::cin, line) && !line.empty()) {
    const std::size_t space = line.find(' ');
    const std::string op = line.substr(0, space);
    // Without a space the whole line is also the argument string, as in the reference.
    const std::string args = space == std::string::npos ? line : line.substr(space + 1);
    if (op.empty()) continue;
    if (execute(op, args) > 0) std::cerr << "Qasm Op failed - [" << op << "]" << std::endl;
  }
  return 0;
}
