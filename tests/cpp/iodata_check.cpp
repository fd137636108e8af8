// Compiles the reference-side binding (include/m2cg_iodata.hpp) against the
// reference's own IoData.h and runs it on a default IoData or on an input
// file's statements, assigned through the reference's own parser objects
// (parser/Assigner.h, Dictionary.h) the way its grammar does (Parser.y:44-98:
// `under X {` pushes X, a name is looked up in the enclosing `under` scopes
// outward and then among the top-level symbols, `.name` and `[i]` descend).
// The statements come one per line from the test:
//   U <path>                      under <path> {
//   E                             }
//   A <path> <kind> <value>       <path> = value;   kind: sym | int | dbl | str
//   <path> = name {.name | [index]}
// Writes the m2cg_config it builds (raw bytes) to argv[2]; exit 0 ok, 2 bad
// input, 4 the binding refused the input (reason on stdout).
#include <IoData.h>
#include <parser/Dictionary.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "m2cg_iodata.hpp"

static std::vector<Assigner*> under;

// Assignable (Parser.y:65-98)
static Assigner* resolve(std::istringstream& in) {
  std::string first;
  in >> first;
  const int tk = findSysToken(first.c_str());
  Assigner* a = nullptr;
  for (int i = (int)under.size(); i--;) {
    a = under[i]->findSubToken(tk);
    if (a) break;
  }
  if (!a) a = findSysObj(tk);
  std::string op;
  while (a && in >> op) {
    if (op == "=") break;
    if (op[0] == '.') a = a->findSubToken(findSysToken(op.c_str() + 1));
    else if (op[0] == '[') a = a->findIndexObject(atoi(op.c_str() + 1));
    else { std::fprintf(stderr, "bad path element %s\n", op.c_str()); return nullptr; }
  }
  return a;
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  IoData iod;
  iod.setupCmdFileVariables();
  if (std::strcmp(argv[1], "-") != 0) {
    std::ifstream f(argv[1]);
    std::string line;
    while (std::getline(f, line)) {
      std::istringstream in(line);
      std::string cmd;
      in >> cmd;
      if (cmd == "E") {
        if (under.empty()) return 2;
        under.pop_back();
      } else if (cmd == "U" || cmd == "A") {
        Assigner* a = resolve(in);
        if (!a) { std::fprintf(stderr, "cannot resolve: %s\n", line.c_str()); return 2; }
        if (cmd == "U") { under.push_back(a); continue; }
        std::string kind, value;
        in >> kind;
        std::getline(in, value);
        if (!value.empty() && value[0] == ' ') value.erase(0, 1);
        if (kind == "sym") a->assignToken(findSysToken(value.c_str()));
        else if (kind == "int") a->assignInt(std::atoi(value.c_str()));
        else if (kind == "dbl") a->assignDouble(std::strtod(value.c_str(), nullptr));
        else if (kind == "str") a->assignString(strdup(value.c_str()));
        else return 2;
      } else if (!cmd.empty()) {
        return 2;
      }
    }
  }
  m2cg_config c;
  const char* why = nullptr;
  if (!m2cg::config_from_iodata(iod, &c, &why)) {
    std::printf("refused: %s\n", why ? why : "?");
    return 4;
  }
  FILE* o = std::fopen(argv[2], "wb");
  if (!o || std::fwrite(&c, sizeof(c), 1, o) != 1) return 2;
  std::fclose(o);
  return 0;
}
