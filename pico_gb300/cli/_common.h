// Shared pieces of the CLI drivers (see _common.cpp).
#pragma once
#include <string>

#include "kcore.h"

namespace cli {
std::string parse_single_input(int argc, char **argv);
void die(const char *what);
kc_graph *load_coo(const std::string &path);
int run_report(kc_graph *g, int method);
void save_results(const std::string &path, const uint32_t *core, uint32_t n);
}  // namespace cli
