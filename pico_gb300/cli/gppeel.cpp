// gppeel: drop-in for the reference's gppeel binary (peel/gppeel.cu:108-260).
// Usage: gppeel <graph.mtx>; prints the reference's report lines.  Set
// KCORE_OUTPUT=<file> to also write "i core" lines (utility::SaveResults).
#include "_common.h"

int main(int argc, char **argv) {
    const std::string path = cli::parse_single_input(argc, argv);
    return cli::run_report(cli::load_coo(path), KC_GPP);
}
