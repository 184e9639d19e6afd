// run_hyperblocker_exec -- drop-in for the reference's examples/run_hyperblocker.cu.
#include "../../include/hbx.h"

int main(int argc, char** argv) { return hbx_run_cli(argc, (const char* const*)argv); }
