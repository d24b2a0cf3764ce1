// The drop-in `nlchains` executable: `nlchains <model> <common options> <model-specific options>`
// (reference common/main.cpp:142-176), a thin C++ host over the C ABI of libnlchains_gb300.so.
#include <iostream>

#include "../../include/nlchains.h"

int main(int argc, char **argv) {
	if (argc == 1) {
		std::cout << "Please specify as first argument the subprogram to run: DNKG, DNLS, FPUT, Toda, dDNKG" << std::endl;
		return 0;
	}
	return nlc_program_run(argc - 1, argv + 1);
}
