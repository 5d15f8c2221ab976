// The `upside` executable: the driver in libupside.so behind main(), as the
// reference's src/main.cpp:1103-1105.
#include "../../include/upside_main.h"

int main(int argc, const char* const* argv) { return upside_main(argc, argv, 1); }
