// convertor <txt_file> <bin_file> — drop-in for tc/graph/convertor.cpp: text edge list to
// the binary int32 edge list read by bs_tc / rt_tc.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "rtg_reference.h"

int main(int argc, char *argv[]) {
    if (argc != 3) {
        std::printf("Usage: ./bin/convertor txt_file bin_file\n");
        std::exit(1);
    }
    Graph::Txt2Bin(argv[1], argv[2]);
    return 0;
}
