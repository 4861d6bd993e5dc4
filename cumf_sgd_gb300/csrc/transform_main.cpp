// transform_main.cpp - `cumf_transform file_name`: the rating-text converter of
// data/netflix/transform.cpp:9-47 (three header lines skipped, "u v r" triples written as
// 12-byte records to file_name.bin), parsed on the GPU.  Usage errors print the reference's
// message and exit 0 as it does (transform.cpp:11-22); a parse or I/O error prints the
// library's message and exits 1 (the reference stops silently).
#include <stdio.h>

#include "cumf_sgd.h"

int main(int argc, char **argv) {
    if (argc != 2) {
        printf("usage: ./transform file_name\n");
        return 0;
    }
    FILE *probe = fopen(argv[1], "r");
    if (!probe) {
        printf("usage: ./transform file_name\n");
        return 0;
    }
    fclose(probe);
    int64_t n = 0;
    if (cumf_convert_text(argv[1], NULL, 3, &n) != CUMF_OK) {
        printf("%s\n", cumf_last_error());
        return 1;
    }
    return 0;
}
