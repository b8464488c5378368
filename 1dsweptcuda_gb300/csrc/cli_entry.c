/* bin/<Problem><Precision>Out: the reference programs' command line
 * (`nx tpb dt tf freq alg solution.dat [timing.txt]`) over libswept1d.
 * Built once per problem / precision with -DSW_PROBLEM and -DSW_PRECISION.
 * Exit status 0 on success, 255 (the reference's exit(-1)) otherwise. */
#include "swept1d.h"

int main(int argc, char **argv)
{
    return sw_cli_main(SW_PROBLEM, SW_PRECISION, argc, argv) == SW_OK ? 0 : 255;
}
