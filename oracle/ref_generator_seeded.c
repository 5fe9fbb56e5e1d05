/*
 * ref_generator_seeded.c -- test infrastructure. The reference generator (generator.c:86-124) never seeds
 * drand48, so glibc starts it from state 0. This wrapper links generator.c with its main renamed
 * (-Dmain=ref_generator_main, see oracle/Makefile), calls srand48(seed) and then runs the reference's own
 * main unchanged, so a seeded insertion of the reference can be compared with pp_generate.
 *
 *   generator_seeded N density seed      (writes generated.rrr in the working directory)
 */
#include <stdlib.h>

int ref_generator_main(int argc, char *argv[]);

int main(int argc, char *argv[]) {
	if(argc < 4) return 1;
	srand48(atol(argv[3]));
	return ref_generator_main(3, argv);
}
