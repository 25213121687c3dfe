// ORACLE build shim — test infrastructure only.  Compiles the reference CPU sieve
// (sieve/CPU/ctsieve.cpp) unchanged, from where it lies, into a shared library under
// oracle/_ref/ so that tests can run the reference itself.  The source path comes
// from the build recipe (REF_SIEVE_CPP); nothing of the reference is copied here.
#include <cstdint>
#include <cstdio>
#include <csignal>
#include <stdexcept>
#include <iostream>
#include <iomanip>
#include <fstream>
#include <sstream>
#include <string>
#include <cmath>
#include <vector>
#include <chrono>
#include <sys/stat.h>
#include <signal.h>

#define private public
#define main ctsieve_reference_main
#include REF_SIEVE_CPP
#undef main
#undef private

// Runs Sieve::check_pos / check_neg of the reference over [b_min, b_max].
// bits_out[i] = 1 when b_min + i is struck.  When write_files is set, the
// reference's own write(true) produces sv_*.dat and cand_*.txt in the cwd.
extern "C" int ref_sieve(int n, uint64_t b_min, uint64_t b_max,
                         uint64_t p_min_pos, uint64_t p_max_pos, uint64_t p_min_neg, uint64_t p_max_neg,
                         int mode, uint8_t *bits_out, uint64_t *p_last_pos, uint64_t *p_last_neg, int write_files)
{
	void (*old_int)(int) = std::signal(SIGINT, SIG_DFL);
	void (*old_term)(int) = std::signal(SIGTERM, SIG_DFL);
	int rc = 0;
	{
		Sieve s(n, b_min, b_max);
		std::signal(SIGINT, old_int);
		std::signal(SIGTERM, old_term);
		Sieve::_quit = false;
		s._p_min_pos = p_min_pos;
		s._p_min_neg = p_min_neg;
		std::streambuf *old = std::cout.rdbuf();
		std::ostringstream sink;
		std::cout.rdbuf(sink.rdbuf());
		try
		{
			if (mode >= 0) s.check_pos(p_max_pos);
			if (mode <= 0) s.check_neg(p_max_neg);
			if (write_files) s.write(true);
		}
		catch (const std::exception &) { rc = -1; }
		std::cout.rdbuf(old);
		for (size_t i = 0, size = s._bsieve.size(); i < size; ++i) bits_out[i] = s._bsieve[i] ? 1 : 0;
		*p_last_pos = s._p_min_pos;
		*p_last_neg = s._p_min_neg;
	}
	return rc;
}
