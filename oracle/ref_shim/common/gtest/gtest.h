/* Stand-in for <gtest/gtest.h> (gtest is not installed): the reference
 * headers only need the EXPECT_* macros to compile; they become no-ops that
 * still accept a trailing `<< message`. Test infrastructure for oracle/. */
#pragma once
#include <ostream>
namespace dyc_ref_shim {
struct Sink {
    template <class T> Sink &operator<<(const T &) { return *this; }
};
}
#define EXPECT_TRUE(c) if (c) {} else dyc_ref_shim::Sink()
#define EXPECT_LE(a, b) if ((a) <= (b)) {} else dyc_ref_shim::Sink()
#define EXPECT_LT(a, b) if ((a) < (b)) {} else dyc_ref_shim::Sink()
#define EXPECT_EQ(a, b) if ((a) == (b)) {} else dyc_ref_shim::Sink()
