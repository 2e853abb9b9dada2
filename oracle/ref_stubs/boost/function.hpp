// Stand-in for <boost/function.hpp>: TEST INFRASTRUCTURE ONLY.  The
// reference's two-level basis header includes it but uses std::function,
// which the real header brings in through <functional>.
#include <functional>
