// Stand-in for <boost/bind.hpp>: TEST INFRASTRUCTURE ONLY.  The
// reference's two-level basis header includes it but uses std::bind,
// which the real header brings in through <functional>.
#include <functional>
