// Stand-in for <boost/program_options.hpp> (not installed here). The reference's
// gcn/util/util.hpp only declares the namespace alias `po` with it; its Matrix Market reader
// uses nothing from the library. Test infrastructure only.
#pragma once
namespace boost {
namespace program_options {}
}
