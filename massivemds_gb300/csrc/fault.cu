// State of the host-side fault hooks (fault.h) and their C-ABI switch.
#include <atomic>

#include "../../include/mdsx.h"
#include "fault.h"

namespace mdsx {
namespace {
std::atomic<int> g_site{0};       // FaultSite armed, 0 = none
std::atomic<long long> g_after{0};  // calls at that site to let through before the failing one
std::atomic<long long> g_fired{0};
}  // namespace

bool fault_fires(FaultSite site) {
    if (g_site.load(std::memory_order_relaxed) != (int)site) return false;
    if (g_after.fetch_sub(1) > 0) return false;
    g_site.store(0);
    g_fired.fetch_add(1);
    return true;
}

}  // namespace mdsx

extern "C" int mdsx_inject_fault(int site, long long after, long long* fired) {
    if (site < 0 || site > (int)mdsx::FaultSite::kLaunch || after < 0) return MDSX_EINVAL;
    if (fired) *fired = mdsx::g_fired.load();
    mdsx::g_site.store(0);
    mdsx::g_after.store(after);
    mdsx::g_site.store(site);
    return MDSX_OK;
}
