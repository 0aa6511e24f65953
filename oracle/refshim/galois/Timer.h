// Build-local stand-in for the one Galois 6.0 header the reference's
// examples/heat/heat_2d.hpp includes: a StatTimer with the interface that
// example uses (constructed from a name, start, stop, get).  The timer is not
// on the step's arithmetic; it measures nothing here.
#ifndef ADS_REFSHIM_GALOIS_TIMER_H
#define ADS_REFSHIM_GALOIS_TIMER_H

namespace galois {
class StatTimer {
public:
    explicit StatTimer(const char*) { }
    void start() { }
    void stop() { }
    long get() const { return 0; }
};
}  // namespace galois

#endif
