// Single-process stand-in for Boost.MPI's communicator, so that the
// reference's parallel-tempering and umbrella-sampling translation units
// (src/ptmc_simulation.cpp, src/us_simulation.cpp) compile and their member
// functions can be called by one driver process acting as the master rank.
//
// rank() and size() return what the driver set in the mailbox.  send() and
// recv() go through an in-memory mailbox keyed by (source, destination, tag):
// the driver posts the messages the other ranks would have sent to the master
// and collects the ones the master sends to them.  A recv with no posted
// message asks the driver's on_empty hook, then fails loudly.
#pragma once
#include <any>
#include <deque>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>

namespace boost { namespace mpi {

struct Mailbox {
    int rank {0};
    int size {1};
    std::map<std::tuple<int, int, int>, std::deque<std::any>> box;
    std::function<void(int src, int dst, int tag)> on_empty;
    static Mailbox& get() {
        static Mailbox m;
        return m;
    }
    template <class T> void post(int src, int dst, int tag, const T& v) {
        box[std::make_tuple(src, dst, tag)].push_back(std::any(v));
    }
    template <class T> bool take(int src, int dst, int tag, T& v) {
        auto it = box.find(std::make_tuple(src, dst, tag));
        if (it == box.end() || it->second.empty()) return false;
        v = std::any_cast<T>(it->second.front());
        it->second.pop_front();
        return true;
    }
};

class communicator {
  public:
    int rank() const { return Mailbox::get().rank; }
    int size() const { return Mailbox::get().size; }
    template <class T> void send(int dest, int tag, const T& value) const {
        Mailbox::get().post(rank(), dest, tag, value);
    }
    template <class T> void recv(int source, int tag, T& value) const {
        Mailbox& m = Mailbox::get();
        if (m.take(source, rank(), tag, value)) return;
        if (m.on_empty) m.on_empty(source, rank(), tag);
        if (!m.take(source, rank(), tag, value))
            throw std::runtime_error("mpi stand-in: no message from rank " + std::to_string(source) + " with tag " +
                                     std::to_string(tag));
    }
};

}} // namespace boost::mpi
