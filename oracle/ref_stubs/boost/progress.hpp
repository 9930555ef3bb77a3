// Stand-in for boost/progress.hpp (Boost is absent): ktensorCPU constructs a
// progress_display and increments it once per tensor point
// (src/demag_cu.cu:138, :230).  Here it counts silently.
// TEST INFRASTRUCTURE ONLY.
#pragma once
namespace boost {
class progress_display {
 public:
  explicit progress_display(unsigned long expected) : expected_(expected) {}
  progress_display& operator++() {
    ++count_;
    return *this;
  }
  unsigned long count() const { return count_; }
  unsigned long expected() const { return expected_; }

 private:
  unsigned long expected_ = 0, count_ = 0;
};
}  // namespace boost
