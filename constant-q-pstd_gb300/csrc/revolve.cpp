// revolve.cpp -- see revolve.h.
#include "revolve.h"

namespace qp {

static const int kMaxCheck = 64;  // checkpoint and repetition bound (src.c:176-177)

int Revolve::numforw(int steps, int snaps) {
    if (snaps < 1 || snaps > kMaxCheck) return -1;
    int reps = 0, range = 1;
    while (range < steps) {
        reps++;
        range = range * (reps + snaps) / reps;
    }
    if (reps > kMaxCheck) return -1;
    return reps * steps - range * reps / (snaps + 1);
}

RevolveAction Revolve::next() {
    if (check_ < -1 || capo_ > fine_) return RV_ERROR;
    if (check_ == -1 && capo_ < fine_) {
        turn_ = 0;
        ch_[0] = capo_ - 1;
    }
    const int span = fine_ - capo_;
    if (span == 0) {
        // nothing left between capo and fine: go back to the last checkpoint
        if (check_ == -1 || capo_ == ch_[0]) {
            check_ -= 1;
            return RV_TERMINATE;
        }
        capo_ = ch_[check_];
        oldfine_ = fine_;
        return RV_RESTORE;
    }
    if (span == 1) {
        // one step to reverse: the first time is the "first turn"
        fine_ -= 1;
        if (check_ >= 0 && ch_[check_] == capo_) check_ -= 1;
        oldfine_ = fine_;
        if (turn_ == 0) {
            turn_ = 1;
            return RV_FIRSTURN;
        }
        return RV_YOUTURN;
    }
    if (check_ == -1 || ch_[check_] != capo_) {
        // the current state is not yet stored: store it
        check_ += 1;
        if (check_ >= kMaxCheck) { info_ = 10; return RV_ERROR; }
        if (check_ + 1 > snaps_) { info_ = 11; return RV_ERROR; }
        ch_[check_] = capo_;
        if (check_ == 0) {
            oldsnaps_ = snaps_;
            if (snaps_ > kMaxCheck) { info_ = 14; return RV_ERROR; }
            if (numforw(fine_ - capo_, snaps_) == -1) { info_ = 12; return RV_ERROR; }
        }
        oldfine_ = fine_;
        return RV_TAKESHOT;
    }
    // advance capo by the binomially optimal amount for the free checkpoints
    if (oldfine_ < fine_ && snaps_ == check_ + 1) { info_ = 13; return RV_ERROR; }
    const int oldcapo = capo_;
    const int free_snaps = snaps_ - check_;
    if (free_snaps < 1) { info_ = 11; return RV_ERROR; }
    int reps = 0, range = 1;
    while (range < fine_ - capo_) {
        reps++;
        range = range * (reps + free_snaps) / reps;
    }
    if (reps > kMaxCheck) { info_ = 15; return RV_ERROR; }
    if (snaps_ != oldsnaps_ && snaps_ > kMaxCheck) { info_ = 14; return RV_ERROR; }
    const int d = free_snaps;
    const int b1 = range * reps / (d + reps);
    const int b2 = (d > 1) ? b1 * d / (d + reps - 1) : 1;
    const int b3 = (d == 1) ? 0 : ((d > 2) ? b2 * (d - 1) / (d + reps - 2) : 1);
    const int b4 = b2 * (reps - 1) / d;
    const int b5 = (d < 3) ? 0 : ((d > 3) ? b3 * (d - 2) / reps : 1);
    if (fine_ - capo_ <= b1 + b3)
        capo_ += b4;
    else if (fine_ - capo_ >= range - b5)
        capo_ += b1;
    else
        capo_ = fine_ - b2 - b3;
    if (capo_ == oldcapo) capo_ = oldcapo + 1;
    oldfine_ = fine_;
    return RV_ADVANCE;
}

}  // namespace qp
