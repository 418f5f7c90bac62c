// revolve.h -- re-entrant binomial checkpointing schedule.
//
// The schedule is Griewank & Walther's revolve (ACM TOMS 26(1), 2000,
// Algorithm 799), the same controller the reference links as a C file with
// function-static state (sgpstd-qrtm/src.c:314).  The action sequence must be
// identical to the reference's for the RTM image to match, so the decision
// rule is the published one; the state is held per object, so many shots can
// be scheduled at once.
#pragma once

namespace qp {

enum RevolveAction { RV_ADVANCE = 0, RV_TAKESHOT, RV_RESTORE, RV_FIRSTURN, RV_YOUTURN, RV_TERMINATE, RV_ERROR };

class Revolve {
public:
    Revolve(int steps, int snaps) : check_(-1), capo_(0), fine_(steps), snaps_(snaps), info_(3) {}
    RevolveAction next();
    int check() const { return check_; }
    int capo() const { return capo_; }
    int info() const { return info_; }
    static int numforw(int steps, int snaps);

private:
    int check_, capo_, fine_, snaps_, info_;
    int turn_ = 0, oldsnaps_ = 0, oldfine_ = 0;
    int ch_[64] = {0};
};

}  // namespace qp
