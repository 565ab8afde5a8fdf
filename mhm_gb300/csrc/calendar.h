// calendar.h -- model-step calendar, usable on host and device.
//
// Calendar of model step tt (1-based) of a run starting at Julian day number
// jul_start with `timestep` hours per step, by integer Gregorian arithmetic
// (E. G. Richards' JDN <-> date algorithms).  Equal to what do_time_step
// obtains from dec2date(newTime - 0.5) (src/common/mo_common_datetime_type.f90:
// 71-125, src/mHM/mo_mhm_interface_run.f90:360); checked step by step against
// the restated dec2date in the tests.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define MHM_HD __host__ __device__ inline
#else
#define MHM_HD inline
#endif

namespace mhm {

struct StepDate {
    int32_t year, month, day, hour, doy;
};

MHM_HD int64_t gregorian_to_jdn(int32_t y, int32_t m, int32_t d)
{
    const int64_t a = (14 - m) / 12;
    const int64_t yy = (int64_t)y + 4800 - a;
    const int64_t mm = m + 12 * a - 3;
    return d + (153 * mm + 2) / 5 + 365 * yy + yy / 4 - yy / 100 + yy / 400 - 32045;
}

MHM_HD void jdn_to_gregorian(int64_t J, int32_t *y, int32_t *m, int32_t *d)
{
    const int64_t f = J + 1401 + (((4 * J + 274277) / 146097) * 3) / 4 - 38;
    const int64_t e = 4 * f + 3;
    const int64_t g = (e % 1461) / 4;
    const int64_t h = 5 * g + 2;
    *d = (int32_t)((h % 153) / 5 + 1);
    *m = (int32_t)(((h / 153 + 2) % 12) + 1);
    *y = (int32_t)(e / 1461 - 4716 + (12 + 2 - *m) / 12);
}

MHM_HD StepDate step_date(int32_t jul_start, int32_t timestep, int64_t tt)
{
    const int64_t hours = (tt - 1) * (int64_t)timestep;
    const int64_t J = jul_start + hours / 24;
    StepDate s;
    s.hour = (int32_t)(hours % 24);
    jdn_to_gregorian(J, &s.year, &s.month, &s.day);
    s.doy = (int32_t)(J - gregorian_to_jdn(s.year, 1, 1) + 1);
    return s;
}

// Day flag of step tt and whether step tt + 1 starts a new day, month or year
// (is_new_day / is_new_month / is_new_year after datetimeinfo_increment,
// src/common/mo_common_datetime_type.f90:106-133); bits as StepFlags.
MHM_HD int32_t step_dflags(int32_t jul_start, int32_t timestep, int64_t tt)
{
    const StepDate sd = step_date(jul_start, timestep, tt);
    const StepDate nx = step_date(jul_start, timestep, tt + 1);
    int32_t fl = (sd.hour > 6 && sd.hour <= 18) ? 1 : 0; // isday, src/meteo/mo_meteo_handler.f90:1048
    if (nx.day != sd.day) fl |= 2;
    if (nx.month != sd.month) fl |= 4;
    if (nx.year != sd.year) fl |= 8;
    return fl;
}

// iLAI of step tt (datetimeinfo_update_LAI_timestep,
// src/common/mo_common_datetime_type.f90:138-155): the month for monthly LAI
// slots (timeStep_LAI_input 0, 1); for a gridded series (-1 daily, -2
// monthly, -3 yearly) the count of days / months / years from the run's first
// step through tt, i.e. the reference's counter raised at every new day /
// month / year with the first step counting as new.
MHM_HD int32_t step_lai(int32_t jul_start, int32_t timestep, int64_t tt, int32_t mode)
{
    const StepDate sd = step_date(jul_start, timestep, tt);
    if (mode >= 0) return sd.month;
    if (mode == -1) return (int32_t)(((tt - 1) * (int64_t)timestep) / 24 + 1);
    int32_t y0, m0, d0;
    jdn_to_gregorian(jul_start, &y0, &m0, &d0);
    if (mode == -2) return (sd.year - y0) * 12 + (sd.month - m0) + 1;
    return sd.year - y0 + 1;
}

} // namespace mhm
