/*
 * mhm_oracle.c -- CPU restatement of the mHM / mRM hot path (TEST
 * INFRASTRUCTURE: the checker for the GPU kernels, never part of the product).
 * See mhm_oracle.h for the build variants and conventions.  Citations are
 * file:line in the mHM source tree (v5.13.2-dev0).
 */
#include "mhm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_LIBM
#define ORA_EXP(x) exp(x)
#define ORA_LOG(x) log(x)
#define ORA_POW(x, y) pow((x), (y))
int ora_math_kind(void) { return 1; }
#else
#include "hmath.h"
#define ORA_EXP(x) hm_exp(x)
#define ORA_LOG(x) hm_log(x)
#define ORA_POW(x, y) hm_pow((x), (y))
int ora_math_kind(void) { return 0; }
#endif

/* src/common/mo_common_constants.f90:25  eps_dp = epsilon(1.0_dp) */
#define EPS_DP DBL_EPSILON
/* FORCES mo_constants: twothird_dp = 2/3 (nearest double) */
static const double TWOTHIRD_DP = 2.0 / 3.0;
/* FORCES mo_constants (values pinned by src/tests/test_pet.pf, YearDays = 365) */
static const double PI_D = 3.141592653589793238462643383279502884197;
static const double TWOPI_D = 6.283185307179586476925286766559005768394;
static const double DAYSECS = 86400.0;
static const double YEARDAYS = 365.0;
static const double SOLARCONST_DP = 1367.0;
static const double SPECHEATET_DP = 2.45e06;
static const double DEG2RAD_DP = 3.141592653589793238462643383279502884197 / 180.0;
static const double PSYCHRO_DP = 0.0646;
static const double RHO0_DP = 1.225;
static const double CP0_DP = 1005.0;
static const double T0_DP = 273.15; /* FORCES mo_constants T0_dp: Celsius <-> Kelvin */
/* src/mHM/mo_mhm_constants.f90 */
static const double DUFFIE_DR = 0.0330;
static const double DUFFIE_DELTA1 = 0.4090;
static const double DUFFIE_DELTA2 = 1.3900;
static const double TETENS_C1 = 0.6108;
static const double TETENS_C2 = 17.270;
static const double TETENS_C3 = 237.30;
static const double SATPRESSURESLOPE1 = 4098.0;
static const double HARSAMCONST = 17.800;
/* src/mHM/mo_mhm_constants.f90 / src/MPR/mo_mpr_constants.f90 initial states */
static const double P1_INIT = 0.0, P2_INIT = 15.0, P3_INIT = 10.0, P4_INIT = 75.0,
                    P5_INIT = 1500.0, C1_INITSM = 0.25;
static const double HOURSECS = 3600.0;

/* src/mHM/mo_canopy_interc.f90:75-133 */
void ora_canopy_interc(double pet, double interc_max, double precip, double *interc,
                       double *throughfall, double *evap_canopy)
{
    double aux_help = *interc + precip;
    if (aux_help >= interc_max) {
        *throughfall = aux_help - interc_max;
        *interc = interc_max;
    } else {
        *throughfall = 0.0;
        *interc = aux_help;
    }
    if (interc_max > EPS_DP)
        *evap_canopy = pet * ORA_POW(*interc / interc_max, TWOTHIRD_DP);
    else
        *evap_canopy = 0.0;
    if (*evap_canopy < 0.0)
        *evap_canopy = 0.0;
    if (*interc > *evap_canopy) {
        *interc = *interc - *evap_canopy;
    } else {
        *evap_canopy = *interc;
        *interc = 0.0;
    }
}

/* src/mHM/mo_snow_accum_melt.f90:70-158 */
void ora_snow_accum_melt(double deg_day_incr, double deg_day_max, double deg_day_noprec,
                         double prec, double temperature, double temperature_thresh,
                         double thrfall, double *snow_pack, double *deg_day, double *melt,
                         double *prec_effect, double *rain, double *snow)
{
    if (temperature > temperature_thresh) {
        *snow = 0.0;
        *rain = thrfall;
    } else {
        *snow = thrfall;
        *rain = 0.0;
    }
    if (prec <= (deg_day_max - deg_day_noprec) / deg_day_incr)
        *deg_day = deg_day_noprec + deg_day_incr * prec;
    else
        *deg_day = deg_day_max;
    if (temperature > temperature_thresh) {
        if (*snow_pack > 0.0) {
            double aux_help = *deg_day * (temperature - temperature_thresh);
            if (aux_help > *snow_pack) {
                *melt = *snow_pack;
                *snow_pack = 0.0;
            } else {
                *melt = aux_help;
                *snow_pack = *snow_pack - aux_help;
            }
        } else {
            *melt = 0.0;
            *snow_pack = 0.0;
        }
    } else {
        *melt = 0.0;
        *snow_pack = *snow_pack + *snow;
    }
    *prec_effect = *melt + *rain;
}

/* src/mHM/mo_soil_moisture.f90:333-363 */
double ora_feddes_et_reduction(double sm, double fc, double pw, double froots)
{
    if (sm >= fc)
        return froots;
    else if (sm > pw)
        return froots * (sm - pw) / (fc - pw);
    return 0.0;
}

/* src/mHM/mo_soil_moisture.f90:405-446 (result undefined for NaN theta: 0 here) */
double ora_jarvis_et_reduction(double sm, double sat, double pw, double froots, double c1)
{
    double theta = (sm - pw) / (sat - pw);
    if (theta < 0.0)
        theta = 0.0;
    if (theta > 1.0)
        theta = 1.0;
    if (theta >= c1)
        return froots;
    else if (theta < c1)
        return froots * (theta / c1);
    return 0.0;
}

/* src/mHM/mo_soil_moisture.f90:94-290 (body :176-286) */
void ora_soil_moisture(int processCase, int nH, double frac_sealed, double water_thresh_sealed,
                       double pet, double evap_coeff, const double *sm_sat, const double *frac_roots,
                       const double *sm_fc, const double *wilting_point, const double *sm_exponen,
                       double jarvis_thresh_c1, double aet_canopy, double prec_effec,
                       double *runoff_sealed, double *storage_sealed, double *infiltration,
                       double *soil_moist, double *aet, double *aet_sealed)
{
    *runoff_sealed = 0.0;
    *aet_sealed = 0.0;
    if (frac_sealed > 0.0) {
        double tmp = *storage_sealed + prec_effec;
        if (tmp > water_thresh_sealed) {
            *runoff_sealed = tmp - water_thresh_sealed;
            *storage_sealed = water_thresh_sealed;
        } else {
            *runoff_sealed = 0.0;
            *storage_sealed = tmp;
        }
        if (water_thresh_sealed > EPS_DP) {
            *aet_sealed = (pet / evap_coeff - aet_canopy) * (*storage_sealed / water_thresh_sealed);
            if (*aet_sealed < 0.0)
                *aet_sealed = 0.0;
        } else {
            *aet_sealed = DBL_MAX; /* huge(1.0_dp) */
        }
        if (*storage_sealed > *aet_sealed) {
            *storage_sealed = *storage_sealed - *aet_sealed;
        } else {
            *aet_sealed = *storage_sealed;
            *storage_sealed = 0.0;
        }
    }
    for (int h = 0; h < nH; ++h) {
        aet[h] = 0.0;
        infiltration[h] = 0.0;
    }
    double prec_effec_soil = prec_effec;
    for (int h = 0; h < nH; ++h) {
        if (h != 0)
            prec_effec_soil = infiltration[h - 1];
        if (soil_moist[h] > sm_sat[h]) {
            infiltration[h] = prec_effec_soil;
        } else {
            double frac_runoff;
            if (soil_moist[h] > EPS_DP)
                frac_runoff = ORA_EXP(sm_exponen[h] * ORA_LOG(soil_moist[h] / sm_sat[h]));
            else
                frac_runoff = 0.0;
            double tmp = prec_effec_soil * (1.0 - frac_runoff);
            if ((soil_moist[h] + tmp) > sm_sat[h]) {
                infiltration[h] = prec_effec_soil + (soil_moist[h] - sm_sat[h]);
                soil_moist[h] = sm_sat[h];
            } else {
                infiltration[h] = prec_effec_soil - tmp;
                soil_moist[h] = soil_moist[h] + tmp;
            }
        }
        /* :254-255: demand minus the positive aet of the horizons above, summed in order */
        aet[h] = pet - aet_canopy;
        if (h != 0) {
            double s = 0.0;
            for (int j = 0; j < h; ++j)
                if (aet[j] > 0.0)
                    s = s + aet[j];
            aet[h] = aet[h] - s;
        }
        double stress;
        if (processCase == 1 || processCase == 4)
            stress = ora_feddes_et_reduction(soil_moist[h], sm_fc[h], wilting_point[h], frac_roots[h]);
        else
            stress = ora_jarvis_et_reduction(soil_moist[h], sm_sat[h], wilting_point[h], frac_roots[h],
                                             jarvis_thresh_c1);
        aet[h] = aet[h] * stress;
        if (aet[h] < 0.0)
            aet[h] = 0.0;
        if (soil_moist[h] > aet[h]) {
            soil_moist[h] = soil_moist[h] - aet[h];
        } else {
            aet[h] = soil_moist[h] - EPS_DP;
            soil_moist[h] = EPS_DP;
        }
        if (soil_moist[h] < EPS_DP)
            soil_moist[h] = EPS_DP;
    }
}

/* src/mHM/mo_runoff.f90:74-154 */
void ora_runoff_unsat_zone(double k1, double kp, double k0, double alpha, double karst_loss,
                           double pefec_soil, double unsat_thresh, double *sat_storage,
                           double *unsat_storage, double *slow_interflow, double *fast_interflow,
                           double *perc)
{
    *unsat_storage = *unsat_storage + pefec_soil;
    *fast_interflow = 0.0;
    if (*unsat_storage > unsat_thresh) {
        double a = k0 * (*unsat_storage - unsat_thresh);
        double b = *unsat_storage - EPS_DP;
        *fast_interflow = (a < b) ? a : b; /* Fortran MIN, no NaN operands here */
    }
    *unsat_storage = *unsat_storage - *fast_interflow;
    *slow_interflow = 0.0;
    if (*unsat_storage > EPS_DP) {
        double a = k1 * ORA_POW(*unsat_storage, 1.0 + alpha);
        double b = *unsat_storage - EPS_DP;
        *slow_interflow = (a < b) ? a : b;
    }
    *unsat_storage = *unsat_storage - *slow_interflow;
    *perc = kp * *unsat_storage;
    if (*unsat_storage > *perc) {
        *unsat_storage = *unsat_storage - *perc;
        *sat_storage = *sat_storage + *perc * karst_loss;
    } else {
        *sat_storage = *sat_storage + *unsat_storage * karst_loss;
        *unsat_storage = 0.0;
    }
}

/* src/mHM/mo_runoff.f90:191-212 */
void ora_runoff_sat_zone(double k2, double *sat_storage, double *baseflow)
{
    if (*sat_storage > 0.0) {
        *baseflow = k2 * *sat_storage;
        *sat_storage = *sat_storage - *baseflow;
    } else {
        *baseflow = 0.0;
        *sat_storage = 0.0;
    }
}

/* src/mHM/mo_runoff.f90:248-274 */
double ora_L1_total_runoff(double fsealed, double fast, double slow, double base, double direct)
{
    return ((base + slow + fast) * (1.0 - fsealed)) + (direct * fsealed);
}

/* src/mHM/mo_pet.f90:314-355 */
double ora_extraterr_rad_approx(int doy, double latitude)
{
    double dr = 1.0 + DUFFIE_DR * cos(TWOPI_D * doy / YEARDAYS);
    double delta = DUFFIE_DELTA1 * sin(TWOPI_D * doy / YEARDAYS - DUFFIE_DELTA2);
    double arg = -tan(latitude) * tan(delta);
    if (arg < -1.0)
        arg = -1.0;
    if (arg > 1.0)
        arg = 1.0;
    double omega = acos(arg);
    return DAYSECS / PI_D / SPECHEATET_DP * SOLARCONST_DP * dr *
           (omega * sin(latitude) * sin(delta) + cos(latitude) * cos(delta) * sin(omega));
}

/* FORCES mo_utils LE(a, b), restated from the in-tree copy
 * pre-proc/mtCLIM/mo_utils.f90 (lesserequal_dp): false only when a > b and
 * |a - b| exceeds epsilon*|b|. */
static int ora_le(double a, double b)
{
    if (((EPS_DP * fabs(b) - fabs(a - b)) < 0.0) && (a > b))
        return 0;
    return 1;
}

/* src/mHM/mo_pet.f90:73-116 */
double ora_pet_hargreaves(double HarSamCoeff, double HarSamConst, double tavg, double tmax,
                          double tmin, double latitude, int doy)
{
    double delta_temp = tmax - tmin;
    if (ora_le(delta_temp, 0.0) || ora_le(tavg, -HarSamConst))
        return 0.0;
    return HarSamCoeff * ora_extraterr_rad_approx(doy, DEG2RAD_DP * latitude) * (tavg + HarSamConst) *
           sqrt(delta_temp);
}

/* src/mHM/mo_pet.f90:426-441 */
double ora_sat_vap_pressure(double tavg)
{
    return TETENS_C1 * ORA_EXP(TETENS_C2 * tavg / (tavg + TETENS_C3));
}

/* src/mHM/mo_pet.f90:384-399 */
double ora_slope_satpressure(double tavg)
{
    return SATPRESSURESLOPE1 * ora_sat_vap_pressure(tavg) / ORA_EXP(2.0 * ORA_LOG(tavg + TETENS_C3));
}

/* src/mHM/mo_pet.f90:149-174 */
double ora_pet_priestly(double alpha, double rn, double tavg)
{
    double delta = ora_slope_satpressure(tavg);
    return alpha * delta / (PSYCHRO_DP + delta) * (rn * DAYSECS / SPECHEATET_DP);
}

/* src/mHM/mo_pet.f90:235-272 */
double ora_pet_penman(double net_rad, double tavg, double act_vap_pressure, double aerodyn_resistance,
                      double bulksurface_resistance, double a_s, double a_sh)
{
    return DAYSECS / SPECHEATET_DP *
           (ora_slope_satpressure(tavg) * net_rad +
            RHO0_DP * CP0_DP * (ora_sat_vap_pressure(tavg) - act_vap_pressure) * a_sh / aerodyn_resistance) /
           (ora_slope_satpressure(tavg) +
            PSYCHRO_DP * a_sh / a_s * (1.0 + bulksurface_resistance / aerodyn_resistance));
}

/* src/meteo/mo_meteo_temporal_tools.f90:32-50 */
double ora_disagg_meteo_weights(double day_val, double weight, double correction)
{
    return (day_val + correction) * weight - correction;
}

/* src/meteo/mo_meteo_temporal_tools.f90:66-96 */
double ora_disagg_flux_daynight(int isday, double ntimesteps_day, double day_val, double fday,
                                double fnight)
{
    if (ntimesteps_day > 1.0) {
        if (isday)
            return 2.0 * day_val * fday / ntimesteps_day;
        return 2.0 * day_val * fnight / ntimesteps_day;
    }
    return day_val;
}

/* src/meteo/mo_meteo_temporal_tools.f90:113-161 */
double ora_disagg_state_daynight(int isday, double ntimesteps_day, double day_val, double fday,
                                 double fnight, int add_correction)
{
    if (ntimesteps_day > 1.0) {
        if (add_correction)
            return isday ? day_val + fday : day_val + fnight;
        return isday ? 2.0 * day_val * fday : 2.0 * day_val * fnight;
    }
    return day_val;
}

/* ---- calendar: FORCES mo_julian, restated from the in-tree copy
 * pre-proc/mtCLIM/mo_julian.f90 (juldayJulian :966-1002, caldatJulian
 * :555-591, dec2dateJulian :811-891).  The literal 30.6001 in julday is a
 * default-kind (single precision) real in the Fortran source. ---- */
int32_t ora_julday(int32_t dd, int32_t mm, int32_t yy)
{
    const int32_t IGREG2 = 15 + 31 * (10 + 12 * 1582);
    const int32_t IGREG1 = 4 + 31 * (10 + 12 * 1582);
    int64_t jd, jm, jy, A, B = 0;
    if (mm > 2) {
        jm = mm;
        jy = yy;
    } else {
        jm = mm + 12;
        jy = yy - 1;
    }
    jd = dd;
    if (dd + 31 * (mm + 12 * yy) >= IGREG2) {
        A = jy / 100;
        B = 2 - A + A / 4;
    } else if (dd + 31 * (mm + 12 * yy) <= IGREG1) {
        B = 0;
    }
    const double c306 = (double)30.6001f;
    return (int32_t)(365.25 * (double)(jy + 4716) + (double)(int64_t)(c306 * (double)(jm + 1)) +
                     (double)(jd + B) - 1524.5 + 0.5);
}

void ora_caldat(int32_t julian, int32_t *dd, int32_t *mm, int32_t *yy)
{
    const int32_t IGREG = 2299161;
    int64_t A, B, C, D, E, g;
    if (julian < IGREG) {
        A = julian;
    } else {
        g = (int64_t)(((double)julian - 1867216.25) / 36524.25);
        A = julian + 1 + g - g / 4;
    }
    B = A + 1524;
    C = (int64_t)(((double)B - 122.1) / 365.25);
    D = (int64_t)(365.25 * (double)C);
    E = (int64_t)((double)(B - D) / 30.6001);
    *dd = (int32_t)(B - D - (int64_t)(30.6001 * (double)E));
    *mm = (int32_t)(E < 14 ? E - 1 : E - 13);
    *yy = (int32_t)(*mm > 2 ? C - 4716 : C - 4715);
}

void ora_dec2date(double julian, int32_t *dd, int32_t *mm, int32_t *yy, int32_t *hh, int32_t *nn,
                  int32_t *ss)
{
    const int32_t IGREG = 2299161;
    int64_t A, B, C, D, E, g, Z;
    int32_t day, month, year, hour, minute, second;
    Z = (int64_t)(julian + 0.5);
    if (Z < IGREG) {
        A = Z;
    } else {
        g = (int64_t)(((double)Z - 1867216.25) / 36524.25);
        A = Z + 1 + g - g / 4;
    }
    B = A + 1524;
    C = (int64_t)(((double)B - 122.1) / 365.25);
    D = (int64_t)(365.25 * (double)C);
    E = (int64_t)((double)(B - D) / 30.6001);
    day = (int32_t)(B - D - (int64_t)(30.6001 * (double)E));
    month = (int32_t)(E < 14 ? E - 1 : E - 13);
    year = (int32_t)(month > 2 ? C - 4716 : C - 4715);
    double fraction = julian + 0.5 - (double)Z;
    int32_t fh = (int32_t)floor(fraction * 24.0);
    hour = fh < 0 ? 0 : (fh > 23 ? 23 : fh);
    fraction = fraction - (double)hour / 24.0;
    int32_t fm = (int32_t)floor(fraction * 1440.0);
    minute = fm < 0 ? 0 : (fm > 59 ? 59 : fm);
    double sec = (fraction - (double)minute / 1440.0) * 86400.0;
    second = (int32_t)lround(sec); /* Fortran nint: half away from zero */
    if (second < 0)
        second = 0;
    if (second == 60) {
        second = 0;
        minute = minute + 1;
        if (minute == 60) {
            minute = 0;
            hour = hour + 1;
            if (hour == 24) {
                hour = 0;
                ora_caldat(ora_julday(day, month, year) + 1, &day, &month, &year);
            }
        }
    }
    if (dd) *dd = day;
    if (mm) *mm = month;
    if (yy) *yy = year;
    if (hh) *hh = hour;
    if (nn) *nn = minute;
    if (ss) *ss = second;
}

/* datetimeinfo_init / datetimeinfo_increment (src/common/mo_common_datetime_type.f90:71-125)
 * plus do_time_step's dec2date(newTime - 0.5) (src/mHM/mo_mhm_interface_run.f90:360,397)
 * and FORCES datetime%doy (day of year = julday - julday(1 Jan) + 1). */
void ora_step_calendar(int32_t jul_start, int32_t timestep, int32_t nSteps, int32_t *month,
                       int32_t *hour, int32_t *doy, int32_t *day, int32_t *year)
{
    ora_step_calendar_ex(jul_start, timestep, nSteps, month, hour, doy, day, year, NULL);
}

/* ... and is_new_day / is_new_month / is_new_year as set by the increment that
 * follows step tt (bits 1, 2, 3 of new_flags[tt]) */
void ora_step_calendar_ex(int32_t jul_start, int32_t timestep, int32_t nSteps, int32_t *month,
                          int32_t *hour, int32_t *doy, int32_t *day, int32_t *year, int32_t *new_flags)
{
    double newTime = (double)jul_start;
    int32_t y, m, d, h = 0;
    ora_caldat((int32_t)newTime, &d, &m, &y);
    for (int32_t tt = 0; tt < nSteps; ++tt) {
        int32_t dd, mm, yy, hh;
        ora_dec2date(newTime - 0.5, &dd, &mm, &yy, &hh, NULL, NULL);
        if (month) month[tt] = mm;
        if (hour) hour[tt] = hh;
        if (day) day[tt] = dd;
        if (year) year[tt] = yy;
        if (doy) doy[tt] = ora_julday(dd, mm, yy) - ora_julday(1, 1, yy) + 1;
        /* increment */
        const int32_t pd = d, pm = m, py = y;
        h = h + timestep;
        newTime = (double)ora_julday(d, m, y) + (double)h / 24.0;
        h = h % 24;
        ora_caldat((int32_t)newTime, &d, &m, &y);
        if (new_flags)
            new_flags[tt] = (pd != d ? 2 : 0) | (pm != m ? 4 : 0) | (py != y ? 8 : 0);
    }
}

/* iLAI of steps 1 .. nSteps by datetimeinfo_update_LAI_timestep
 * (src/common/mo_common_datetime_type.f90:138-155) on the flags of the
 * increment: month for timeStep_LAI_input 0 / 1, else a counter raised at
 * every new day (-1), month (-2) or year (-3), all flags true at the first
 * step (datetimeinfo_init, :88-91). */
void ora_step_lai(int32_t jul_start, int32_t timestep, int32_t lai_mode, int32_t nSteps, int32_t *lai)
{
    int32_t *month = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)(nSteps > 0 ? nSteps : 1));
    if (!month)
        return;
    int32_t *flags = month + (nSteps > 0 ? nSteps : 1);
    ora_step_calendar_ex(jul_start, timestep, nSteps, month, NULL, NULL, NULL, NULL, flags);
    int32_t ilai = 0;
    for (int32_t t = 0; t < nSteps; ++t) {
        const int32_t fl = t == 0 ? 14 : flags[t - 1];
        switch (lai_mode) {
        case -1: ilai += (fl & 2) ? 1 : 0; break;
        case -2: ilai += (fl & 4) ? 1 : 0; break;
        case -3: ilai += (fl & 8) ? 1 : 0; break;
        default: ilai = month[t]; break;
        }
        lai[t] = ilai;
    }
    free(month);
}

/* ---- routing ---- */

/* src/mRM/mo_mrm_mpr.f90:61-119 */
void ora_reg_rout(const double *param, const double *length, const double *slope,
                  const double *fFPimp, int nLinks, double TS, double *C1, double *C2)
{
    double ssMax = -HUGE_VAL;
    for (int i = 0; i < nLinks; ++i)
        if (slope[i] > ssMax)
            ssMax = slope[i];
    for (int i = 0; i < nLinks; ++i) {
        double K = param[0] + param[1] * (length[i] * 0.001) + param[2] * slope[i] + param[3] * fFPimp[i];
        double xi = param[4] * (1.0 + slope[i] / ssMax);
        if (xi > 0.5)
            xi = 0.5;
        if (xi < 0.005)
            xi = 0.005;
        if (K > 0.5 * TS / xi)
            K = 0.5 * TS / xi;
        if (K < 0.5 * TS / (1.0 - xi))
            K = 0.5 * TS / (1.0 - xi);
        C1[i] = TS / (K * (1.0 - xi) + 0.5 * TS);
        C2[i] = 1.0 - C1[i] * K / TS;
    }
}

/* src/mRM/mo_mrm_pre_routing.f90:77-143 */
void ora_L11_runoff_acc(int nCells, int nNodes, const double *qAll, const double *efecArea,
                        const int32_t *L1_L11_Id, const double *L11_areaCell,
                        const int32_t *L11_L1_Id, int TS, int map_flag, double *qAcc)
{
    double TST = HOURSECS * TS;
    if (map_flag) {
        for (int i = 0; i < nNodes; ++i)
            qAcc[i] = 0.0;
        for (int k = 0; k < nCells; ++k)
            qAcc[L1_L11_Id[k] - 1] = qAcc[L1_L11_Id[k] - 1] + qAll[k] * efecArea[k];
        for (int i = 0; i < nNodes; ++i)
            qAcc[i] = qAcc[i] * 1000.0 / TST;
    } else {
        for (int i = 0; i < nNodes; ++i)
            qAcc[i] = qAll[L11_L1_Id[i] - 1];
        for (int i = 0; i < nNodes; ++i)
            qAcc[i] = qAcc[i] * L11_areaCell[i] * 1000.0 / TST;
    }
}

/* add_inflow, src/mRM/mo_mrm_pre_routing.f90:179-214: gauges in list order;
 * a headwater gauge adds its discharge to the node's runoff, any other one
 * replaces it */
void ora_add_inflow(int nInflowGauges, const int32_t *InflowHeadwater, const int32_t *InflowNodeList,
                    const double *QInflow, double *qOut)
{
    for (int ii = 0; ii < nInflowGauges; ++ii) {
        const int v = InflowNodeList[ii] - 1;
        if (InflowHeadwater[ii])
            qOut[v] = qOut[v] + QInflow[ii];
        else
            qOut[v] = QInflow[ii];
    }
}

/* src/mRM/mo_mrm_routing.f90:380-481: links in netPerm order; the routed
 * outflow of a link that drains into a non-headwater inflow gauge's node is
 * cut (:447-452) */
void ora_L11_routing_ex(int nNodes, int nLinks, const int32_t *netPerm, const int32_t *fromN, const int32_t *toN,
                        const double *C1, const double *C2, const double *qOUT, int nInflowGauges,
                        const int32_t *InflowHeadwater, const int32_t *InflowNodeList, double *qTIN, double *qTR,
                        double *Qmod)
{
    double *qTIN1 = qTIN, *qTIN2 = qTIN + nNodes; /* columns IT1 = 1, IT = 2 */
    double *qTR1 = qTR, *qTR2 = qTR + nNodes;
    for (int i = 0; i < nNodes; ++i)
        qTIN2[i] = 0.0;
    for (int k = 0; k < nLinks; ++k) {
        int i = netPerm[k] - 1;
        int iNode = fromN[i] - 1;
        int tNode = toN[i] - 1;
        qTIN2[iNode] = qTIN2[iNode] + qOUT[iNode];
        qTR2[iNode] = qTR1[iNode] + C1[i] * (qTIN1[iNode] - qTR1[iNode]) +
                      C2[i] * (qTIN2[iNode] - qTIN1[iNode]);
        for (int g = 0; g < nInflowGauges; ++g)
            if (tNode == InflowNodeList[g] - 1 && !InflowHeadwater[g])
                qTR2[iNode] = 0.0;
        qTIN2[tNode] = qTIN2[tNode] + qTR2[iNode];
    }
    if (nLinks > 0) {
        int tNode = toN[netPerm[nLinks - 1] - 1] - 1;
        qTIN2[tNode] = qTIN2[tNode] + qOUT[tNode];
    }
    for (int i = 0; i < nNodes; ++i) {
        Qmod[i] = qTIN2[i];
        qTR1[i] = qTR2[i];
        qTIN1[i] = qTIN2[i];
    }
}

/* src/mRM/mo_mrm_routing.f90:380-481 (no inflow gauges) */
void ora_L11_routing(int nNodes, int nLinks, const int32_t *netPerm, const int32_t *fromN,
                     const int32_t *toN, const double *C1, const double *C2, const double *qOUT,
                     double *qTIN, double *qTR, double *Qmod)
{
    ora_L11_routing_ex(nNodes, nLinks, netPerm, fromN, toN, C1, C2, qOUT, 0, NULL, NULL, qTIN, qTR, Qmod);
}

/* moveDownOneCell, src/mRM/mo_mrm_net_startup.f90:1768-1801 */
static void ora_move_down(int32_t fdir, int32_t *i, int32_t *j)
{
    switch (fdir) {
    case 1: *j += 1; break;
    case 2: *i += 1; *j += 1; break;
    case 4: *i += 1; break;
    case 8: *i += 1; *j -= 1; break;
    case 16: *j -= 1; break;
    case 32: *i -= 1; *j -= 1; break;
    case 64: *i -= 1; break;
    case 128: *i -= 1; *j += 1; break;
    default: break;
    }
}

/* src/mRM/mo_mrm_net_startup.f90:630-727 */
int ora_L11_set_network_topology(int nrows, int ncols, const int32_t *id2d, int nCells,
                                 const int32_t *cellRow, const int32_t *cellCol,
                                 const int32_t *fDir11, int32_t *fromN, int32_t *toN)
{
    int jj = 0;
    for (int k = 0; k < nCells; ++k) {
        fromN[k] = -9999;
        toN[k] = -9999;
    }
    for (int kk = 0; kk < nCells; ++kk) {
        int32_t ic = cellRow[kk], jc = cellCol[kk];
        int32_t fn = kk + 1;
        ora_move_down(fDir11[kk], &ic, &jc);
        int32_t tn = id2d[(size_t)(jc - 1) * nrows + (ic - 1)];
        if (fn == tn)
            continue;
        fromN[jj] = fn;
        toN[jj] = tn;
        ++jj;
    }
    (void)ncols;
    return jj;
}

/* src/mRM/mo_mrm_net_startup.f90:728-886, literally (O(nLinks^2) per sweep) */
void ora_L11_routing_order(int nNodes, int nOutlets, const int32_t *fromN, const int32_t *toN,
                           int32_t *netPerm, int32_t *rOrder)
{
    int nLinks = nNodes - nOutlets;
    for (int i = 0; i < nNodes; ++i) {
        netPerm[i] = -9999;
        rOrder[i] = -9999;
    }
    if (nNodes <= 1)
        return;
    for (int i = 0; i < nLinks; ++i)
        rOrder[i] = 1;
    for (int ii = 0; ii < nLinks; ++ii) {
        for (int jj = 0; jj < nLinks; ++jj) {
            if (jj == ii)
                continue;
            if (fromN[ii] == toN[jj])
                rOrder[ii] = -9;
            if (rOrder[ii] == -9)
                break;
        }
    }
    int kk = 0;
    for (int ii = 0; ii < nLinks; ++ii)
        if (rOrder[ii] == 1)
            rOrder[ii] = ++kk;
    for (;;) {
        int minv = 1 << 30;
        for (int ii = 0; ii < nLinks; ++ii)
            if (rOrder[ii] < minv)
                minv = rOrder[ii];
        if (!(minv < 0))
            break;
        for (int ii = 0; ii < nLinks; ++ii) {
            if (rOrder[ii] != -9)
                continue;
            int flag = 1;
            for (int jj = 0; jj < nLinks; ++jj) {
                if (jj == ii || fromN[ii] != toN[jj])
                    continue;
                if (!(fromN[ii] == toN[jj] && rOrder[jj] > 0)) {
                    flag = 0;
                    break;
                }
            }
            if (flag)
                rOrder[ii] = ++kk;
        }
    }
    for (int ii = 0; ii < nLinks; ++ii)
        netPerm[rOrder[ii] - 1] = ii + 1;
}

/* The same ranks as ora_L11_routing_order (the same sweeps over the links in
 * index order, a link ranked once every link draining into its from-node is
 * ranked, including links ranked earlier in the same sweep), with each link's
 * upstream links listed once up front instead of found by a scan of all
 * links: O(sweeps * links) instead of O(sweeps * links^2), usable at 62,500
 * nodes.  Returns 0, or -1 if a sweep ranks nothing (a cycle). */
int ora_L11_routing_order_listed(int nNodes, int nOutlets, const int32_t *fromN, const int32_t *toN,
                                 int32_t *netPerm, int32_t *rOrder)
{
    int nLinks = nNodes - nOutlets;
    for (int i = 0; i < nNodes; ++i) {
        netPerm[i] = -9999;
        rOrder[i] = -9999;
    }
    if (nNodes <= 1 || nLinks <= 0)
        return 0;
    /* links by the node they drain into (1-based node ids) */
    int32_t *cnt = (int32_t *)calloc((size_t)nNodes + 2, sizeof(int32_t));
    int32_t *lst = (int32_t *)malloc((size_t)nLinks * sizeof(int32_t));
    if (!cnt || !lst) {
        free(cnt);
        free(lst);
        return -1;
    }
    for (int jj = 0; jj < nLinks; ++jj)
        if (toN[jj] >= 1 && toN[jj] <= nNodes)
            cnt[toN[jj] + 1]++;
    for (int v = 1; v <= nNodes + 1; ++v)
        cnt[v] += cnt[v - 1];
    {
        int32_t *fill = (int32_t *)malloc(((size_t)nNodes + 1) * sizeof(int32_t));
        if (!fill) {
            free(cnt);
            free(lst);
            return -1;
        }
        memcpy(fill, cnt, ((size_t)nNodes + 1) * sizeof(int32_t));
        for (int jj = 0; jj < nLinks; ++jj)
            if (toN[jj] >= 1 && toN[jj] <= nNodes)
                lst[fill[toN[jj]]++] = jj;
        free(fill);
    }
    int kk = 0;
    for (int ii = 0; ii < nLinks; ++ii) {
        int up = 0;
        int v = fromN[ii];
        for (int q = cnt[v]; q < cnt[v + 1]; ++q)
            if (lst[q] != ii)
                up = 1;
        rOrder[ii] = up ? -9 : 1;
    }
    for (int ii = 0; ii < nLinks; ++ii)
        if (rOrder[ii] == 1)
            rOrder[ii] = ++kk;
    int rc = 0;
    while (kk < nLinks) {
        int before = kk;
        for (int ii = 0; ii < nLinks; ++ii) {
            if (rOrder[ii] != -9)
                continue;
            int flag = 1, v = fromN[ii];
            for (int q = cnt[v]; q < cnt[v + 1]; ++q) {
                int jj = lst[q];
                if (jj != ii && !(rOrder[jj] > 0)) {
                    flag = 0;
                    break;
                }
            }
            if (flag)
                rOrder[ii] = ++kk;
        }
        if (kk == before) {
            rc = -1;
            break;
        }
    }
    if (rc == 0)
        for (int ii = 0; ii < nLinks; ++ii)
            netPerm[rOrder[ii] - 1] = ii + 1;
    free(cnt);
    free(lst);
    return rc;
}

/* ---- whole-domain run ---- */

/* fluxes_states_default_init (src/mHM/mo_init_states.f90:258-345) and
 * fluxes_states_default_init_routing (src/mRM/mo_mrm_init.f90:453-499) */
void ora_default_states(const ora_domain *d, const double *horizon_depth, ora_state *s)
{
    int N = d->nCells, H = d->nH;
    for (int k = 0; k < N; ++k) {
        s->interc[k] = P1_INIT;
        s->snowpack[k] = P2_INIT;
        s->sealSTW[k] = P1_INIT;
        s->unsat[k] = P3_INIT;
        s->sat[k] = P4_INIT;
    }
    for (int h = 0; h < H - 1; ++h) {
        double v = (h == 0) ? horizon_depth[0] * C1_INITSM
                            : (horizon_depth[h] - horizon_depth[h - 1]) * C1_INITSM;
        for (int k = 0; k < N; ++k)
            s->SM[(size_t)h * N + k] = v;
    }
    {
        double v = (P5_INIT - (H >= 2 ? horizon_depth[H - 2] : 0.0)) * C1_INITSM;
        for (int k = 0; k < N; ++k)
            s->SM[(size_t)(H - 1) * N + k] = v;
    }
    for (int i = 0; i < d->nNodes; ++i) {
        s->qTIN[i] = s->qTIN[d->nNodes + i] = P1_INIT;
        s->qTR[i] = s->qTR[d->nNodes + i] = P1_INIT;
        s->qOUT[i] = P1_INIT;
        s->Qmod[i] = P1_INIT;
        s->C1[i] = P1_INIT;
        s->C2[i] = P1_INIT;
    }
}

/* The mhm_eval time loop (src/mHM/mo_mhm_eval.f90:136-150) for one domain:
 * do_time_step (src/mHM/mo_mhm_interface_run.f90:341-638) = meteo getters
 * (src/meteo/mo_meteo_handler.f90:915-1285) + mHM() (src/mHM/mo_mhm.f90:229-521)
 * + mRM_routing (src/mRM/mo_mrm_routing.f90:104-303, processCase 1). */
/* src/mRM/mo_mrm_constants.F90:42-46 */
static const double GIVEN_TS[19] = {60.0,   120.0,  180.0,   240.0,   300.0,   360.0,   600.0,
                                    720.0,  900.0,  1200.0,  1800.0,  3600.0,  7200.0,  10800.0,
                                    14400.0, 21600.0, 28800.0, 43200.0, 86400.0};

/* FORCES locate (in-tree copy pre-proc/mtCLIM/mo_utils.f90:1329-1346): the
 * index (1-based) of the nearest table value, minus one when that value is
 * above y (LE with the relative-epsilon equality) */
static int ora_locate(const double *x, int n, double y)
{
    int c = 0;
    double best = fabs(x[0] - y);
    for (int i = 1; i < n; ++i)
        if (fabs(x[i] - y) < best) {
            best = fabs(x[i] - y);
            c = i;
        }
    return ora_le(x[c], y) ? c + 1 : c;
}

/* mrm_update_param, src/mRM/mo_mrm_mpr.f90:241-329: K = L11_length / celerity
 * (case 2: one celerity; case 3: L11_celerity of each link) */
double ora_update_param_links(const double *link_celerity, double celerity, const double *length, int nLinks,
                              double *C1, double *C2)
{
    const double xi = fabs(0.0); /* rout_space_weight */
    double kmin = HUGE_VAL;
    for (int i = 0; i < nLinks; ++i) {
        double K = length[i] / (link_celerity ? link_celerity[i] : celerity);
        if (K < kmin)
            kmin = K;
    }
    int ind = ora_locate(GIVEN_TS, 19, kmin);
    if (ind < 1)
        ind = 1;
    const double ts = GIVEN_TS[ind - 1];
    for (int i = 0; i < nLinks; ++i) {
        double K = length[i] / (link_celerity ? link_celerity[i] : celerity);
        C1[i] = ts / (K * (1.0 - xi) + 0.5 * ts);
        C2[i] = 1.0 - C1[i] * K / ts;
    }
    return ts;
}

double ora_update_param_case2(double celerity, const double *length, int nLinks, double *C1, double *C2)
{
    return ora_update_param_links(NULL, celerity, length, nLinks, C1, C2);
}

/* L11_calc_celerity, src/mRM/mo_mrm_net_startup.f90:2212-2423, for one link:
 * the harmonic mean of slope_factor * sqrt(slope / 100) over the L0 cells of
 * the link's river path, from its source cell to its outlet cell inclusive
 * (slopes in percent, after the reference's lower bound of 0.1 and its
 * outlier filter) */
double ora_link_celerity(double slope_factor, const double *path_slope, int n)
{
    double s = 0.0;
    for (int j = 0; j < n; ++j)
        s = s + 1.0 / (slope_factor * sqrt(path_slope[j] / 100.0));
    return (double)n / s;
}

/* ---- aggregated outputs ---- */

/* variables in the order mHM_OutputDataset creates them
 * (src/mHM/mo_write_fluxes_states.f90:82-262) */
static const int ORA_OUT_ORDER[21] = {1, 2, 3, 4, 5, 6, 7, 8, 18, 9, 10, 11, 12, 13, 14, 15, 16, 17, 19, 20, 21};

int ora_output_planes(ora_output *o, int nH)
{
    int n = 0;
    for (int f = 0; f < 22; ++f)
        o->plane[f] = -1;
    for (int i = 0; i < 21; ++i) {
        const int f = ORA_OUT_ORDER[i];
        if (!o->flags[f - 1])
            continue;
        if (f == 18)
            return -1; /* neutrons: process 10 */
        o->plane[f] = n;
        n += (f == 3 || f == 4 || f == 17 || f == 19) ? nH : 1;
    }
    o->n_planes = n;
    return n;
}

/* datetimeinfo_writeout, src/common/mo_common_datetime_type.f90:157-185 */
static int ora_writeout(int interval, int32_t tindex, int32_t tt, int32_t n_tt, int32_t new_flags)
{
    if (interval > 0)
        return (tindex % interval == 0) || tt == n_tt;
    switch (interval) {
    case 0: return tt == n_tt;
    case -1: return (new_flags & 2) || tt == n_tt;
    case -2: return (new_flags & 4) || tt == n_tt;
    case -3: return (new_flags & 8) || tt == n_tt;
    default: return 0; /* no output at all */
    }
}

int ora_run(const ora_domain *d, const ora_params *p, ora_state *s, const ora_forcing *f,
            int32_t tt0, int32_t nT, double *q_gauge, double *total_runoff_out, double *qmod_out,
            int nthreads)
{
    return ora_run_ex(d, p, s, f, tt0, nT, q_gauge, total_runoff_out, qmod_out, nthreads, NULL);
}

int ora_run_ex(const ora_domain *d, const ora_params *p, ora_state *s, const ora_forcing *f,
               int32_t tt0, int32_t nT, double *q_gauge, double *total_runoff_out, double *qmod_out,
               int nthreads, ora_output *out)
{
    const int N = d->nCells, H = d->nH, L = d->nNodes;
    const int nLinks = L - d->nOutlets;
    const double c2TSTu = (double)d->timestep / 24.0;          /* mo_startup.f90:168 */
    const double nTstepDay_dp = 24.0 / (double)d->timestep;   /* nTstepDay = 24/timestep */
    if (tt0 < 1 || nT < 0 || H < 1 || H > 16)
        return -1;
    int32_t *cal = (int32_t *)malloc(sizeof(int32_t) * 5 * (size_t)(tt0 + nT));
    if (!cal)
        return -2;
    int32_t *cal_month = cal, *cal_hour = cal + (tt0 + nT), *cal_doy = cal + 2 * (tt0 + nT);
    int32_t *cal_new = cal + 3 * (tt0 + nT), *cal_lai = cal + 4 * (tt0 + nT);
    ora_step_calendar_ex(d->jul_start, d->timestep, tt0 - 1 + nT, cal_month, cal_hour, cal_doy, NULL, NULL,
                         cal_new);
    /* iLAI of every step from the run's first (datetimeinfo_update_LAI_timestep,
     * src/common/mo_common_datetime_type.f90:138-155): the month for LAI slots;
     * for a series a counter raised when the step starts a new day / month /
     * year, is_new_* being true at the first step (:88-91) */
    {
        int32_t ilai = 0;
        for (int32_t t = 0; t < tt0 - 1 + nT; ++t) {
            const int32_t fl = t == 0 ? 14 : cal_new[t - 1];
            switch (d->lai_mode) {
            case -1: ilai += (fl & 2) ? 1 : 0; break;
            case -2: ilai += (fl & 4) ? 1 : 0; break;
            case -3: ilai += (fl & 8) ? 1 : 0; break;
            default: ilai = cal_month[t]; break;
            }
            cal_lai[t] = ilai;
        }
        if (d->lai_mode < 0 && (tt0 - 1 + nT) > 0 && cal_lai[tt0 - 2 + nT] > d->n_lai) {
            free(cal);
            return -6; /* the LAI series does not cover the run */
        }
    }
    double *pet_calc = (double *)malloc(sizeof(double) * (size_t)N);
    double *temp_calc = (double *)malloc(sizeof(double) * (size_t)N);
    double *prec_calc = (double *)malloc(sizeof(double) * (size_t)N);
    double *tro = (double *)malloc(sizeof(double) * (size_t)N);
    if (!pet_calc || !temp_calc || !prec_calc || !tro) {
        free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
        return -2;
    }
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    /* reg_rout is step-invariant (called every step for processCase 1, not after a restart) */
    if (d->proc_rout == 1 && !d->read_states && L > 1)
        ora_reg_rout(d->rout_param, d->length, d->slope, d->ffp_imp, nLinks, (double)d->timestep,
                     s->C1, s->C2);
    /* routing case 2: one routing time step for the run (mrm_init_param / mrm_update_param) and
     * tsRoutFactor = TSrout / (timestep * HourSecs) (src/mHM/mo_mhm_interface_run.f90:480-511) */
    double ts_factor = 1.0;
    int rout_loop = 1, win = 1;
    if (d->proc_rout >= 2 && L > 1) {
        const double tsrout = ora_update_param_links(d->proc_rout == 3 ? d->link_celerity : NULL, d->rout_param[0],
                                                     d->length, nLinks, s->C1, s->C2);
        ts_factor = tsrout / ((double)d->timestep * 3600.0);
        if (ts_factor < 1.0) {
            rout_loop = (int)lround(1.0 / ts_factor);
            if (rout_loop < 1)
                rout_loop = 1;
        } else {
            win = (int)lround(ts_factor);
            if (!s->run_to_rout || (tt0 - 1) % win != 0 || nT % win != 0) {
                free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
                return -4; /* runs must cover whole routing steps */
            }
        }
    }
    double *qacc = (double *)malloc(sizeof(double) * (size_t)L);
    if (!qacc) {
        free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
        return -2;
    }
    /* inflow gauges: the step's InflowDischarge = InflowGauge%Q(iDischargeTS, :),
     * iDischargeTS = ceiling(tt / nTstepDay) (src/mHM/mo_mhm_interface_run.f90:463-511);
     * with a routing step of several model steps summed from 0 and divided by
     * tsRoutFactorIn, then reset after routing (:602-611) */
    const int nIn = (d->proc_rout >= 1) ? d->nInflow : 0;
    const int32_t steps_day = 24 / d->timestep;
    double qin[64], qin_acc[64];
    if (nIn > 64) {
        free(qacc); free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
        return -5;
    }
    for (int g = 0; g < nIn; ++g) {
        qin[g] = 0.0;
        qin_acc[g] = 0.0;
    }
    if (nIn > 0) {
        const int32_t day_a = (tt0 + steps_day - 1) / steps_day, day_b = (tt0 + nT - 1 + steps_day - 1) / steps_day;
        if (day_a < d->inflow_day0 || day_b > d->inflow_day0 + d->inflow_ndays - 1) {
            free(qacc); free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
            return -5; /* inflow discharge does not cover the run */
        }
    }

    for (int32_t it = 0; it < nT; ++it) {
        const int32_t tt = tt0 + it;
        const int month = cal_month[tt - 1];
        const int hour = cal_hour[tt - 1];
        const int doy = cal_doy[tt - 1];
        const int isday = (hour > 6) && (hour <= 18);              /* mo_meteo_handler.f90:1048 */
        const int is_hourly = (d->nTstepForcingDay == 24);
        /* update_timestep, mo_meteo_handler.f90:575-620 */
        const int32_t stride = (int32_t)lround(24.0 / (double)d->nTstepForcingDay);
        const int32_t iMeteoTS = (int32_t)ceil((double)tt / (double)stride);
        const int32_t row = iMeteoTS - f->forc_row0;
        if (row < 0 || row >= f->n_rows) {
            free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
            return -3;
        }
        const double *pre = f->pre + (size_t)row * N;
        const double *tmp = f->temp + (size_t)row * N;
        const double *pet = f->pet ? f->pet + (size_t)row * N : NULL;
        const double *tmin = f->tmin ? f->tmin + (size_t)row * N : NULL;
        const double *tmax = f->tmax ? f->tmax + (size_t)row * N : NULL;
        const double *netrad = f->netrad ? f->netrad + (size_t)row * N : NULL;
        const double *eabs = f->eabs ? f->eabs + (size_t)row * N : NULL;
        const double *wind = f->windspeed ? f->windspeed + (size_t)row * N : NULL;
        const double evap_coeff = d->evap_coeff[month - 1];
        const int iLAI = cal_lai[tt - 1];
        /* this step's outputs (write_output after do_time_step) */
        const int out_on = out && out->n_planes > 0 && tt > out->warm_steps;
        int out_write = 0, out_slot = 0;
        double out_cnt = 0.0;
        if (out_on) {
            out_write = ora_writeout(out->interval, tt - out->warm_steps, tt, out->n_time_steps, cal_new[tt - 1]);
            out_slot = out->n_slots;
            out_cnt = (double)(out->counter + 1);
            if (out_write && out_slot >= out->max_slots) {
                free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro); free(qacc);
                return -5;
            }
        }
        if (tt == 1 && !d->read_states) /* mo_mhm.f90:448-450 */
            for (int h = 0; h < H; ++h)
                for (int k = 0; k < N; ++k)
                    s->SM[(size_t)h * N + k] = 0.5 * p->FC[(size_t)h * N + k];

#pragma omp parallel for schedule(static)
        for (int k = 0; k < N; ++k) {
            /* get_corrected_pet (:915-1123), get_temp (:1126-1205), get_prec (:1208-1285) */
            double pv;
            switch (d->proc_pet) {
            case -1: pv = p->petLAIcorFactor[(size_t)(iLAI - 1) * N + k] * pet[k]; break;
            case 0: pv = p->fAsp[k] * pet[k]; break;
            case 2: /* Priestley-Taylor, not defined for netrad < 0 (mo_meteo_handler.f90:1079-1084) */
                pv = ora_pet_priestly(p->PrieTayAlpha[(size_t)(iLAI - 1) * N + k],
                                      netrad[k] > 0.0 ? netrad[k] : 0.0, tmp[k]);
                break;
            case 3: /* Penman-Monteith, mo_meteo_handler.f90:1087-1095 */
                pv = ora_pet_penman(netrad[k] > 0.0 ? netrad[k] : 0.0, tmp[k], eabs[k] / 1000.0,
                                    p->aeroResist[(size_t)(iLAI - 1) * N + k] / wind[k],
                                    p->surfResist[(size_t)(iLAI - 1) * N + k], 1.0, 1.0);
                break;
            default:
                pv = p->fAsp[k] * ora_pet_hargreaves(p->HarSamCoeff[k], HARSAMCONST, tmp[k], tmax[k],
                                                     tmin[k], d->latitude[k], doy);
                break;
            }
            double pet_k, temp_k, prec_k;
            if (is_hourly) {
                pet_k = pv;
                temp_k = tmp[k];
                prec_k = pre[k];
            } else if (d->pet_w) {
                /* temporal_disagg_meteo_weights with L1_*_weights(k, month, hour + 1),
                 * src/meteo/mo_meteo_handler.f90:1102-1107, 1183-1189, 1265-1270;
                 * temperature corrected by T0 = 273.15 K */
                const size_t wi = ((size_t)hour * 12 + (size_t)(month - 1)) * N + k;
                pet_k = ora_disagg_meteo_weights(pv, d->pet_w[wi], 0.0);
                temp_k = ora_disagg_meteo_weights(tmp[k], d->temp_w[wi], T0_DP);
                prec_k = ora_disagg_meteo_weights(pre[k], d->pre_w[wi], 0.0);
            } else {
                pet_k = ora_disagg_flux_daynight(isday, nTstepDay_dp, pv, d->fday_pet[month - 1],
                                                 d->fnight_pet[month - 1]);
                temp_k = ora_disagg_state_daynight(isday, nTstepDay_dp, tmp[k], d->fday_temp[month - 1],
                                                   d->fnight_temp[month - 1], 1);
                prec_k = ora_disagg_flux_daynight(isday, nTstepDay_dp, pre[k], d->fday_prec[month - 1],
                                                  d->fnight_prec[month - 1]);
            }
            pet_calc[k] = pet_k;
            temp_calc[k] = temp_k;
            prec_calc[k] = prec_k;

            /* mHM() cell body, mo_mhm.f90:460-493 */
            double throughfall, aet_canopy;
            double interc_max = p->maxInter[(size_t)(iLAI - 1) * N + k];
            ora_canopy_interc(pet_k, interc_max, prec_k, &s->interc[k], &throughfall, &aet_canopy);
            double deg_day, melt, prec_effect, rain, snow;
            ora_snow_accum_melt(p->degDayInc[k], p->degDayMax[k] * c2TSTu, p->degDayNoPre[k] * c2TSTu,
                                prec_k, temp_k, p->tempThresh[k], throughfall, &s->snowpack[k], &deg_day,
                                &melt, &prec_effect, &rain, &snow);
            double sm_sat[16], froots[16], fc[16], pw[16], beta[16], sm[16], infil[16], aet[16];
            for (int h = 0; h < H; ++h) {
                size_t o = (size_t)h * N + k;
                sm_sat[h] = p->SMs[o];
                froots[h] = p->fRoots[o];
                fc[h] = p->FC[o];
                pw[h] = p->PW[o];
                beta[h] = p->beta[o];
                sm[h] = s->SM[o];
            }
            double runoff_sealed, aet_sealed;
            ora_soil_moisture(d->proc_sm, H, p->fSealed[k], p->sealedThresh[k], pet_k, evap_coeff, sm_sat,
                              froots, fc, pw, beta, p->jarvis_c1 ? p->jarvis_c1[k] : 0.0, aet_canopy, prec_effect,
                              &runoff_sealed, &s->sealSTW[k], infil, sm, aet, &aet_sealed);
            for (int h = 0; h < H; ++h)
                s->SM[(size_t)h * N + k] = sm[h];
            double slow, fast, perc, base;
            ora_runoff_unsat_zone(c2TSTu / p->kSlowFlow[k], c2TSTu / p->kPerco[k], c2TSTu / p->kFastFlow[k],
                                  p->alpha[k], p->karstLoss[k], infil[H - 1], p->unsatThresh[k], &s->sat[k],
                                  &s->unsat[k], &slow, &fast, &perc);
            ora_runoff_sat_zone(c2TSTu / p->kBaseFlow[k], &s->sat[k], &base);
            tro[k] = ora_L1_total_runoff(p->fSealed[k], fast, slow, base, runoff_sealed);

            if (out_on) { /* mHM_updateDataset, src/mHM/mo_write_fluxes_states.f90:283-438 */
                const int w = out->tt_w == tt;
                const double fS = w ? out->w_fsealed[k] : p->fSealed[k];
                const double fNS = 1.0 - fS; /* run_cfg%L1_fNotSealed */
                const int *pl = out->plane;
                double *A = out->acc;
#define ORA_ADD(PLANE, X) (A[(size_t)(PLANE) * N + k] = A[(size_t)(PLANE) * N + k] + (X))
                if (pl[1] >= 0) ORA_ADD(pl[1], s->interc[k]);
                if (pl[2] >= 0) ORA_ADD(pl[2], s->snowpack[k]);
                for (int h = 0; h < H; ++h) {
                    const double sat_h = w ? out->w_sms[(size_t)h * N + k] : sm_sat[h];
                    if (pl[3] >= 0) ORA_ADD(pl[3] + h, sm[h]);
                    if (pl[4] >= 0) ORA_ADD(pl[4] + h, sm[h] / sat_h);
                }
                if (pl[5] >= 0) {
                    double ssm = 0.0, ssat = 0.0;
                    for (int h = 0; h < H; ++h) {
                        ssm = ssm + sm[h];
                        ssat = ssat + (w ? out->w_sms[(size_t)h * N + k] : sm_sat[h]);
                    }
                    ORA_ADD(pl[5], ssm / ssat);
                }
                if (pl[6] >= 0) ORA_ADD(pl[6], s->sealSTW[k]);
                if (pl[7] >= 0) ORA_ADD(pl[7], s->unsat[k]);
                if (pl[8] >= 0) ORA_ADD(pl[8], s->sat[k]);
                if (pl[9] >= 0) ORA_ADD(pl[9], pet_k);
                if (pl[10] >= 0) {
                    double aet_soil = 0.0;
                    for (int h = 0; h < H; ++h)
                        aet_soil = aet_soil + aet[h];
                    ORA_ADD(pl[10], aet_soil * fNS + aet_canopy + aet_sealed * fS);
                }
                if (pl[11] >= 0) ORA_ADD(pl[11], tro[k]);
                if (pl[12] >= 0) ORA_ADD(pl[12], runoff_sealed * fS);
                if (pl[13] >= 0) ORA_ADD(pl[13], fast * fNS);
                if (pl[14] >= 0) ORA_ADD(pl[14], slow * fNS);
                if (pl[15] >= 0) ORA_ADD(pl[15], base * fNS);
                if (pl[16] >= 0) ORA_ADD(pl[16], perc * fNS);
                for (int h = 0; h < H; ++h) {
                    if (pl[17] >= 0) ORA_ADD(pl[17] + h, infil[h] * fNS);
                    if (pl[19] >= 0) ORA_ADD(pl[19] + h, aet[h] * fNS);
                }
                if (pl[20] >= 0) ORA_ADD(pl[20], prec_effect);
                if (pl[21] >= 0) ORA_ADD(pl[21], melt);
#undef ORA_ADD
                if (out_write) { /* writeVariableTimestep, src/common/mo_nc_output.f90:158-175 */
                    for (int i = 0; i < 21; ++i) {
                        const int fl = ORA_OUT_ORDER[i];
                        if (pl[fl] < 0)
                            continue;
                        const int np = (fl == 3 || fl == 4 || fl == 17 || fl == 19) ? H : 1;
                        for (int j = 0; j < np; ++j) {
                            const size_t a = (size_t)(pl[fl] + j) * N + k;
                            const double v = (fl <= 8) ? A[a] / out_cnt : A[a]; /* avg for the states */
                            out->out[((size_t)out_slot * out->n_planes + pl[fl] + j) * N + k] = v;
                            A[a] = 0.0;
                        }
                    }
                }
            }
        }
        if (out_on) {
            out->counter = out_write ? 0 : out->counter + 1;
            if (out_write) {
                out->slot_tt[out->n_slots] = tt;
                out->n_slots = out->n_slots + 1;
            }
        }
        if (total_runoff_out)
            memcpy(total_runoff_out + (size_t)it * N, tro, sizeof(double) * (size_t)N);

        /* mRM_routing, processCase 1 (mo_mrm_routing.f90:104-303): rout_loop = 1; case 2 below */
        const double *qday = nIn > 0 ? d->inflow_q + (size_t)((tt + steps_day - 1) / steps_day - d->inflow_day0) * nIn
                                     : NULL;
        if (d->proc_rout == 1) {
            ora_L11_runoff_acc(N, L, tro, d->l1_area_km2, d->l1_l11_id, d->l11_area_km2, d->l11_l1_id,
                               d->timestep, d->map_flag, s->qOUT);
            ora_add_inflow(nIn, d->inflow_headwater, d->inflow_node, qday, s->qOUT);
            if (L > 1) {
                ora_L11_routing_ex(L, nLinks, d->net_perm, d->from_n, d->to_n, s->C1, s->C2, s->qOUT, nIn,
                                   d->inflow_headwater, d->inflow_node, s->qTIN, s->qTR, s->Qmod);
                /* L11_qMod = L11_qAcc / real(rout_loop): (0 + Qmod) / 1 */
                for (int i = 0; i < L; ++i)
                    s->Qmod[i] = (0.0 + s->Qmod[i]) / 1.0;
            } else {
                s->Qmod[0] = s->qOUT[0];
            }
            if (q_gauge)
                for (int g = 0; g < d->nGauges; ++g)
                    q_gauge[(size_t)it * d->nGauges + g] = s->Qmod[d->gauge_node[g] - 1];
            if (qmod_out)
                memcpy(qmod_out + (size_t)it * L, s->Qmod, sizeof(double) * (size_t)L);
        } else if (d->proc_rout >= 2) {
            int route_now = 1, ts_rout = d->timestep;
            const double *run = tro;
            if (win > 1) { /* accumulate until the routing step is complete (:489-511) */
                for (int k = 0; k < N; ++k)
                    s->run_to_rout[k] = s->run_to_rout[k] + tro[k];
                route_now = (tt % win) == 0;
                ts_rout = d->timestep * win;
                run = s->run_to_rout;
            }
            if (ts_factor < 1.0) {
                for (int g = 0; g < nIn; ++g)
                    qin[g] = qday[g];
            } else { /* summed over the routing step, then a mean (:503-510) */
                for (int g = 0; g < nIn; ++g)
                    qin_acc[g] = qin_acc[g] + qday[g];
                if (route_now)
                    for (int g = 0; g < nIn; ++g)
                        qin[g] = qin_acc[g] / ts_factor;
            }
            if (route_now) {
                ora_L11_runoff_acc(N, L, run, d->l1_area_km2, d->l1_l11_id, d->l11_area_km2, d->l11_l1_id,
                                   ts_rout, d->map_flag, s->qOUT);
                ora_add_inflow(nIn, d->inflow_headwater, d->inflow_node, qin, s->qOUT);
                for (int g = 0; g < nIn; ++g)
                    qin_acc[g] = 0.0;
                if (L > 1) {
                    for (int i = 0; i < L; ++i)
                        qacc[i] = 0.0;
                    for (int r = 0; r < rout_loop; ++r) { /* mo_mrm_routing.f90:238-277 */
                        ora_L11_routing_ex(L, nLinks, d->net_perm, d->from_n, d->to_n, s->C1, s->C2, s->qOUT,
                                           nIn, d->inflow_headwater, d->inflow_node, s->qTIN, s->qTR, s->Qmod);
                        for (int i = 0; i < L; ++i)
                            qacc[i] = qacc[i] + s->Qmod[i];
                    }
                    for (int i = 0; i < L; ++i)
                        s->Qmod[i] = qacc[i] / (double)rout_loop;
                } else {
                    s->Qmod[0] = s->qOUT[0];
                }
                if (win > 1)
                    for (int k = 0; k < N; ++k)
                        s->run_to_rout[k] = 0.0;
                /* the routed value stands for every model step of the routing step
                 * (mRM_runoff copy-back, src/mHM/mo_mhm_interface_run.f90:603-608) */
                for (int j = 0; j < win; ++j) {
                    const int32_t jt = it - j;
                    if (q_gauge)
                        for (int g = 0; g < d->nGauges; ++g)
                            q_gauge[(size_t)jt * d->nGauges + g] = s->Qmod[d->gauge_node[g] - 1];
                    if (qmod_out)
                        memcpy(qmod_out + (size_t)jt * L, s->Qmod, sizeof(double) * (size_t)L);
                }
            }
        }
        /* mRM_updateDataset with the discharge state after this step
         * (src/mRM/mo_mrm_write_fluxes_states.f90:130-133; Qrouted is a mean) */
        if (out && out->qrouted && d->proc_rout >= 1 && tt > out->warm_steps) {
            for (int i = 0; i < L; ++i)
                out->acc_mrm[i] = out->acc_mrm[i] + s->Qmod[i];
            out->counter_mrm = out->counter_mrm + 1;
            if (ora_writeout(out->interval_mrm, tt - out->warm_steps, tt, out->n_time_steps, cal_new[tt - 1])) {
                if (out->n_slots_mrm >= out->max_slots) {
                    free(qacc); free(cal); free(pet_calc); free(temp_calc); free(prec_calc); free(tro);
                    return -5;
                }
                for (int i = 0; i < L; ++i) {
                    out->out_mrm[(size_t)out->n_slots_mrm * L + i] = out->acc_mrm[i] / (double)out->counter_mrm;
                    out->acc_mrm[i] = 0.0;
                }
                out->slot_tt_mrm[out->n_slots_mrm] = tt;
                out->n_slots_mrm = out->n_slots_mrm + 1;
                out->counter_mrm = 0;
            }
        }
    }
    free(qacc);
    free(cal);
    free(pet_calc);
    free(temp_calc);
    free(prec_calc);
    free(tro);
    return 0;
}
