"""Every benchmark configuration, at reduced size, within the reference's
a-priori error bound of the exact result (tests/accuracy_report.py runs the
same at full size)."""
import accuracy_report


def test_errors_within_gamma_bound(oracle):
    for row in accuracy_report.report(quick=True):
        assert row["max_err_over_sum_abs"] <= row["gamma_n"], row
