"""GB300-native superparameterized CRM step (the reference's crm()).

Public API:
  crm(...)                the drop-in call (crm_gb300.crm)
  CrmContext              a configured handle over the C ABI
  CrmConfig, CrmInput, CrmState, CrmRad, CrmOutput   the derived types
  synthetic               seeded idealised GCM columns
"""
from .crm_types import (CrmConfig, CrmInput, CrmOutput, CrmRad, CrmState,  # noqa: F401
                    CRM_OK, CRM_FP64, CRM_FP32_MIXED, CRM_PER_COLUMN,
                    CRM_REFERENCE_BATCH, OUTPUT_FIELDS, call_desc)
from .lib import CrmContext, CrmError, load  # noqa: F401
from .crm import crm, get_context  # noqa: F401
from . import synthetic  # noqa: F401
