from .Angles2Backbone import Angles2Backbone
